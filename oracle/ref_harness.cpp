// Harness that exposes the reference's own header-only hot-path math through a C ABI so that the
// FP64 restatement in vbd_oracle.cpp can be checked against it.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile from the reference sources where they lie
// (the reference's `source/` directory on the include path, never copied), with the stand-in
// headers of oracle/ref_stubs/.  Output goes to oracle/_ref/ only.
//
// Reference code called verbatim:
//   physics/StableNeoHookeanEnergy.h  (eval, grad, gradAndHessian)
//   sim/vbd/Kernels.h                 (InitialPositionsForSolve, ChebyshevOmega,
//                                      AccumulateElasticHessian/Gradient, AddDamping,
//                                      AddInertiaDerivatives, IntegratePositions,
//                                      AccumulateVertexTriangleContact)
//   graph/Color.h                     (GreedyColor)
//   geometry/Morton.h                 (Morton3D)

#include <algorithm>
#include <cmath>
// sim/vbd/Kernels.h calls unqualified min/max on host scalars; the reference build gets them from
// its Eigen headers, this harness brings the std overloads into the global namespace instead.
using std::max;
using std::min;

#include "pbat/geometry/EdgeEdgeCcd.h"
#include "pbat/geometry/Morton.h"
#include "pbat/geometry/PointTriangleCcd.h"
#include "pbat/graph/Color.h"
#include "pbat/physics/StableNeoHookeanEnergy.h"
#include "pbat/sim/vbd/Kernels.h"

#include <array>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "orc_problem.h"

namespace {
namespace mini = pbat::math::linalg::mini;
using pbat::sim::vbd::EInitializationStrategy;

template <int M, int N>
mini::SMatrix<double, M, N> load(double const* a)
{
    mini::SMatrix<double, M, N> A;
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < M; ++i)
            A(i, j) = a[j * M + i];
    return A;
}

// Reference per-vertex solve: the body of sim/vbd/Integrator.cpp:98-136 with its kernels.
void ref_vertex_solve_impl(
    int32_t n,
    double const* xe,  // n x (3x4 column-major)
    double const* GPs, // n x (4x3 row-major: row a = grad N_a)
    int32_t const* il,
    double const* wgs,
    double const* mus,
    double const* lambdas,
    double const* xti,
    double const* xtildei,
    double mi,
    double kD,
    double sdt,
    double sdt2,
    double detHZero,
    double* xio,
    double* gout,
    double* Hout)
{
    mini::SMatrix<double, 3, 3> Hi = mini::Zeros<double, 3, 3>();
    mini::SVector<double, 3> gi    = mini::Zeros<double, 3, 1>();
    for (int32_t q = 0; q < n; ++q)
    {
        mini::SMatrix<double, 4, 3> GPe;
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                GPe(a, d) = GPs[12 * q + 3 * a + d];
        mini::SMatrix<double, 3, 4> xq = load<3, 4>(xe + 12 * q);
        mini::SMatrix<double, 3, 3> Fe = xq * GPe;
        pbat::physics::StableNeoHookeanEnergy<3> Psi{};
        mini::SVector<double, 9> gF;
        mini::SMatrix<double, 9, 9> HF;
        Psi.gradAndHessian(Fe, mus[q], lambdas[q], gF, HF);
        pbat::sim::vbd::kernels::AccumulateElasticHessian(il[q], wgs[q], GPe, HF, Hi);
        pbat::sim::vbd::kernels::AccumulateElasticGradient(il[q], wgs[q], GPe, gF, gi);
    }
    mini::SVector<double, 3> xt  = load<3, 1>(xti);
    mini::SVector<double, 3> xtl = load<3, 1>(xtildei);
    mini::SVector<double, 3> x   = load<3, 1>(xio);
    pbat::sim::vbd::kernels::AddDamping(sdt, xt, x, kD, gi, Hi);
    pbat::sim::vbd::kernels::AddInertiaDerivatives(sdt2, mi, xtl, x, gi, Hi);
    if (gout)
        for (int r = 0; r < 3; ++r)
            gout[r] = gi(r);
    if (Hout)
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                Hout[3 * c + r] = Hi(r, c);
    pbat::sim::vbd::kernels::IntegratePositions(gi, Hi, x, detHZero);
    for (int r = 0; r < 3; ++r)
        xio[r] = x(r);
}

} // namespace

extern "C" {

double ref_snh_eval(double const* F, double mu, double lambda)
{
    pbat::physics::StableNeoHookeanEnergy<3> Psi{};
    return Psi.eval(load<3, 3>(F), mu, lambda);
}

void ref_snh_grad_hessian(double const* F, double mu, double lambda, double* g, double* H)
{
    pbat::physics::StableNeoHookeanEnergy<3> Psi{};
    mini::SVector<double, 9> gF;
    mini::SMatrix<double, 9, 9> HF;
    Psi.gradAndHessian(load<3, 3>(F), mu, lambda, gF, HF);
    for (int k = 0; k < 9; ++k)
        g[k] = gF(k);
    for (int r = 0; r < 9; ++r)
        for (int c = 0; c < 9; ++c)
            H[r * 9 + c] = HF(r, c);
}

void ref_snh_grad(double const* F, double mu, double lambda, double* g)
{
    pbat::physics::StableNeoHookeanEnergy<3> Psi{};
    auto G = Psi.grad(load<3, 3>(F), mu, lambda);
    for (int k = 0; k < 9; ++k)
        g[k] = G(k);
}

void ref_initial_positions(
    double const* xt,
    double const* vtm1,
    double const* vt,
    double const* a,
    double dt,
    double dt2,
    int32_t strategy,
    double* x)
{
    auto r = pbat::sim::vbd::kernels::InitialPositionsForSolve(
        load<3, 1>(xt),
        load<3, 1>(vtm1),
        load<3, 1>(vt),
        load<3, 1>(a),
        dt,
        dt2,
        static_cast<EInitializationStrategy>(strategy));
    for (int k = 0; k < 3; ++k)
        x[k] = r(k);
}

double ref_chebyshev_omega(int32_t k, double rho2, double omega)
{
    return pbat::sim::vbd::kernels::ChebyshevOmega(k, rho2, omega);
}

void ref_vertex_solve(
    int32_t n,
    double const* xe,
    double const* GPs,
    int32_t const* il,
    double const* wgs,
    double const* mus,
    double const* lambdas,
    double const* xti,
    double const* xtildei,
    double mi,
    double kD,
    double sdt,
    double sdt2,
    double detHZero,
    double* xi,
    double* gout,
    double* Hout)
{
    ref_vertex_solve_impl(
        n, xe, GPs, il, wgs, mus, lambdas, xti, xtildei, mi, kD, sdt, sdt2, detHZero, xi, gout, Hout);
}

// graph::GreedyColor on a CSR vertex graph (neighbours including self).
void ref_greedy_color(
    int32_t n,
    int32_t const* ptr,
    int32_t const* adj,
    int32_t ordering,
    int32_t selection,
    int32_t* colors)
{
    Eigen::Vector<int32_t, Eigen::Dynamic> p(n + 1), a(ptr[n]);
    for (int32_t i = 0; i <= n; ++i)
        p(i) = ptr[i];
    for (int32_t k = 0; k < ptr[n]; ++k)
        a(k) = adj[k];
    auto C = pbat::graph::GreedyColor(
        p,
        a,
        static_cast<pbat::graph::EGreedyColorOrderingStrategy>(ordering),
        static_cast<pbat::graph::EGreedyColorSelectionStrategy>(selection));
    for (int32_t i = 0; i < n; ++i)
        colors[i] = C(i);
}

uint32_t ref_morton3d(float x, float y, float z)
{
    std::array<float, 3> p{x, y, z};
    return pbat::geometry::Morton3D(p);
}

// Vertex-triangle contact energy/gradient/Hessian (sim/vbd/Kernels.h:215-302), FP32 like the
// reference's GPU kernel.  xtf, xf: 3x3 column-major triangle vertex positions.
float ref_vertex_triangle_contact(
    float const* xtv,
    float const* xv,
    float const* xtf,
    float const* xf,
    float dt,
    float muC,
    float muF,
    float epsv,
    float* g,
    float* H)
{
    mini::SVector<float, 3> xtv_, xv_;
    mini::SMatrix<float, 3, 3> xtf_, xf_;
    for (int r = 0; r < 3; ++r)
    {
        xtv_(r) = xtv[r];
        xv_(r)  = xv[r];
        for (int c = 0; c < 3; ++c)
        {
            xtf_(r, c) = xtf[3 * c + r];
            xf_(r, c)  = xf[3 * c + r];
        }
    }
    mini::SVector<float, 3> gi = mini::Zeros<float, 3, 1>();
    mini::SMatrix<float, 3, 3> Hi = mini::Zeros<float, 3, 3>();
    for (int r = 0; r < 3; ++r)
    {
        gi(r) = g[r];
        for (int c = 0; c < 3; ++c)
            Hi(r, c) = H[3 * c + r];
    }
    float E = pbat::sim::vbd::kernels::AccumulateVertexTriangleContact(
        xtv_, xv_, xtf_, xf_, dt, muC, muF, epsv, &gi, &Hi);
    for (int r = 0; r < 3; ++r)
    {
        g[r] = gi(r);
        for (int c = 0; c < 3; ++c)
            H[3 * c + r] = Hi(r, c);
    }
    return E;
}

// The same kernel instantiated in FP64.
double ref_vertex_triangle_contact_d(
    double const* xtv,
    double const* xv,
    double const* xtf,
    double const* xf,
    double dt,
    double muC,
    double muF,
    double epsv,
    double* g,
    double* H)
{
    mini::SVector<double, 3> xtv_ = load<3, 1>(xtv), xv_ = load<3, 1>(xv);
    mini::SMatrix<double, 3, 3> xtf_ = load<3, 3>(xtf), xf_ = load<3, 3>(xf);
    mini::SVector<double, 3> gi      = load<3, 1>(g);
    mini::SMatrix<double, 3, 3> Hi   = load<3, 3>(H);
    double E = pbat::sim::vbd::kernels::AccumulateVertexTriangleContact(xtv_, xv_, xtf_, xf_, dt, muC, muF, epsv, &gi, &Hi);
    for (int r = 0; r < 3; ++r)
    {
        g[r] = gi(r);
        for (int c = 0; c < 3; ++c)
            H[3 * c + r] = Hi(r, c);
    }
    return E;
}

// A full step loop (sim/vbd/Integrator.cpp:22-96, ChebyshevIntegrator.cpp:15-32) whose
// per-vertex work is the reference's own kernels.  Same argument meaning as orc_run.
int ref_run(orc_problem const* Pp, double* x, double* v, double* vprev, double dt, int32_t iterations, int32_t substeps, int32_t nsteps)
{
    orc_problem const& P = *Pp;
    int32_t const nV     = P.nV;
    std::vector<double> xt(size_t(nV) * 3), xtilde(size_t(nV) * 3), vtm1(size_t(nV) * 3), xkm1, xkm2;
    if (P.acceleration == 1)
    {
        xkm1.assign(x, x + size_t(nV) * 3);
        xkm2.assign(x, x + size_t(nV) * 3);
    }
    double const sdt  = dt / double(substeps);
    double const sdt2 = sdt * sdt;
    std::vector<double> xe, GPs, wgs, mus, las;
    std::vector<int32_t> ils;
    for (int32_t step = 0; step < nsteps; ++step)
        for (int32_t s = 0; s < substeps; ++s)
        {
            std::memcpy(xt.data(), x, sizeof(double) * 3 * size_t(nV));
            std::memcpy(vtm1.data(), P.semantics == 1 ? vprev : v, sizeof(double) * 3 * size_t(nV));
            for (int32_t i = 0; i < nV; ++i)
            {
                auto y = pbat::sim::vbd::kernels::InertialTarget(
                    load<3, 1>(&xt[3 * size_t(i)]),
                    load<3, 1>(v + 3 * size_t(i)),
                    load<3, 1>(P.aext + 3 * size_t(i)),
                    sdt,
                    sdt2);
                for (int d = 0; d < 3; ++d)
                    xtilde[3 * size_t(i) + d] = y(d);
                ref_initial_positions(
                    &xt[3 * size_t(i)],
                    &vtm1[3 * size_t(i)],
                    v + 3 * size_t(i),
                    P.aext + 3 * size_t(i),
                    sdt,
                    sdt2,
                    P.strategy,
                    x + 3 * size_t(i));
            }
            double const rho2 = P.rho * P.rho;
            double omega      = 0;
            for (int32_t k = 0; k < iterations; ++k)
            {
                for (int32_t p = 0; p < P.nPartitions; ++p)
                    for (int32_t kk = P.Pptr[p]; kk < P.Pptr[p + 1]; ++kk)
                    {
                        int32_t const i = P.Padj[kk];
                        int32_t const b = P.GVGp[i], e = P.GVGp[i + 1], n = e - b;
                        xe.resize(size_t(n) * 12);
                        GPs.resize(size_t(n) * 12);
                        wgs.resize(n);
                        mus.resize(n);
                        las.resize(n);
                        ils.resize(n);
                        for (int32_t q = 0; q < n; ++q)
                        {
                            int32_t const el = P.GVGe[b + q];
                            ils[q]           = P.GVGilocal[b + q];
                            wgs[q]           = P.wg[el];
                            mus[q]           = P.mu[el];
                            las[q]           = P.lambda[el];
                            for (int a = 0; a < 4; ++a)
                                for (int r = 0; r < 3; ++r)
                                    xe[12 * q + 3 * a + r] = x[3 * P.T[4 * el + a] + r];
                            for (int c = 0; c < 12; ++c)
                                GPs[12 * q + c] = P.GP[12 * el + c];
                        }
                        ref_vertex_solve_impl(
                            n,
                            xe.data(),
                            GPs.data(),
                            ils.data(),
                            wgs.data(),
                            mus.data(),
                            las.data(),
                            &xt[3 * size_t(i)],
                            &xtilde[3 * size_t(i)],
                            P.m[i],
                            P.kD,
                            sdt,
                            sdt2,
                            P.detHZero,
                            x + 3 * size_t(i),
                            nullptr,
                            nullptr);
                    }
                if (P.acceleration == 1)
                {
                    omega = pbat::sim::vbd::kernels::ChebyshevOmega(k, rho2, omega);
                    for (size_t q = 0; q < size_t(nV) * 3; ++q)
                    {
                        if (k > 1)
                            x[q] = omega * (x[q] - xkm2[q]) + xkm2[q];
                        xkm2[q] = xkm1[q];
                        xkm1[q] = x[q];
                    }
                }
            }
            for (size_t q = 0; q < size_t(nV) * 3; ++q)
            {
                if (vprev)
                    vprev[q] = v[q];
                v[q] = (x[q] - xt[q]) / sdt;
            }
        }
    return 0;
}

// The reference's own CCD queries (geometry/PointTriangleCcd.h:125-160, geometry/EdgeEdgeCcd.h:
// 125-161) in FP64.  xt, x: four points at the start and the end of the step, 3 doubles each
// (point-triangle: x, a, b, c; edge-edge: p1, q1, p2, q2).  out: the reference's result vector
// (point-triangle: t and three barycentric coordinates; edge-edge: t and two edge parameters).
void ref_point_triangle_ccd(double const* xt, double const* x, double* out)
{
    mini::SVector<double, 3> P[8];
    for (int k = 0; k < 4; ++k)
        for (int r = 0; r < 3; ++r)
        {
            P[k](r)     = xt[3 * k + r];
            P[4 + k](r) = x[3 * k + r];
        }
    mini::SVector<double, 4> const r = pbat::geometry::PointTriangleCcd(P[0], P[1], P[2], P[3], P[4], P[5], P[6], P[7]);
    for (int k = 0; k < 4; ++k)
        out[k] = r(k);
}

void ref_edge_edge_ccd(double const* xt, double const* x, double* out)
{
    mini::SVector<double, 3> P[8];
    for (int k = 0; k < 4; ++k)
        for (int r = 0; r < 3; ++r)
        {
            P[k](r)     = xt[3 * k + r];
            P[4 + k](r) = x[3 * k + r];
        }
    mini::SVector<double, 3> const r = pbat::geometry::EdgeEdgeCcd(P[0], P[1], P[2], P[3], P[4], P[5], P[6], P[7]);
    for (int k = 0; k < 3; ++k)
        out[k] = r(k);
}

} // extern "C"
