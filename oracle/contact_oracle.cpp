// FP64 restatement of the reference GPU integrator's contact-enabled VBD step (TEST
// INFRASTRUCTURE ONLY; see vbd_oracle.cpp).
//
//   Step order          gpu/impl/vbd/Integrator.cu:82-103 (active set on the full-step prediction,
//                       per substep: inertial target, initial guess, contact list, sweeps,
//                       velocity; finalise at the end), GPU velocity semantics
//   active set          gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:51-223, with brute-force
//                       overlaps instead of the BVH (the same sets: every box pair is tested); the
//                       search radius of a vertex overlapping several triangles is the largest
//                       joint-box diagonal
//   nearest triangles   gpu/impl/geometry/Bvh.cuh:347-474: the branch and bound visits the leaves
//                       of the LBVH in descending Morton order (the right child is popped first)
//                       and keeps a FIFO list that restarts on a strictly nearer triangle.  Pruning
//                       never drops a triangle within the current radius, so visiting every
//                       triangle in that leaf order gives the same list; the order is taken from
//                       FP32 Morton codes of the swept triangle boxes at each step's initialise,
//                       stably sorted (the LBVH restatement in lbvh_oracle.cpp)
//   contact energy      gpu/impl/vbd/Kernels.cuh:80-114,203-223 and sim/vbd/Kernels.h:215-302
//   colour pass reads   the reference writes every vertex of a colour to a buffer and copies it
//                       back after the pass, so a contact triangle's corners are read as they were
//                       at the start of the pass; this oracle reads them from a snapshot
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "orc_accel.h"
#include "orc_problem.h"

namespace {

using Real = double;

struct V3
{
    Real x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(Real s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline Real dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 at(Real const* x, int32_t i) { return {x[3 * size_t(i)], x[3 * size_t(i) + 1], x[3 * size_t(i) + 2]}; }

// Closest point on a triangle by Voronoi regions (Ericson, section 5.1.5); squared distance.
Real point_triangle_sqdist(V3 p, V3 a, V3 b, V3 c)
{
    V3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    Real d1 = dot(ab, ap), d2 = dot(ac, ap);
    V3 q;
    if (d1 <= 0 && d2 <= 0)
        q = a;
    else
    {
        V3 bp   = sub(p, b);
        Real d3 = dot(ab, bp), d4 = dot(ac, bp);
        Real vc = d1 * d4 - d3 * d2;
        V3 cp   = sub(p, c);
        Real d5 = dot(ab, cp), d6 = dot(ac, cp);
        Real vb = d5 * d2 - d1 * d6;
        Real va = d3 * d6 - d5 * d4;
        if (d3 >= 0 && d4 <= d3)
            q = b;
        else if (vc <= 0 && d1 >= 0 && d3 <= 0)
            q = add(a, mul(d1 / (d1 - d3), ab));
        else if (d6 >= 0 && d5 <= d6)
            q = c;
        else if (vb <= 0 && d2 >= 0 && d6 <= 0)
            q = add(a, mul(d2 / (d2 - d6), ac));
        else if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0)
            q = add(b, mul((d4 - d3) / ((d4 - d3) + (d5 - d6)), sub(c, b)));
        else
        {
            Real den = 1 / (va + vb + vc);
            q        = add(a, add(mul(vb * den, ab), mul(vc * den, ac)));
        }
    }
    V3 d = sub(p, q);
    return dot(d, d);
}

// sim/vbd/Kernels.h:215-302: adds to g and H (column-major 3x3) and returns the energy (normal
// penalty 1/2 lambda d and IPC friction muF |lambda| f0(|u|), f0 as the reference writes it).
Real vertex_triangle_contact(V3 xtv, V3 xv, V3 const* xtf, V3 const* xf, Real dt, Real muC, Real muF, Real epsv, Real* g, Real* H, Real epsilon = Real(FLT_EPSILON))
{
    V3 e0 = sub(xf[1], xf[0]), e1 = sub(xf[2], xf[0]);
    V3 n  = cross(e0, e1);
    Real const dbl = std::sqrt(dot(n, n));
    if (dbl <= 1e-8)
        return 0;
    n           = mul(1 / dbl, n);
    Real const t = dot(n, sub(xv, xf[0]));
    V3 ap        = sub(sub(xv, mul(t, n)), xf[0]);
    Real d00 = dot(e0, e0), d01 = dot(e0, e1), d11 = dot(e1, e1), d20 = dot(ap, e0), d21 = dot(ap, e1);
    Real denom = d00 * d11 - d01 * d01;
    Real bv = (d11 * d20 - d01 * d21) / denom, bw = (d00 * d21 - d01 * d20) / denom, bu = 1 - bv - bw;
    if (!(bu >= 0 && bu <= 1 && bv >= 0 && bv <= 1 && bw >= 0 && bw <= 1))
        return 0;
    V3 xb  = add(add(mul(bu, xf[0]), mul(bv, xf[1])), mul(bw, xf[2]));
    V3 xtb = add(add(mul(bu, xtf[0]), mul(bv, xtf[1])), mul(bw, xtf[2]));
    Real const dn     = dot(sub(xv, xb), n);
    Real const d      = std::min(Real(0), dn);
    Real const lambda = muC * d;
    Real const nn[3]  = {n.x, n.y, n.z};
    g[0] += lambda * n.x;
    g[1] += lambda * n.y;
    g[2] += lambda * n.z;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            H[3 * c + r] += muC * nn[r] * nn[c];
    V3 b1      = cross(n, e0);
    V3 dx      = sub(sub(xv, xtv), sub(xb, xtb));
    Real u0    = dot(e0, dx), u1 = dot(b1, dx);
    // The reference adds numeric_limits<Scalar>::epsilon(); its contact runs in FP32 on the GPU.
    Real unorm = std::sqrt(u0 * u0 + u1 * u1) + epsilon;
    Real epsvh = epsv * dt;
    Real y     = unorm / epsvh;
    Real f1    = y < 1 ? 2 * y - y * y : Real(1);
    Real s     = muF * std::abs(lambda) * f1 / unorm;
    V3 gt      = add(mul(u0, e0), mul(u1, b1));
    g[0] += s * gt.x;
    g[1] += s * gt.y;
    g[2] += s * gt.z;
    Real const E0[3] = {e0.x, e0.y, e0.z}, E1[3] = {b1.x, b1.y, b1.z};
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            H[3 * c + r] += s * (E0[r] * E0[c] + E1[r] * E1[c]);
    Real const un2 = unorm * unorm;
    return Real(0.5) * lambda * d + muF * std::abs(lambda) * (epsvh / 3 + un2 / epsvh - un2 * unorm / (3 * epsvh * epsvh));
}

// SNH closed-form vertex block in FP64 (same contraction the full 9x9 reference Hessian reduces
// to; the CPU oracle without contact uses the full form, this one is checked against it).
void elastic_block(orc_problem const& P, int32_t i, Real const* x, Real* H, Real* g)
{
    for (int k = 0; k < 9; ++k)
        H[k] = 0;
    g[0] = g[1] = g[2] = 0;
    Real s = 0;
    for (int32_t n = P.GVGp[i]; n < P.GVGp[i + 1]; ++n)
    {
        int32_t const e   = P.GVGe[n];
        int32_t const il  = P.GVGilocal[n];
        int32_t const* t  = P.T + 4 * e;
        double const* GPe = P.GP + 12 * e;
        Real F[9]         = {0};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                for (int r = 0; r < 3; ++r)
                    F[3 * d + r] += x[3 * t[a] + r] * GPe[3 * a + d];
        Real const* w = GPe + 3 * il;
        V3 f0{F[0], F[1], F[2]}, f1{F[3], F[4], F[5]}, f2{F[6], F[7], F[8]};
        V3 k0 = cross(f1, f2), k1 = cross(f2, f0), k2 = cross(f0, f1);
        Real J = dot(f0, k0);
        V3 c   = add(add(mul(w[0], k0), mul(w[1], k1)), mul(w[2], k2));
        V3 Fw  = add(add(mul(w[0], f0), mul(w[1], f1)), mul(w[2], f2));
        Real const mu = P.mu[e] * P.wg[e], la = P.lambda[e] * P.wg[e];
        Real const sl = la * (J - 1 - P.mu[e] / P.lambda[e]);
        g[0] += mu * Fw.x + sl * c.x;
        g[1] += mu * Fw.y + sl * c.y;
        g[2] += mu * Fw.z + sl * c.z;
        s += mu * (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        Real const cc[3] = {c.x, c.y, c.z};
        for (int cc_ = 0; cc_ < 3; ++cc_)
            for (int r = 0; r < 3; ++r)
                H[3 * cc_ + r] += la * cc[r] * cc[cc_];
    }
    H[0] += s;
    H[4] += s;
    H[8] += s;
}

} // namespace

extern "C" {
double orc_objective(orc_problem const* Pp, double const* x, double const* xtilde, double dt);

struct orc_contact
{
    int32_t nSurfV;
    int32_t const* V;
    int32_t nF;
    int32_t const* F; // 3 x nF
    int32_t const* B; // nV
    double const* XVA;
    double const* FA;
    double muC, muF, epsv;
    int32_t freq;
    float wmin[3], wmax[3]; // scene box the Morton codes are normalised by
    // persistent state (caller-owned)
    uint8_t* active;  // nSurfV
    double* dupper;   // nSurfV
    int32_t* fc;      // nV * 8
    // Replay (nullable): contact lists to use at every list update instead of the oracle's own
    // nearest-triangle queries, nV * 8 per update (the device's lists), so that positions can be
    // compared with the discrete decisions held equal.
    int32_t const* forced_fc;
};

namespace {

// Nearest triangles of collision vertex q (gpu/impl/geometry/Bvh.cuh:408-466 with the callbacks of
// gpu/impl/contact/VertexTriangleMixedCcdDcd.cuh:109-162).  order: triangles in the order the
// depth-first traversal reaches their leaves.  Triangles of the vertex's own body are skipped.
void nearest(orc_contact const& C, Real const* x, int32_t q, std::vector<int32_t> const& order, std::vector<int32_t>& list)
{
    int32_t const i = C.V[q];
    V3 const p      = at(x, i);
    Real const eps  = Real(FLT_EPSILON);
    Real dmin       = C.dupper[q];
    list.clear();
    for (int32_t f : order)
    {
        int32_t const* t = C.F + 3 * size_t(f);
        if (C.B[t[0]] == C.B[i])
            continue;
        Real const d = point_triangle_sqdist(p, at(x, t[0]), at(x, t[1]), at(x, t[2]));
        if (d < dmin - eps)
        {
            list.assign(1, f);
            dmin = d;
        }
        else if (d <= dmin + eps && list.size() < 8)
            list.push_back(f);
    }
}

// Leaf order of the LBVH over the FP32 swept triangle boxes, reversed: the depth-first visit order.
extern "C" void orc_morton(int32_t n, float const* lo, float const* hi, float const* wmin, float const* wmax, uint32_t* codes);

void visit_order(orc_contact const& C, std::vector<V3> const& flo, std::vector<V3> const& fhi, std::vector<int32_t>& order)
{
    size_t const n = size_t(C.nF);
    std::vector<float> lo(3 * n), hi(3 * n);
    for (size_t f = 0; f < n; ++f)
    {
        lo[3 * f + 0] = float(flo[f].x);
        lo[3 * f + 1] = float(flo[f].y);
        lo[3 * f + 2] = float(flo[f].z);
        hi[3 * f + 0] = float(fhi[f].x);
        hi[3 * f + 1] = float(fhi[f].y);
        hi[3 * f + 2] = float(fhi[f].z);
    }
    std::vector<uint32_t> codes(n);
    orc_morton(C.nF, lo.data(), hi.data(), C.wmin, C.wmax, codes.data());
    order.resize(n);
    for (size_t f = 0; f < n; ++f)
        order[f] = int32_t(f);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return codes[a] < codes[b]; });
    std::reverse(order.begin(), order.end());
}

} // namespace

// Advance nsteps contact-enabled steps (GPU integrator semantics).  x, v, vprev: nV x 3.
int orc_run_contact(orc_problem const* Pp, orc_contact const* Cp, double* x, double* v, double* vprev, double dt, int32_t iterations, int32_t substeps, int32_t nsteps)
{
    orc_problem const& P = *Pp;
    orc_contact const& C = *Cp;
    int32_t const nV     = P.nV;
    size_t const n3      = size_t(nV) * 3;
    std::vector<Real> xt(n3), xtilde(n3), xpred(n3), snap(n3), vtm1(n3);
    Real const sdt = dt / Real(substeps), sdt2 = sdt * sdt;
    std::vector<int32_t> list, order;
    for (int32_t step = 0; step < nsteps; ++step)
    {
        // InitializeActiveSet on the full-step prediction.
        for (size_t k = 0; k < n3; ++k)
            xpred[k] = x[k] + dt * v[k] + dt * dt * P.aext[k];
        std::vector<V3> flo(size_t(C.nF)), fhi(size_t(C.nF));
        for (int32_t f = 0; f < C.nF; ++f)
        {
            int32_t const* t = C.F + 3 * size_t(f);
            V3 lo = at(x, t[0]), hi = lo;
            for (int k = 0; k < 3; ++k)
                for (Real const* src : {x, xpred.data()})
                {
                    V3 p = at(src, t[k]);
                    lo   = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
                    hi   = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
                }
            flo[f] = lo;
            fhi[f] = hi;
        }
        visit_order(C, flo, fhi, order);
#pragma omp parallel for schedule(dynamic, 16)
        for (int32_t q = 0; q < C.nSurfV; ++q)
        {
            int32_t const i = C.V[q];
            V3 a = at(x, i), b = at(xpred.data(), i);
            V3 lo{std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)};
            V3 hi{std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)};
            Real best = 0;
            bool hit  = false;
            for (int32_t f = 0; f < C.nF; ++f)
            {
                bool const ov = lo.x <= fhi[f].x && lo.y <= fhi[f].y && lo.z <= fhi[f].z && flo[f].x <= hi.x &&
                                flo[f].y <= hi.y && flo[f].z <= hi.z;
                if (!ov)
                    continue;
                int32_t const* t = C.F + 3 * size_t(f);
                if (C.B[i] == C.B[t[0]])
                    continue;
                V3 jl = a, jh = a;
                for (Real const* src : {x, xpred.data()})
                {
                    for (int k = 0; k < 4; ++k)
                    {
                        V3 p = at(src, k < 3 ? t[k] : i);
                        jl   = {std::min(jl.x, p.x), std::min(jl.y, p.y), std::min(jl.z, p.z)};
                        jh   = {std::max(jh.x, p.x), std::max(jh.y, p.y), std::max(jh.z, p.z)};
                    }
                }
                V3 dg = sub(jh, jl);
                best  = std::max(best, dot(dg, dg));
                hit   = true;
            }
            if (hit)
            {
                C.dupper[q] = best;
                C.active[q] = 1;
            }
        }
        for (int32_t s = 0; s < substeps; ++s)
        {
            std::memcpy(xt.data(), x, sizeof(Real) * n3);
            std::memcpy(vtm1.data(), vprev, sizeof(Real) * n3);
            for (int32_t i = 0; i < nV; ++i)
            {
                Real const* vv = v + 3 * size_t(i);
                Real const* aa = P.aext + 3 * size_t(i);
                Real const* tt = xt.data() + 3 * size_t(i);
                Real* xo       = x + 3 * size_t(i);
                for (int d = 0; d < 3; ++d)
                    xtilde[3 * size_t(i) + d] = tt[d] + sdt * vv[d] + sdt2 * aa[d];
                // InitialPositionsForSolve (sim/vbd/Kernels.h:39-94)
                Real an2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
                Real atl = 1;
                if (P.strategy == 0)
                {
                    for (int d = 0; d < 3; ++d)
                        xo[d] = tt[d];
                    continue;
                }
                if (P.strategy == 1)
                    atl = 0;
                else if (P.strategy >= 3)
                {
                    atl = 0;
                    if (an2 != 0)
                    {
                        Real const* vm = vtm1.data() + 3 * size_t(i);
                        if (P.strategy == 3)
                        {
                            Real dd = 0;
                            for (int d = 0; d < 3; ++d)
                                dd += ((vv[d] - vm[d]) / sdt) * aa[d];
                            atl = std::min(std::max(dd / an2, Real(0)), Real(1));
                        }
                        else
                        {
                            Real vn = std::sqrt(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]) + std::numeric_limits<Real>::min();
                            Real dd = 0;
                            for (int d = 0; d < 3; ++d)
                                dd += (vv[d] / vn) * aa[d];
                            atl = std::min(std::abs(dd / an2), Real(1));
                        }
                    }
                }
                for (int d = 0; d < 3; ++d)
                    xo[d] = tt[d] + sdt * vv[d] + sdt2 * atl * aa[d];
            }
            if (s % C.freq == 0 && C.forced_fc)
            {
                size_t const update = (size_t(step) * size_t(substeps) + size_t(s)) / size_t(C.freq);
                std::memcpy(C.fc, C.forced_fc + update * 8 * size_t(nV), sizeof(int32_t) * 8 * size_t(nV));
            }
            else if (s % C.freq == 0)
            {
                for (int32_t q = 0; q < C.nSurfV; ++q)
                {
                    if (!C.active[q])
                        continue;
                    nearest(C, x, q, order, list);
                    int32_t const i = C.V[q];
                    for (int c = 0; c < 8; ++c)
                        C.fc[8 * size_t(i) + c] = c < int(list.size()) ? list[c] : -1;
                }
            }
            auto sweep = [&] {
                for (int32_t p = 0; p < P.nPartitions; ++p)
                {
                    std::memcpy(snap.data(), x, sizeof(Real) * n3);
#pragma omp parallel for schedule(dynamic, 32)
                    for (int32_t kk = P.Pptr[p]; kk < P.Pptr[p + 1]; ++kk)
                    {
                        int32_t const i = P.Padj[kk];
                        Real H[9], g[3];
                        elastic_block(P, i, snap.data(), H, g);
                        Real* xi        = x + 3 * size_t(i);
                        Real const* xti = xt.data() + 3 * size_t(i);
                        Real const D    = P.kD / sdt;
                        Real hx[3]      = {0, 0, 0};
                        for (int r = 0; r < 3; ++r)
                            for (int c = 0; c < 3; ++c)
                                hx[r] += H[3 * c + r] * (xi[c] - xti[c]);
                        for (int r = 0; r < 3; ++r)
                            g[r] += D * hx[r];
                        for (int q = 0; q < 9; ++q)
                            H[q] *= 1 + D;
                        // Contacts: corners as at the start of the pass.
                        int32_t const* f = C.fc + 8 * size_t(i);
                        int nc           = 0;
                        for (int c = 0; c < 8; ++c)
                            nc += f[c] >= 0 ? 1 : 0;
                        if (nc > 0)
                        {
                            Real sumfa = 0;
                            for (int c = 0; c < nc; ++c)
                                sumfa += C.FA[f[c]];
                            Real const kC = C.XVA[i] * C.muC / sumfa;
                            for (int c = 0; c < nc; ++c)
                            {
                                int32_t const* t = C.F + 3 * size_t(f[c]);
                                V3 xtf[3], xf[3];
                                for (int m = 0; m < 3; ++m)
                                {
                                    xtf[m] = at(xt.data(), t[m]);
                                    xf[m]  = at(snap.data(), t[m]);
                                }
                                vertex_triangle_contact(at(xt.data(), i), at(snap.data(), i), xtf, xf, sdt, kC * C.FA[f[c]], C.muF, C.epsv, g, H);
                            }
                        }
                        Real const K = P.m[i] / sdt2;
                        for (int r = 0; r < 3; ++r)
                        {
                            H[4 * r] += K;
                            g[r] += K * (xi[r] - xtilde[3 * size_t(i) + r]);
                        }
                        Real a00 = H[4] * H[8] - H[5] * H[7], a01 = H[7] * H[2] - H[1] * H[8], a02 = H[1] * H[5] - H[4] * H[2];
                        Real a11 = H[0] * H[8] - H[2] * H[6], a12 = H[2] * H[3] - H[0] * H[5], a22 = H[0] * H[4] - H[1] * H[3];
                        Real det = H[0] * a00 + H[3] * a01 + H[6] * a02;
                        if (!(std::abs(det) > P.detHZero))
                            continue;
                        Real const inv = 1 / det;
                        Real const dx0 = inv * (a00 * g[0] + a01 * g[1] + a02 * g[2]);
                        Real const dx1 = inv * (a01 * g[0] + a11 * g[1] + a12 * g[2]);
                        Real const dx2 = inv * (a02 * g[0] + a12 * g[1] + a22 * g[2]);
                        xi[0] -= dx0;
                        xi[1] -= dx1;
                        xi[2] -= dx2;
                    }
                }
            };
            // The GPU integrator's accelerations with contact (gpu/vbd/Integrator.cu:15-33 builds
            // Anderson and trust-region integrators whatever the data carries); the objective of
            // the trust region adds the contact energy of the active vertices
            // (gpu/impl/vbd/TrustRegionIntegrator.cu:265-360).
            auto objective = [&] {
                Real f = orc_objective(&P, x, xtilde.data(), sdt);
                for (int32_t q = 0; q < C.nSurfV; ++q)
                {
                    if (!C.active[q])
                        continue;
                    int32_t const i = C.V[q];
                    int32_t const* fl = C.fc + 8 * size_t(i);
                    Real sumfa = 0;
                    int nc     = 0;
                    for (int c = 0; c < 8; ++c)
                        if (fl[c] >= 0)
                            sumfa += C.FA[fl[c]], ++nc;
                    if (nc == 0)
                        continue;
                    Real const kC = C.XVA[i] * C.muC / sumfa;
                    for (int c = 0; c < 8; ++c)
                    {
                        if (fl[c] < 0)
                            continue;
                        int32_t const* t = C.F + 3 * size_t(fl[c]);
                        V3 xtf[3], xf[3];
                        for (int m = 0; m < 3; ++m)
                        {
                            xtf[m] = at(xt.data(), t[m]);
                            xf[m]  = at(x, t[m]);
                        }
                        Real g[3] = {0, 0, 0}, H[9] = {0};
                        f += vertex_triangle_contact(at(xt.data(), i), at(x, i), xtf, xf, sdt, kC * C.FA[fl[c]], C.muF, C.epsv, g, H);
                    }
                }
                return f;
            };
            if (P.acceleration == 2)
                orc::anderson_solve(P, x, nV, iterations, sweep);
            else if (P.acceleration == 5 && !P.tr_curved)
            {
                size_t const entry = 4 * (size_t(step) * size_t(substeps) + size_t(s)) * size_t(iterations);
                orc::trust_region_solve(P, x, nV, iterations, sweep, objective, P.tr_forced ? P.tr_forced + entry : nullptr,
                                        P.tr_log ? P.tr_log + entry : nullptr);
            }
            else
                for (int32_t k = 0; k < iterations; ++k)
                    sweep();
            for (size_t k = 0; k < n3; ++k)
            {
                vprev[k] = v[k];
                v[k]     = (x[k] - xt[k]) / sdt;
            }
        }
        // FinalizeActiveSet: a vertex stays active while behind its nearest triangle's plane.
        for (int32_t q = 0; q < C.nSurfV; ++q)
        {
            if (!C.active[q])
                continue;
            nearest(C, x, q, order, list);
            if (list.empty())
                continue;
            int32_t const* t = C.F + 3 * size_t(list.back());
            V3 a = at(x, t[0]);
            V3 nrm = cross(sub(at(x, t[1]), a), sub(at(x, t[2]), a));
            C.active[q] = dot(sub(at(x, C.V[q]), a), nrm) < 0 ? 1 : 0;
        }
    }
    return 0;
}

// FP64 evaluation of one vertex-triangle contact (for comparison with the reference's kernel);
// epsilon regularises |u| (FLT_EPSILON for the GPU path, DBL_EPSILON for an FP64 instantiation).
void orc_vertex_triangle_contact(double const* xtv, double const* xv, double const* xtf, double const* xf, double dt, double muC, double muF, double epsv, double epsilon, double* g, double* H)
{
    V3 tf[3], f[3];
    for (int k = 0; k < 3; ++k)
    {
        tf[k] = at(xtf, k);
        f[k]  = at(xf, k);
    }
    vertex_triangle_contact(at(xtv, 0), at(xv, 0), tf, f, dt, muC, muF, epsv, g, H, epsilon);
}

// ---------------------------------------------------------------------------------------------
// Discrete half of the CPU multibody mesh contact detector (sim/contact/MultibodyMeshMixedCcdDcd.h:
// ForEachBodyPair 733-751, ForEachPenetratingVertex 754-803, HandleDcdPairs 805-845), an
// independent check on the GPU path's active set and contact lists:
//   * body pairs: bodies whose collision-vertex boxes overlap, both orders;
//   * a collision vertex of body oi penetrates body oj when it lies in one of oj's tetrahedra
//     (geometry/OverlapQueries.h:562-587: outside any face plane, d > 0, means outside; the
//     boundary counts as inside); the first body found is kept (bodies in increasing order here;
//     the reference takes its BVH's visit order, which matters only for a vertex inside two bodies);
//   * each penetrating vertex reports the nearest surface triangles of the body it penetrates
//     (AabbKdTreeHierarchy::NearestNeighbours with radius = max and eps = 0: exact ties only),
//     at most 8, in triangle index order.
// Brute force over tetrahedra and triangles with box prefilters: for test-sized scenes.
// body[q] = penetrated body or -1; nearest[8 q ..] = triangles (-1 pad); d2[q] = their squared
// distance (or -1).  The continuous half follows below (orc_ccd_vertex_triangle,
// orc_ccd_vertex_triangle_pairs, orc_ccd_edge_edge).
int orc_dcd_contacts(
    int32_t nV,
    double const* x,
    int32_t nT,
    int32_t const* T,
    int32_t nF,
    int32_t const* F,
    int32_t nCV,
    int32_t const* V,
    int32_t const* B,
    int32_t* body,
    int32_t* nearest,
    double* d2)
{
    (void)nV;
    int32_t nB = 0;
    for (int32_t q = 0; q < nCV; ++q)
        nB = std::max(nB, B[V[q]] + 1);
    std::vector<V3> blo(static_cast<size_t>(nB), V3{1e300, 1e300, 1e300}), bhi(static_cast<size_t>(nB), V3{-1e300, -1e300, -1e300});
    for (int32_t q = 0; q < nCV; ++q)
    {
        V3 const p = at(x, V[q]);
        int32_t const b = B[V[q]];
        blo[size_t(b)] = {std::min(blo[size_t(b)].x, p.x), std::min(blo[size_t(b)].y, p.y), std::min(blo[size_t(b)].z, p.z)};
        bhi[size_t(b)] = {std::max(bhi[size_t(b)].x, p.x), std::max(bhi[size_t(b)].y, p.y), std::max(bhi[size_t(b)].z, p.z)};
    }
    auto overlap = [](V3 l1, V3 u1, V3 l2, V3 u2) {
        return l1.x <= u2.x && l1.y <= u2.y && l1.z <= u2.z && l2.x <= u1.x && l2.y <= u1.y && l2.z <= u1.z;
    };
    // Tetrahedra and triangles per body, with their boxes.
    std::vector<std::vector<int32_t>> tetsOf(static_cast<size_t>(nB)), trisOf(static_cast<size_t>(nB));
    std::vector<V3> tlo(static_cast<size_t>(nT)), thi(static_cast<size_t>(nT));
    for (int32_t e = 0; e < nT; ++e)
    {
        int32_t const* t = T + 4 * size_t(e);
        if (B[t[0]] < nB)
            tetsOf[size_t(B[t[0]])].push_back(e);
        V3 l = at(x, t[0]), u = l;
        for (int a = 1; a < 4; ++a)
        {
            V3 const p = at(x, t[a]);
            l = {std::min(l.x, p.x), std::min(l.y, p.y), std::min(l.z, p.z)};
            u = {std::max(u.x, p.x), std::max(u.y, p.y), std::max(u.z, p.z)};
        }
        tlo[size_t(e)] = l;
        thi[size_t(e)] = u;
    }
    for (int32_t f = 0; f < nF; ++f)
        if (B[F[3 * size_t(f)]] < nB)
            trisOf[size_t(B[F[3 * size_t(f)]])].push_back(f);
    auto outside = [](V3 p, V3 a, V3 b, V3 c) { return dot(sub(p, a), cross(sub(b, a), sub(c, a))) > 0; };
    for (int32_t q = 0; q < nCV; ++q)
    {
        body[q] = -1;
        d2[q]   = -1;
        for (int k = 0; k < 8; ++k)
            nearest[8 * size_t(q) + size_t(k)] = -1;
        V3 const p     = at(x, V[q]);
        int32_t const oi = B[V[q]];
        for (int32_t oj = 0; oj < nB && body[q] < 0; ++oj)
        {
            if (oj == oi || !overlap(blo[size_t(oi)], bhi[size_t(oi)], blo[size_t(oj)], bhi[size_t(oj)]))
                continue;
            for (int32_t e : tetsOf[size_t(oj)])
            {
                if (!overlap(p, p, tlo[size_t(e)], thi[size_t(e)]))
                    continue;
                int32_t const* t = T + 4 * size_t(e);
                V3 const A = at(x, t[0]), Bv = at(x, t[1]), Cv = at(x, t[2]), D = at(x, t[3]);
                if (outside(p, A, Bv, D) || outside(p, Bv, Cv, D) || outside(p, Cv, A, D) || outside(p, A, Cv, Bv))
                    continue;
                body[q] = oj;
                break;
            }
        }
        if (body[q] < 0)
            continue;
        Real best = std::numeric_limits<Real>::max();
        int count = 0;
        for (int32_t f : trisOf[size_t(body[q])])
        {
            int32_t const* t = F + 3 * size_t(f);
            Real const d = point_triangle_sqdist(p, at(x, t[0]), at(x, t[1]), at(x, t[2]));
            if (d < best)
            {
                best  = d;
                count = 0;
            }
            if (d == best && count < 8)
                nearest[8 * size_t(q) + size_t(count++)] = f;
        }
        for (int k = count; k < 8; ++k)
            nearest[8 * size_t(q) + size_t(k)] = -1;
        d2[q] = best;
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Continuous half, vertex-triangle part (sim/contact/MultibodyMeshMixedCcdDcd.h
// ReportVertexTriangleCcdContacts; geometry/PointTriangleCcd.h:125-160): the earliest time
// t in [0, 1] at which a linearly moving point lies in a linearly moving triangle.  The
// coplanarity condition ((b - a) x (c - a)) . (x - a) = 0 is a cubic in t; its roots in [0, 1] are
// visited in increasing order and the first one whose barycentric coordinates
// (geometry/IntersectionQueries.h:50-67) all lie in [0, 1] is the time of impact.  The reference
// finds the roots with the solver of its math/polynomial/Roots.h; this restatement brackets them
// between the cubic's critical points and bisects each bracket to full precision.  Brute force over
// the triangles of other bodies whose swept boxes overlap the vertex's swept box: for test-sized
// scenes.  t[q] = earliest time of impact of collision vertex q (-1: none), f[q] = its triangle.
// orc_ccd_vertex_triangle_pairs reports every hit pair instead, as the reference's callback does.

namespace {

// Roots of c0 + c1 t + c2 t^2 + c3 t^3 in [0, 1], increasing.  As in the reference's root finder
// (math/polynomial/Roots.h, the cubic method of C. Yuksel, "High-Performance Polynomial Root
// Finding for Graphics", HPG 2022), [0, 1] is cut at the real critical points and a piece holds a
// root when the sign bits of its end values differ (a value of exactly 0 counts as positive, so a
// root exactly at t = 0 is not reported unless the cubic goes negative after it).  Each such piece
// is bisected to full precision, stopping early at an exact zero.
int cubic_roots_01(Real const c[4], Real* roots)
{
    auto f  = [&](Real t) { return ((c[3] * t + c[2]) * t + c[1]) * t + c[0]; };
    auto df = [&](Real t) { return (3 * c[3] * t + 2 * c[2]) * t + c[1]; };
    // Breakpoints: 0, the real critical points inside (0, 1), 1.
    Real bp[4];
    int nb   = 0;
    bp[nb++] = 0;
    Real const qa = 3 * c[3], qb = 2 * c[2], qc = c[1];
    Real crit[2];
    int nc = 0;
    if (qa != 0)
    {
        Real const disc = qb * qb - 4 * qa * qc;
        if (disc > 0)
        {
            Real const sq = std::sqrt(disc);
            Real const r0 = (-qb - sq) / (2 * qa), r1 = (-qb + sq) / (2 * qa);
            crit[nc++] = std::min(r0, r1);
            crit[nc++] = std::max(r0, r1);
        }
    }
    else if (qb != 0)
        crit[nc++] = -qc / qb;
    for (int k = 0; k < nc; ++k)
        if (crit[k] > 0 && crit[k] < 1)
            bp[nb++] = crit[k];
    bp[nb++] = 1;
    int n = 0;
    for (int k = 0; k + 1 < nb; ++k)
    {
        Real lo = bp[k], hi = bp[k + 1];
        Real flo = f(lo), fhi = f(hi);
        if ((flo < 0) == (fhi < 0))
            continue;
        // Newton from the middle of the piece, clamped to it, while it moves (at most 16 steps).
        Real xr = Real(0.5) * (lo + hi);
        bool done = false;
        for (int it = 0; it < 16; ++it)
        {
            Real const xn = std::min(std::max(xr - f(xr) / df(xr), lo), hi);
            if (xn == xr)
            {
                done = true;
                break;
            }
            xr = xn;
        }
        if (done && std::isfinite(xr))
        {
            roots[n++] = xr;
            continue;
        }
        for (int it = 0; it < 200 && hi - lo > 0; ++it)
        {
            Real const mid = Real(0.5) * (lo + hi);
            if (mid <= lo || mid >= hi)
                break;
            Real const fm = f(mid);
            if (fm == 0)
            {
                lo = hi = mid;
                break;
            }
            if ((fm < 0) == (flo < 0))
                lo = mid, flo = fm;
            else
                hi = mid;
        }
        roots[n++] = Real(0.5) * (lo + hi);
    }
    return n;
}

Real point_triangle_ccd(V3 xt, V3 at, V3 bt, V3 ct, V3 x, V3 a, V3 b, V3 c)
{
    V3 const E1 = sub(bt, at), E2 = sub(ct, at), Q = sub(xt, at);
    V3 const D1 = sub(sub(b, a), E1), D2 = sub(sub(c, a), E2), DQ = sub(sub(x, a), Q);
    V3 const n0 = cross(E1, E2);
    V3 const n1 = add(cross(E1, D2), cross(D1, E2));
    V3 const n2 = cross(D1, D2);
    Real const coeff[4] = {dot(n0, Q), dot(n0, DQ) + dot(n1, Q), dot(n1, DQ) + dot(n2, Q), dot(n2, DQ)};
    Real roots[3];
    int const nr = cubic_roots_01(coeff, roots);
    for (int k = 0; k < nr; ++k)
    {
        Real const t = roots[k];
        auto lerp    = [&](V3 p0, V3 p1) { return add(p0, mul(t, sub(p1, p0))); };
        V3 const P = lerp(xt, x), A = lerp(at, a), B = lerp(bt, b), Cc = lerp(ct, c);
        V3 const ab = sub(B, A), ac = sub(Cc, A), ap = sub(P, A);
        Real const d00 = dot(ab, ab), d01 = dot(ab, ac), d11 = dot(ac, ac), d20 = dot(ap, ab), d21 = dot(ap, ac);
        Real const den = d00 * d11 - d01 * d01;
        Real const v = (d11 * d20 - d01 * d21) / den, w = (d00 * d21 - d01 * d20) / den, u = 1 - v - w;
        if (u >= 0 && u <= 1 && v >= 0 && v <= 1 && w >= 0 && w <= 1)
            return t;
    }
    return -1;
}

// Closest points of two lines p1 + a (q1 - p1) and p2 + b (q2 - p2) (geometry/ClosestPointQueries.h
// Lines, 448-485): a line whose squared length is <= eps is a point; lines whose Gram determinant
// lies in [-eps, eps] are parallel and keep a = 0.
void closest_on_lines(V3 p1, V3 q1, V3 p2, V3 q2, Real eps, Real& a, Real& b)
{
    V3 const d1 = sub(q1, p1), d2 = sub(q2, p2), r = sub(p1, p2);
    Real const d1sq = dot(d1, d1), d2sq = dot(d2, d2), d12 = dot(d1, d2);
    Real const gram = d1sq * d2sq - d12 * d12;
    bool const point1 = d1sq <= eps, point2 = d2sq <= eps, parallel = -eps <= gram && gram <= eps;
    a = 0;
    b = 0;
    if (point1 && point2)
        return;
    if (point1)
        b = dot(r, d2) / d2sq;
    else if (point2)
        a = -dot(r, d1) / d1sq;
    else
    {
        if (!parallel)
            a = dot(r, sub(mul(d12, d2), mul(d2sq, d1))) / gram;
        b = dot(add(r, mul(a, d1)), d2) / d2sq;
    }
}

// Edge-edge CCD (geometry/EdgeEdgeCcd.h:125-161): the candidate times are the roots in [0, 1] of
// the cubic ((q1 - p1) x (q2 - p2)) . (p2 - p1), visited in increasing order; at each, the closest
// points of the two lines are taken with eps = DBL_MIN and the root is a hit when both parameters
// lie in [0, 1] and the squared distance of the two points is <= DBL_MIN (only crossings that are
// exact in floating point count).  As written, the cubic's generator (python/geometry/ccd.py:55,
// expanded in EdgeEdgeCcd.h's EdgeEdgeCcdUnivariatePolynomial) moves the second edge's far end
// as q2(t) = Q2T + t (Q2 - P2T) instead of Q2T + t (Q2 - Q2T), so q2 - p2 = (Q2T - P2T) +
// t (Q2 - P2); the hit test at each root uses the true positions.  Both are kept as written.
// Returns t (-1: none) and the two edge parameters (on a miss, those of the last root visited,
// as in the reference's result vector; 0 without roots).
Real edge_edge_ccd(V3 p1t, V3 q1t, V3 p2t, V3 q2t, V3 p1, V3 q1, V3 p2, V3 q2, Real& u, Real& v)
{
    V3 const A0 = sub(q1t, p1t), B0 = sub(q2t, p2t), C0 = sub(p2t, p1t);
    V3 const A1 = sub(sub(q1, p1), A0), B1 = sub(q2, p2), C1 = sub(sub(p2, p1), C0);
    V3 const n0 = cross(A0, B0);
    V3 const n1 = add(cross(A0, B1), cross(A1, B0));
    V3 const n2 = cross(A1, B1);
    Real const coeff[4] = {dot(n0, C0), dot(n0, C1) + dot(n1, C0), dot(n1, C1) + dot(n2, C0), dot(n2, C1)};
    Real roots[3];
    int const nr = cubic_roots_01(coeff, roots);
    Real constexpr tiny = std::numeric_limits<Real>::min();
    for (int k = 0; k < nr; ++k)
    {
        Real const t = roots[k];
        auto lerp    = [&](V3 a0, V3 a1) { return add(a0, mul(t, sub(a1, a0))); };
        V3 const P1 = lerp(p1t, p1), Q1 = lerp(q1t, q1), P2 = lerp(p2t, p2), Q2 = lerp(q2t, q2);
        Real a, b;
        closest_on_lines(P1, Q1, P2, Q2, tiny, a, b);
        V3 const d    = sub(add(P1, mul(a, sub(Q1, P1))), add(P2, mul(b, sub(Q2, P2))));
        bool const in = a >= 0 && a <= 1 && b >= 0 && b <= 1;
        u = a;
        v = b;
        if (in && dot(d, d) <= tiny)
            return t;
    }
    if (nr == 0)
        u = v = 0;
    return -1;
}

struct Box
{
    V3 lo, hi;
};

Box swept_box(double const* xt, double const* x, int32_t const* idx, int n)
{
    Box b{at(xt, idx[0]), at(xt, idx[0])};
    for (int k = 0; k < n; ++k)
        for (double const* src : {xt, x})
        {
            V3 const p = at(src, idx[k]);
            b.lo = {std::min(b.lo.x, p.x), std::min(b.lo.y, p.y), std::min(b.lo.z, p.z)};
            b.hi = {std::max(b.hi.x, p.x), std::max(b.hi.y, p.y), std::max(b.hi.z, p.z)};
        }
    return b;
}

bool boxes_overlap(Box const& a, Box const& b)
{
    return a.lo.x <= b.hi.x && a.lo.y <= b.hi.y && a.lo.z <= b.hi.z && b.lo.x <= a.hi.x && b.lo.y <= a.hi.y &&
           b.lo.z <= a.hi.z;
}

} // namespace

int orc_ccd_vertex_triangle(
    int32_t nV,
    double const* xt,
    double const* x,
    int32_t nF,
    int32_t const* F,
    int32_t nCV,
    int32_t const* V,
    int32_t const* B,
    double* toi,
    int32_t* tri)
{
    (void)nV;
    std::vector<V3> flo(static_cast<size_t>(nF)), fhi(static_cast<size_t>(nF));
    for (int32_t f = 0; f < nF; ++f)
    {
        int32_t const* t = F + 3 * size_t(f);
        V3 l = at(xt, t[0]), u = l;
        for (int k = 0; k < 3; ++k)
            for (double const* src : {xt, x})
            {
                V3 const p = at(src, t[k]);
                l = {std::min(l.x, p.x), std::min(l.y, p.y), std::min(l.z, p.z)};
                u = {std::max(u.x, p.x), std::max(u.y, p.y), std::max(u.z, p.z)};
            }
        flo[size_t(f)] = l;
        fhi[size_t(f)] = u;
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (int32_t q = 0; q < nCV; ++q)
    {
        int32_t const i = V[q];
        V3 const p0 = at(xt, i), p1 = at(x, i);
        V3 const l{std::min(p0.x, p1.x), std::min(p0.y, p1.y), std::min(p0.z, p1.z)};
        V3 const u{std::max(p0.x, p1.x), std::max(p0.y, p1.y), std::max(p0.z, p1.z)};
        Real best    = -1;
        int32_t bestF = -1;
        for (int32_t f = 0; f < nF; ++f)
        {
            int32_t const* t = F + 3 * size_t(f);
            if (B[t[0]] == B[i])
                continue;
            if (!(l.x <= fhi[size_t(f)].x && l.y <= fhi[size_t(f)].y && l.z <= fhi[size_t(f)].z && flo[size_t(f)].x <= u.x &&
                  flo[size_t(f)].y <= u.y && flo[size_t(f)].z <= u.z))
                continue;
            Real const tc = point_triangle_ccd(p0, at(xt, t[0]), at(xt, t[1]), at(xt, t[2]), p1, at(x, t[0]), at(x, t[1]), at(x, t[2]));
            if (tc >= 0 && (best < 0 || tc < best))
            {
                best  = tc;
                bestF = f;
            }
        }
        toi[q] = best;
        tri[q] = bestF;
    }
    return 0;
}

// Every vertex-triangle CCD hit (sim/contact/MultibodyMeshMixedCcdDcd.h
// ReportVertexTriangleCcdContacts 884-932): collision vertex V[q] of one body against each triangle
// of another body whose swept box overlaps the vertex's swept box; vertices flagged in
// penetrating[] (nullable; the discrete half's vertices) are skipped.  Pairs come out ordered by
// (vertex, triangle); at most capacity are written, the return value is the total count.
int64_t orc_ccd_vertex_triangle_pairs(
    int32_t nV,
    double const* xt,
    double const* x,
    int32_t nF,
    int32_t const* F,
    int32_t nCV,
    int32_t const* V,
    int32_t const* B,
    uint8_t const* penetrating,
    int64_t capacity,
    int32_t* vertex,
    int32_t* triangle,
    double* toi)
{
    (void)nV;
    std::vector<Box> fb(static_cast<size_t>(nF));
    for (int32_t f = 0; f < nF; ++f)
        fb[size_t(f)] = swept_box(xt, x, F + 3 * size_t(f), 3);
    int64_t n = 0;
    for (int32_t q = 0; q < nCV; ++q)
    {
        int32_t const i = V[q];
        if (penetrating && penetrating[i])
            continue;
        Box const vb = swept_box(xt, x, &i, 1);
        V3 const p0 = at(xt, i), p1 = at(x, i);
        for (int32_t f = 0; f < nF; ++f)
        {
            int32_t const* t = F + 3 * size_t(f);
            if (B[t[0]] == B[i] || !boxes_overlap(vb, fb[size_t(f)]))
                continue;
            Real const tc = point_triangle_ccd(p0, at(xt, t[0]), at(xt, t[1]), at(xt, t[2]), p1, at(x, t[0]), at(x, t[1]), at(x, t[2]));
            if (tc < 0)
                continue;
            if (n < capacity)
            {
                vertex[n]   = i;
                triangle[n] = f;
                toi[n]      = tc;
            }
            ++n;
        }
    }
    return n;
}

// Every edge-edge CCD hit (sim/contact/MultibodyMeshMixedCcdDcd.h ReportEdgeEdgeCcdContacts
// 934-985): collision edges E[2 e ..] of two different bodies whose swept boxes overlap, neither
// with an end point flagged in penetrating[] (nullable).  Each unordered pair is visited once, with
// the edge of the lower body first (the reference visits each overlapping body pair once, in its
// body tree's order); pairs come out ordered by (first edge, second edge).  tuv[3 n ..] = time of
// impact and the parameters along the first and second edge.  At most capacity are written; the
// return value is the total count.
int64_t orc_ccd_edge_edge(
    int32_t nV,
    double const* xt,
    double const* x,
    int32_t nE,
    int32_t const* E,
    int32_t const* B,
    uint8_t const* penetrating,
    int64_t capacity,
    int32_t* ei,
    int32_t* ej,
    double* tuv)
{
    (void)nV;
    std::vector<Box> eb(static_cast<size_t>(nE));
    for (int32_t e = 0; e < nE; ++e)
        eb[size_t(e)] = swept_box(xt, x, E + 2 * size_t(e), 2);
    auto masked = [&](int32_t const* e) { return penetrating && (penetrating[e[0]] || penetrating[e[1]]); };
    int64_t n = 0;
    for (int32_t a = 0; a < nE; ++a)
    {
        int32_t const* ea = E + 2 * size_t(a);
        if (masked(ea))
            continue;
        for (int32_t b = 0; b < nE; ++b)
        {
            int32_t const* e2 = E + 2 * size_t(b);
            if (B[ea[0]] >= B[e2[0]] || masked(e2) || !boxes_overlap(eb[size_t(a)], eb[size_t(b)]))
                continue;
            Real u, v;
            Real const tc = edge_edge_ccd(at(xt, ea[0]), at(xt, ea[1]), at(xt, e2[0]), at(xt, e2[1]), at(x, ea[0]),
                                          at(x, ea[1]), at(x, e2[0]), at(x, e2[1]), u, v);
            if (tc < 0)
                continue;
            if (n < capacity)
            {
                ei[n]          = a;
                ej[n]          = b;
                tuv[3 * n]     = tc;
                tuv[3 * n + 1] = u;
                tuv[3 * n + 2] = v;
            }
            ++n;
        }
    }
    return n;
}

// One edge-edge CCD query on explicit end points (12 doubles each at t and at t + 1, ordered
// p1, q1, p2, q2); out = (t, u, v), t = -1 when the edges do not cross.
void orc_edge_edge_ccd(double const* xt, double const* x, double* out)
{
    Real u, v;
    out[0] = edge_edge_ccd(at(xt, 0), at(xt, 1), at(xt, 2), at(xt, 3), at(x, 0), at(x, 1), at(x, 2), at(x, 3), u, v);
    out[1] = u;
    out[2] = v;
}

// One vertex-triangle CCD query on explicit end points (x, a, b, c at t and at t + 1); returns t or -1.
double orc_point_triangle_ccd(double const* xt, double const* x)
{
    return point_triangle_ccd(at(xt, 0), at(xt, 1), at(xt, 2), at(xt, 3), at(x, 0), at(x, 1), at(x, 2), at(x, 3));
}

} // extern "C"
