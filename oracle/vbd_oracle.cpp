// FP64 CPU restatement of PBAT's Vertex Block Descent path.
//
// TEST INFRASTRUCTURE ONLY: this file is the parity oracle.  Only the test suite, the smoke check
// and the CPU-baseline leg of the benchmark load it; the product (the CUDA library) never does.
//
// Every function cites the reference function it restates (paths relative to the reference's
// `source/pbat/`).  The arithmetic is FP64, the per-colour vertex loop is OpenMP-parallel (the
// reference's `tbb::parallel_for`, sim/vbd/Integrator.cpp:82-85); vertices of one colour share no
// tetrahedron, so the result does not depend on the thread count.
//
// Pinned by: the reference headers themselves, compiled into `oracle/_ref` by `oracle/Makefile`
// (tests compare this file's SNH derivatives, per-vertex solve, initialisation strategies,
// Chebyshev weights and greedy colouring with the reference's own code), and by the reference
// doctest known-answer values committed under tests/golden/.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Real = double;

// ---------------------------------------------------------------------------------------------
// Small dense helpers (column-major 3x3: A[3*c + r]).
// ---------------------------------------------------------------------------------------------

inline Real det3(Real const* A)
{
    // math/linalg/mini/Determinant.h:31-35 (cofactor expansion along the first row).
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[3] * (A[1] * A[8] - A[2] * A[7]) +
           A[6] * (A[1] * A[5] - A[2] * A[4]);
}

inline void cross3(Real const* a, Real const* b, Real* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Inverse of a 3x3 by cofactors / determinant (math/linalg/mini/Inverse.h:40-55 computes the same
// closed form).
inline void inv3(Real const* A, Real* Ai)
{
    Real c0[3], c1[3], c2[3];
    // Rows of the inverse are cross products of the columns of A divided by det.
    cross3(A + 3, A + 6, c0);
    cross3(A + 6, A + 0, c1);
    cross3(A + 0, A + 3, c2);
    Real const d = A[0] * c0[0] + A[1] * c0[1] + A[2] * c0[2];
    Real const s = Real(1) / d;
    for (int k = 0; k < 3; ++k)
    {
        Ai[3 * k + 0] = c0[k] * s;
        Ai[3 * k + 1] = c1[k] * s;
        Ai[3 * k + 2] = c2[k] * s;
    }
}

// ---------------------------------------------------------------------------------------------
// Stable Neo-Hookean energy (physics/StableNeoHookeanEnergy.h:621-1325).
//   Psi(F) = mu/2 (tr(F^T F) - 3) + lambda/2 (det F - 1 - mu/lambda)^2
// F is a column-major 9-vector.  Derivatives are written from the formula:
//   dPsi/dF   = mu F + lambda (J - alpha) cof(F)
//   d2Psi/dF2 = mu I9 + lambda vec(cof F) vec(cof F)^T + lambda (J - alpha) d2J/dF2
// with alpha = 1 + mu/lambda and d2J/dF_a dF_b = -[F_c]x for (a,b,c) a cyclic permutation of
// (0,1,2) (its transpose for the anti-cyclic order, zero on the diagonal blocks).
// ---------------------------------------------------------------------------------------------

inline void cofactor(Real const* F, Real* C)
{
    cross3(F + 3, F + 6, C + 0);
    cross3(F + 6, F + 0, C + 3);
    cross3(F + 0, F + 3, C + 6);
}

Real snh_eval(Real const* F, Real mu, Real lambda)
{
    Real I2 = 0;
    for (int k = 0; k < 9; ++k)
        I2 += F[k] * F[k];
    Real const a = det3(F) - Real(1) - mu / lambda;
    return Real(0.5) * lambda * a * a + Real(0.5) * mu * (I2 - Real(3));
}

void snh_grad(Real const* F, Real mu, Real lambda, Real* g)
{
    Real C[9];
    cofactor(F, C);
    Real const J = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
    Real const s = lambda * (J - Real(1) - mu / lambda);
    for (int k = 0; k < 9; ++k)
        g[k] = mu * F[k] + s * C[k];
}

// Skew matrix [v]x (column-major) scaled by s, added into the 3x3 block (rows r0.., cols c0..)
// of a 9x9 row-major matrix H.
inline void add_skew(Real* H, int r0, int c0, Real const* v, Real s)
{
    // [v]x = [[0, -v2, v1], [v2, 0, -v0], [-v1, v0, 0]]
    Real const S[3][3] = {{0, -v[2], v[1]}, {v[2], 0, -v[0]}, {-v[1], v[0], 0}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            H[(r0 + i) * 9 + (c0 + j)] += s * S[i][j];
}

void snh_grad_hessian(Real const* F, Real mu, Real lambda, Real* g, Real* H)
{
    Real C[9];
    cofactor(F, C);
    Real const J  = F[0] * C[0] + F[1] * C[1] + F[2] * C[2];
    Real const Ja = J - Real(1) - mu / lambda;
    for (int k = 0; k < 9; ++k)
        g[k] = mu * F[k] + lambda * Ja * C[k];
    for (int r = 0; r < 9; ++r)
        for (int c = 0; c < 9; ++c)
            H[r * 9 + c] = lambda * C[r] * C[c] + (r == c ? mu : Real(0));
    Real const s = lambda * Ja;
    // Off-diagonal column blocks of d2J/dF2.
    int const cyc[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    for (auto const& t : cyc)
    {
        int const a = t[0], b = t[1], c = t[2];
        add_skew(H, 3 * a, 3 * b, F + 3 * c, -s); // block(a,b) = -[F_c]x
        add_skew(H, 3 * b, 3 * a, F + 3 * c, s);  // block(b,a) = +[F_c]x
    }
}

} // namespace

#include "orc_accel.h"
#include "orc_problem.h"

extern "C" {

// ---- Lame coefficients (physics/HyperElasticity.cpp:6-11) -----------------------------------
void orc_lame(double E, double nu, double* mu, double* lambda)
{
    *mu     = E / (2. * (1. + nu));
    *lambda = (E * nu) / ((1. + nu) * (1. - 2. * nu));
}

// ---- SNH entry points for tests --------------------------------------------------------------
double orc_snh_eval(double const* F, double mu, double lambda)
{
    return snh_eval(F, mu, lambda);
}
void orc_snh_grad(double const* F, double mu, double lambda, double* g)
{
    snh_grad(F, mu, lambda, g);
}
void orc_snh_grad_hessian(double const* F, double mu, double lambda, double* g, double* H)
{
    snh_grad_hessian(F, mu, lambda, g, H);
}

// ---- Data::Construct precompute (sim/vbd/Data.cpp:179-243) ----------------------------------
//
// Outputs (caller-allocated): m[nV], GP[nT*12], wg[nT], GVGp[nV+1], GVGe[4nT], GVGilocal[4nT],
// colors[nV], Pptr[>= 129], Padj[nV].  Returns 0 on success, 1 on a degenerate/inverted tet,
// 2 on an out-of-range index, 3 when the colour palette (128) overflows.
int orc_construct(
    int32_t nV,
    int32_t nT,
    double const* X,
    int32_t const* T,
    double const* rhoe,
    int32_t const* dbc,
    int32_t nDbc,
    int32_t ordering,
    int32_t selection,
    double* m,
    double* GP,
    double* wg,
    int32_t* GVGp,
    int32_t* GVGe,
    int32_t* GVGilocal,
    int32_t* colors,
    int32_t* Pptr,
    int32_t* nPartitions,
    int32_t* Padj,
    int32_t* nPadj)
{
    for (int64_t k = 0; k < int64_t(nT) * 4; ++k)
        if (T[k] < 0 || T[k] >= nV)
            return 2;
    // Element geometry: fem/ShapeFunctions.h:267-296 (GP = GN J^-1 for the linear tet),
    // fem/MeshQuadrature.h:75-88 (order-1 weight = |det J|/6), fem/Mass.h:357-397 with
    // Data.cpp:210-219 (lumped mass = rho V / 4 per incident tet).
    std::fill(m, m + nV, 0.0);
    for (int32_t e = 0; e < nT; ++e)
    {
        int32_t const* t = T + 4 * e;
        Real J[9];
        for (int d = 0; d < 3; ++d)
            for (int r = 0; r < 3; ++r)
                J[3 * d + r] = X[3 * t[d + 1] + r] - X[3 * t[0] + r];
        Real const detJ = det3(J);
        if (!(detJ > 0))
            return 1;
        Real Ji[9];
        inv3(J, Ji);
        double* G = GP + 12 * e;
        // Row a (a = 1..3) of GP is row a-1 of J^-1; row 0 is minus their sum.
        for (int a = 1; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                G[3 * a + d] = Ji[3 * d + (a - 1)];
        for (int d = 0; d < 3; ++d)
            G[d] = -(G[3 + d] + G[6 + d] + G[9 + d]);
        wg[e]         = std::abs(detJ) / 6.0;
        Real const me = rhoe[e] * wg[e] / 4.0;
        for (int a = 0; a < 4; ++a)
            m[t[a]] += me;
    }
    // Vertex -> tet adjacency, tets ascending per vertex (graph/Mesh.h:42-104 transposed,
    // Data.cpp:223-226).
    std::fill(GVGp, GVGp + nV + 1, 0);
    for (int64_t k = 0; k < int64_t(nT) * 4; ++k)
        ++GVGp[T[k] + 1];
    for (int32_t i = 0; i < nV; ++i)
        GVGp[i + 1] += GVGp[i];
    {
        std::vector<int32_t> fill(GVGp, GVGp + nV);
        for (int32_t e = 0; e < nT; ++e)
            for (int a = 0; a < 4; ++a)
            {
                int32_t const i = T[4 * e + a];
                GVGe[fill[i]]      = e;
                GVGilocal[fill[i]] = a;
                ++fill[i];
            }
    }
    // Primal vertex graph G G^T (graph/Mesh.h:117-123): neighbours incl. self, no duplicates.
    std::vector<int32_t> Gp(nV + 1, 0), Gv;
    {
        std::vector<int32_t> mark(nV, -1), nb;
        Gv.reserve(size_t(nV) * 16);
        for (int32_t i = 0; i < nV; ++i)
        {
            nb.clear();
            for (int32_t k = GVGp[i]; k < GVGp[i + 1]; ++k)
            {
                int32_t const* t = T + 4 * GVGe[k];
                for (int a = 0; a < 4; ++a)
                    if (mark[t[a]] != i)
                    {
                        mark[t[a]] = i;
                        nb.push_back(t[a]);
                    }
            }
            std::sort(nb.begin(), nb.end());
            Gv.insert(Gv.end(), nb.begin(), nb.end());
            Gp[i + 1] = int32_t(Gv.size());
        }
    }
    // Greedy colouring (graph/Color.h:45-135).  Visiting order: stable argsort of degree
    // (common/ArgSort.h:31-39); selection: LeastUsed (least-used usable colour, ties to the lowest
    // index, i.e. std::min_element semantics) or FirstAvailable.
    std::vector<int32_t> order(nV);
    std::iota(order.begin(), order.end(), 0);
    auto degree = [&](int32_t i) { return Gp[i + 1] - Gp[i]; };
    if (ordering == 1) // SmallestDegree
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
            return degree(a) < degree(b);
        });
    else if (ordering == 2) // LargestDegree
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
            return degree(a) > degree(b);
        });
    std::fill(colors, colors + nV, -1);
    int constexpr kPalette = 128;
    std::vector<int32_t> palette;
    std::vector<char> usable;
    for (int32_t u : order)
    {
        std::fill(usable.begin(), usable.end(), 1);
        int nUnusable = 0;
        for (int32_t k = Gp[u]; k < Gp[u + 1]; ++k)
        {
            int32_t const cv = colors[Gv[k]];
            if (cv >= 0 && usable[cv])
            {
                usable[cv] = 0;
                ++nUnusable;
            }
        }
        if (nUnusable == int(palette.size()))
        {
            if (int(palette.size()) == kPalette)
                return 3;
            colors[u] = int32_t(palette.size());
            palette.push_back(1);
            usable.push_back(0);
        }
        else
        {
            int best = 0;
            for (int c = 1; c < int(palette.size()); ++c)
            {
                bool less;
                if (usable[c] && usable[best])
                    less = (selection == 0) ? palette[c] < palette[best] : c < best;
                else
                    less = usable[c];
                if (less)
                    best = c;
            }
            colors[u] = best;
            ++palette[best];
        }
    }
    // Partitions: stable argsort by colour (graph/Adjacency.h:172-181), then drop Dirichlet
    // vertices (Data.cpp:236-243, graph/Adjacency.h:307-342).
    int32_t const nC = nV > 0 ? *std::max_element(colors, colors + nV) + 1 : 0;
    std::vector<char> pinned(nV, 0);
    for (int32_t k = 0; k < nDbc; ++k)
        if (dbc[k] >= 0 && dbc[k] < nV)
            pinned[dbc[k]] = 1;
    Pptr[0] = 0;
    int32_t n = 0;
    for (int32_t c = 0; c < nC; ++c)
    {
        for (int32_t i = 0; i < nV; ++i)
            if (colors[i] == c && !pinned[i])
                Padj[n++] = i;
        Pptr[c + 1] = n;
    }
    *nPartitions = nC;
    *nPadj       = n;
    return 0;
}

// ---- Integrator ---------------------------------------------------------------------------

static void initial_positions(
    Real const* xt,
    Real const* vtm1,
    Real const* vt,
    Real const* a,
    Real dt,
    Real dt2,
    int strategy,
    Real* x)
{
    // sim/vbd/Kernels.h:39-94 (InitialPositionsForSolve).
    if (strategy == 0) // Position
    {
        for (int d = 0; d < 3; ++d)
            x[d] = xt[d];
        return;
    }
    if (strategy == 1) // Inertia
    {
        for (int d = 0; d < 3; ++d)
            x[d] = xt[d] + dt * vt[d];
        return;
    }
    if (strategy == 2) // KineticEnergyMinimum
    {
        for (int d = 0; d < 3; ++d)
            x[d] = xt[d] + dt * vt[d] + dt2 * a[d];
        return;
    }
    Real const an2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    Real at        = 0;
    if (an2 != Real(0))
    {
        if (strategy == 3) // AdaptiveVbd
        {
            Real dot = 0;
            for (int d = 0; d < 3; ++d)
                dot += ((vt[d] - vtm1[d]) / dt) * a[d];
            at = std::min(std::max(dot / an2, Real(0)), Real(1));
        }
        else // AdaptivePbat
        {
            Real const vn =
                std::sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]) +
                std::numeric_limits<Real>::min();
            Real dot = 0;
            for (int d = 0; d < 3; ++d)
                dot += (vt[d] / vn) * a[d];
            at = std::min(std::abs(dot / an2), Real(1));
        }
    }
    for (int d = 0; d < 3; ++d)
        x[d] = xt[d] + dt * vt[d] + dt2 * at * a[d];
}

void orc_initial_positions(
    double const* xt,
    double const* vtm1,
    double const* vt,
    double const* a,
    double dt,
    double dt2,
    int32_t strategy,
    double* x)
{
    initial_positions(xt, vtm1, vt, a, dt, dt2, strategy, x);
}

// Accumulate the elastic gradient and 3x3 Hessian of vertex i (sim/vbd/Integrator.cpp:102-121,
// sim/vbd/Kernels.h:131-171), then damping, inertia and the Newton step (Kernels.h:179-191,
// 310-339).  x is updated in place.  HinvOut (optional): the inverse of the 3x3 Newton matrix,
// zero when the step is skipped.
static void solve_vertex(orc_problem const& P, int32_t i, Real const* xt, Real const* xtilde, Real* x, Real sdt, Real sdt2, Real* HinvOut = nullptr)
{
    Real H[9] = {0}, g[3] = {0};
    for (int32_t n = P.GVGp[i]; n < P.GVGp[i + 1]; ++n)
    {
        int32_t const e    = P.GVGe[n];
        int32_t const il   = P.GVGilocal[n];
        int32_t const* t   = P.T + 4 * e;
        double const* GPe  = P.GP + 12 * e;
        Real F[9]          = {0};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                for (int r = 0; r < 3; ++r)
                    F[3 * d + r] += x[3 * t[a] + r] * GPe[3 * a + d];
        Real gF[9], HF[81];
        snh_grad_hessian(F, P.mu[e], P.lambda[e], gF, HF);
        Real const w = P.wg[e];
        for (int kj = 0; kj < 3; ++kj)
            for (int ki = 0; ki < 3; ++ki)
            {
                Real const s = w * GPe[3 * il + ki] * GPe[3 * il + kj];
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c)
                        H[3 * c + r] += s * HF[(3 * ki + r) * 9 + (3 * kj + c)];
            }
        for (int k = 0; k < 3; ++k)
        {
            Real const s = w * GPe[3 * il + k];
            for (int r = 0; r < 3; ++r)
                g[r] += s * gF[3 * k + r];
        }
    }
    Real* xi        = x + 3 * i;
    Real const* xti = xt + 3 * i;
    // AddDamping (Kernels.h:179-191)
    Real const D = P.kD / sdt;
    for (int r = 0; r < 3; ++r)
    {
        Real hx = 0;
        for (int c = 0; c < 3; ++c)
            hx += H[3 * c + r] * (xi[c] - xti[c]);
        g[r] += D * hx;
    }
    for (int k = 0; k < 9; ++k)
        H[k] *= Real(1) + D;
    // AddInertiaDerivatives (Kernels.h:310-322)
    Real const K = P.m[i] / sdt2;
    for (int r = 0; r < 3; ++r)
    {
        H[3 * r + r] += K;
        g[r] += K * (xi[r] - xtilde[3 * i + r]);
    }
    // IntegratePositions (Kernels.h:329-339)
    if (std::abs(det3(H)) <= P.detHZero)
    {
        if (HinvOut)
            std::fill(HinvOut, HinvOut + 9, Real(0));
        return;
    }
    Real Hi[9];
    inv3(H, Hi);
    if (HinvOut)
        std::copy(Hi, Hi + 9, HinvOut);
    for (int r = 0; r < 3; ++r)
    {
        Real dx = 0;
        for (int c = 0; c < 3; ++c)
            dx += Hi[3 * c + r] * g[c];
        xi[r] -= dx;
    }
}

// Chebyshev weight (sim/vbd/Kernels.h:96-102).  formula 0 keeps the reference's expression as
// written, `4/4 - rho2*omega` (= 1 - rho2*omega); formula 1 is the textbook 4/(4 - rho2*omega).
double orc_chebyshev_omega(int32_t k, double rho2, double omega, int32_t formula)
{
    if (k == 0)
        return 1.0;
    if (k == 1)
        return 2.0 / (2.0 - rho2);
    return formula == 0 ? (4.0 / 4.0 - rho2 * omega) : 4.0 / (4.0 - rho2 * omega);
}

// Least-squares coefficients of min |A alpha - f| for the n x m window A (columns A[j]), from the
// Gram matrix A^T A and A^T f in FP64: (A^T A + eps I) alpha = A^T f by Cholesky, eps = 1e-10 of
// the largest diagonal entry.  Where A is well conditioned this is the reference's complete
// orthogonal decomposition solution (sim/vbd/AndersonIntegrator.cpp:26-27,49-55); directions far
// below eps are damped to zero, as in its minimum-norm solution.
static void anderson_lsq(std::vector<std::vector<Real>> const& A, int m, Real const* f, size_t n, Real* alpha)
{
    Real G[16][16] = {}, b[16] = {};
    for (int i = 0; i < m; ++i)
    {
        for (int j = 0; j <= i; ++j)
        {
            Real d = 0;
            for (size_t q = 0; q < n; ++q)
                d += A[i][q] * A[j][q];
            G[i][j] = G[j][i] = d;
        }
        Real d = 0;
        for (size_t q = 0; q < n; ++q)
            d += A[i][q] * f[q];
        b[i] = d;
    }
    Real dmax = 0;
    for (int i = 0; i < m; ++i)
        dmax = std::max(dmax, G[i][i]);
    Real const eps = 1e-10 * dmax + 1e-300;
    for (int i = 0; i < m; ++i)
        G[i][i] += eps;
    Real L[16][16] = {}, y[16];
    for (int j = 0; j < m; ++j)
    {
        Real d = G[j][j];
        for (int k = 0; k < j; ++k)
            d -= L[j][k] * L[j][k];
        L[j][j] = std::sqrt(std::max(d, eps));
        for (int i = j + 1; i < m; ++i)
        {
            Real v = G[i][j];
            for (int k = 0; k < j; ++k)
                v -= L[i][k] * L[j][k];
            L[i][j] = v / L[j][j];
        }
    }
    for (int i = 0; i < m; ++i)
    {
        Real v = b[i];
        for (int k = 0; k < i; ++k)
            v -= L[i][k] * y[k];
        y[i] = v / L[i][i];
    }
    for (int i = m - 1; i >= 0; --i)
    {
        Real v = y[i];
        for (int k = i + 1; k < m; ++k)
            v -= L[k][i] * alpha[k];
        alpha[i] = v / L[i][i];
    }
}

// Advance `nsteps` time steps in place: x, v (nV x 3), vprev (nV x 3, GPU semantics only: the
// velocity of the previous step, initially zero).  sim/vbd/Integrator.cpp:22-96 and
// ChebyshevIntegrator.cpp:15-32.
double orc_objective(orc_problem const* Pp, double const* x, double const* xtilde, double dt);

// Least-squares conjugate gradient on min |A gamma - b|, A = the first mk of the window columns
// (Eigen's LeastSquaresConjugateGradient with IdentityPreconditioner and a zero initial guess, the
// solver BroydenIntegrator.cpp:67-72 calls; Eigen is pinned by the reference at commit
// 7fd305ecae2410714cde018cb6851f49138568c8 and is not part of its sources).  CGLS: the normal
// residual A^T r drives the directions; stop after maxIters steps or when |A^T r|^2 < tol^2 |A^T b|^2.
static void cgls(std::vector<std::vector<Real>> const& A, int mk, Real const* b, size_t n, int maxIters, Real tol, Real* gamma)
{
    std::vector<Real> r(b, b + n), tmp(n);
    Real nr[16], p[16];
    auto At = [&](Real const* v, Real* out) {
        for (int j = 0; j < mk; ++j)
        {
            Real s = 0;
            for (size_t q = 0; q < n; ++q)
                s += A[size_t(j)][q] * v[q];
            out[j] = s;
        }
    };
    for (int j = 0; j < mk; ++j)
        gamma[j] = 0;
    At(b, nr);
    Real rhsNorm2 = 0;
    for (int j = 0; j < mk; ++j)
        rhsNorm2 += nr[j] * nr[j];
    if (rhsNorm2 == 0)
        return;
    Real const threshold = tol * tol * rhsNorm2;
    Real absNew          = rhsNorm2; // |A^T r|^2 with r = b
    if (absNew < threshold)
        return;
    for (int j = 0; j < mk; ++j)
        p[j] = nr[j];
    for (int it = 0; it < maxIters; ++it)
    {
        Real tn = 0;
        for (size_t q = 0; q < n; ++q)
        {
            Real v = 0;
            for (int j = 0; j < mk; ++j)
                v += A[size_t(j)][q] * p[j];
            tmp[q] = v;
            tn += v * v;
        }
        Real const alpha = absNew / tn;
        for (int j = 0; j < mk; ++j)
            gamma[j] += alpha * p[j];
        for (size_t q = 0; q < n; ++q)
            r[q] -= alpha * tmp[q];
        At(r.data(), nr);
        Real rn2 = 0;
        for (int j = 0; j < mk; ++j)
            rn2 += nr[j] * nr[j];
        if (rn2 < threshold)
            break;
        Real const beta = rn2 / absNew;
        absNew          = rn2;
        for (int j = 0; j < mk; ++j)
            p[j] = nr[j] + beta * p[j];
    }
}

// BroydenIntegrator::Solve (sim/vbd/BroydenIntegrator.cpp:41-80): with VBD(f_k) = x_k - x_{k+1}
// the negated sweep step, after each sweep k >= 1 column (k-1) mod m of X gets x_k - x_{k-1}
// (pre-sweep iterates) and of G the change of VBD(f); gamma = CGLS(G, VBD(f_k)) with at most
// max(1, m - k) iterations and tolerance 1e-10, and x <- x - (X - G) gamma.
static void broyden(orc_problem const& P, Real const* xt, Real const* xtilde, Real* x, Real sdt, Real sdt2, int32_t iterations, int nthreads)
{
    (void)nthreads;
    size_t const n3 = size_t(P.nV) * 3;
    int const m     = P.window;
    std::vector<std::vector<Real>> G(static_cast<size_t>(m), std::vector<Real>(n3));
    std::vector<std::vector<Real>> X(static_cast<size_t>(m), std::vector<Real>(n3));
    std::vector<Real> xkm1(x, x + n3), fk(n3), fkm1(n3);
    auto sweep = [&] {
        for (int32_t p = 0; p < P.nPartitions; ++p)
        {
            int32_t const b = P.Pptr[p], e = P.Pptr[p + 1];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
            for (int32_t kk = b; kk < e; ++kk)
                solve_vertex(P, P.Padj[kk], xt, xtilde, x, sdt, sdt2);
        }
    };
    if (iterations <= 0)
        return;
    sweep();
    for (size_t q = 0; q < n3; ++q)
        fkm1[q] = xkm1[q] - x[q];
    for (int32_t k = 1; k < iterations; ++k)
    {
        int const dkl = (k - 1) % m;
        for (size_t q = 0; q < n3; ++q)
        {
            X[size_t(dkl)][q] = x[q] - xkm1[q];
            xkm1[q]           = x[q];
        }
        sweep();
        for (size_t q = 0; q < n3; ++q)
        {
            fk[q]             = xkm1[q] - x[q];
            G[size_t(dkl)][q] = fk[q] - fkm1[q];
            fkm1[q]           = fk[q];
        }
        int const mk = std::min(m, int(k));
        Real gamma[16];
        cgls(G, mk, fk.data(), n3, std::max(1, m - int(k)), Real(1e-10), gamma);
        for (size_t q = 0; q < n3; ++q)
        {
            Real u = 0;
            for (int j = 0; j < mk; ++j)
                u += (X[size_t(j)][q] - G[size_t(j)][q]) * gamma[j];
            x[q] -= u;
        }
    }
}

// Minimiser of the quadratic model a t^2 + b t + c (TrustRegionIntegrator.cu:400-430), with the
// reference's float thresholds: FLT_MIN as zero and FLT_MAX as infinity.
static Real tr_model_optimal_step(Real const aQ[3])
{
    Real const zero = Real(FLT_MIN), inf = Real(FLT_MAX);
    if (std::abs(aQ[0]) > zero)
        return aQ[0] > zero ? -aQ[1] / (Real(2) * aQ[0]) : inf;
    if (std::abs(aQ[1]) > zero)
        return aQ[1] > 0 ? -inf : inf;
    return Real(0);
}

// std::clamp as min(max(v, lo), hi) (the comparisons decide NaN bounds: a NaN upper bound leaves
// max(v, lo)).
static Real tr_clamp(Real v, Real lo, Real hi)
{
    Real const m = (v < lo) ? lo : v;
    return (hi < m) ? hi : m;
}

} // extern "C"

// TrustRegionIntegrator::SolveWithLinearAcceleratedPath (gpu/impl/vbd/TrustRegionIntegrator.cu:
// 48-165).  The first two iterations are plain VBD sweeps that record f and t; from k = 2 on, a
// quadratic model m(t) through (t_{k-2}, f_{k-2}), (t_{k-1}, f_{k-1}), (t_k = 0, f_k) is built,
// the VBD step x_{k-1} -> x is taken and then stretched to x_{k-1} + t (x - x_{k-1}), t the model's
// minimiser clamped to [1, R / |dx|]; the stretched step is kept when the actual decrease is more
// than eta of the predicted one, else rolled back to the VBD step, with the radius R grown or
// shrunk by tau.
void orc::trust_region_solve(orc_problem const& P, double* x, int32_t nV, int32_t iterations, orc::Sweep const& sweep,
                             orc::Objective const& objective, double const* forced, double* log)
{
    size_t const n3 = size_t(nV) * 3;
    std::vector<Real> xkm1(x, x + n3);
    Real const eta = P.tr_eta, tau = P.tr_tau, zero = 1e-6;
    Real fk = objective(), fkm1 = 0, fkm2 = 0, tk = -1, tkm1 = 0, tkm2 = 0, R2 = 0;
    for (int32_t k = 0; k < iterations; ++k)
    {
        if (k >= 2)
        {
            // ConstructModel: translate so that t_k = 0, then solve Q aQ = f.
            tkm2 -= tk;
            tkm1 -= tk;
            tk = 0;
            Real const Q[9] = {tkm2 * tkm2, tkm1 * tkm1, tk * tk, tkm2, tkm1, tk, 1, 1, 1}; // column-major
            Real Qi[9];
            inv3(Q, Qi);
            Real const fv[3] = {fkm2, fkm1, fk};
            Real aQ[3];
            for (int r = 0; r < 3; ++r)
                aQ[r] = Qi[r] * fv[0] + Qi[3 + r] * fv[1] + Qi[6 + r] * fv[2];
            // UpdateIterates
            fkm2 = fkm1, fkm1 = fk, tkm2 = tkm1, tkm1 = tk;
            std::copy(x, x + n3, xkm1.begin());
            sweep();
            Real dx2 = 0;
            for (size_t q = 0; q < n3; ++q)
                dx2 += (x[q] - xkm1[q]) * (x[q] - xkm1[q]);
            if (R2 < dx2 + zero)
                R2 = tau * tau * dx2;
            Real const lower = 1, upper = std::sqrt(R2 / dx2);
            Real t            = tr_clamp(tr_model_optimal_step(aQ), lower, upper);
            bool tryAcc       = !(std::abs(t - lower) < zero);
            double const* F   = forced ? forced + 4 * size_t(k) : nullptr;
            if (F)
            {
                t      = F[0];
                tryAcc = (int(F[3]) & 1) != 0;
            }
            bool accepted = false;
            Real rhoTR    = std::numeric_limits<Real>::quiet_NaN();
            if (tryAcc)
            {
                for (size_t q = 0; q < n3; ++q)
                    x[q] = xkm1[q] + t * (x[q] - xkm1[q]);
                fk               = objective();
                Real const mNext = aQ[0] * t * t + aQ[1] * t + aQ[2];
                rhoTR            = (fkm1 - fk) / (fkm1 - mNext);
                accepted         = F ? (int(F[3]) & 2) != 0 : rhoTR > eta;
            }
            if (accepted)
            {
                if ((upper - t) < zero)
                    R2 *= tau * tau;
                tk = t;
            }
            else
            {
                R2 /= tau * tau;
                if (tryAcc)
                    for (size_t q = 0; q < n3; ++q)
                        x[q] = xkm1[q] + (x[q] - xkm1[q]) / t;
                fk = objective();
                tk = tkm1 + 1;
            }
            if (log)
            {
                double* L = log + 4 * size_t(k);
                L[0] = t, L[1] = rhoTR, L[2] = R2, L[3] = tryAcc ? (accepted ? 3.0 : 1.0) : 0.0;
            }
        }
        else
        {
            fkm2 = fkm1, fkm1 = fk, tkm2 = tkm1, tkm1 = tk;
            std::copy(x, x + n3, xkm1.begin());
            sweep();
            fk = objective();
            tk = Real(k);
            if (log)
            {
                double* L = log + 4 * size_t(k);
                L[0] = 0.0, L[1] = std::numeric_limits<double>::quiet_NaN(), L[2] = R2, L[3] = 0.0;
            }
        }
    }
}

// AndersonIntegrator::Solve (sim/vbd/AndersonIntegrator.cpp:24-57): after each VBD iteration
// k >= 1, G_k = x, F_k = G_k - x_{k-1}; column (k-1) mod m of the window gets G_k - G_{k-1} and
// F_k - F_{k-1}; x = G_k - DG alpha with alpha = argmin |DF alpha - F_k| over the min(m, k) filled
// columns.
void orc::anderson_solve(orc_problem const& P, double* x, int32_t nV, int32_t iterations, orc::Sweep const& sweep)
{
    size_t const n3 = size_t(nV) * 3;
    int const m     = P.window;
    std::vector<std::vector<Real>> DF(static_cast<size_t>(m), std::vector<Real>(n3));
    std::vector<std::vector<Real>> DG(static_cast<size_t>(m), std::vector<Real>(n3));
    std::vector<Real> xkm1(x, x + n3), Gkm1(n3), Fkm1(n3), Fk(n3);
    if (iterations > 0)
    {
        sweep();
        for (size_t q = 0; q < n3; ++q)
        {
            Gkm1[q] = x[q];
            Fkm1[q] = x[q] - xkm1[q];
        }
    }
    for (int32_t k = 1; k < iterations; ++k)
    {
        std::copy(x, x + n3, xkm1.begin());
        sweep();
        int const dkl = (k - 1) % m;
        for (size_t q = 0; q < n3; ++q)
        {
            Fk[q]      = x[q] - xkm1[q];
            DG[dkl][q] = x[q] - Gkm1[q];
            DF[dkl][q] = Fk[q] - Fkm1[q];
            Gkm1[q]    = x[q];
            Fkm1[q]    = Fk[q];
        }
        int const mk = std::min(m, int(k));
        Real alpha[16];
        anderson_lsq(DF, mk, Fk.data(), n3, alpha);
        for (size_t q = 0; q < n3; ++q)
        {
            Real u = x[q];
            for (int j = 0; j < mk; ++j)
                u -= DG[j][q] * alpha[j];
            x[q] = u;
        }
    }
}

extern "C" {

int orc_run(orc_problem const* Pp, double* x, double* v, double* vprev, double dt, int32_t iterations, int32_t substeps, int32_t nsteps)
{
    orc_problem const& P = *Pp;
    int32_t const nV     = P.nV;
#ifdef _OPENMP
    int const nthreads = P.nthreads > 0 ? P.nthreads : omp_get_max_threads();
#else
    int const nthreads = 1;
#endif
    (void)nthreads;
    std::vector<Real> xt(size_t(nV) * 3), xtilde(size_t(nV) * 3), xkm1, xkm2, vtm1(size_t(nV) * 3);
    if (P.acceleration == 1)
    {
        xkm1.assign(x, x + size_t(nV) * 3);
        xkm2.assign(x, x + size_t(nV) * 3);
    }
    Real const sdt  = dt / Real(substeps);
    Real const sdt2 = sdt * sdt;
    for (int32_t step = 0; step < nsteps; ++step)
        for (int32_t s = 0; s < substeps; ++s)
        {
            // xt <- x, vt <- v; with CPU semantics the previous velocity is lost here
            // (Integrator.cpp:31-32), so InitializeSolve sees vtm1 = vt = v.
            std::memcpy(xt.data(), x, sizeof(Real) * 3 * size_t(nV));
            if (P.semantics == 1)
                std::memcpy(vtm1.data(), vprev, sizeof(Real) * 3 * size_t(nV));
            else
                std::memcpy(vtm1.data(), v, sizeof(Real) * 3 * size_t(nV));
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (int32_t i = 0; i < nV; ++i)
            {
                // InertialTarget (Kernels.h:24-37), InitializeSolve (Integrator.cpp:54-71)
                for (int d = 0; d < 3; ++d)
                    xtilde[3 * i + d] = xt[3 * i + d] + sdt * v[3 * i + d] + sdt2 * P.aext[3 * i + d];
                initial_positions(
                    &xt[3 * size_t(i)],
                    &vtm1[3 * size_t(i)],
                    v + 3 * size_t(i),
                    P.aext + 3 * size_t(i),
                    sdt,
                    sdt2,
                    P.strategy,
                    x + 3 * size_t(i));
            }
            Real const rho2 = P.rho * P.rho;
            Real omega      = 0;
            auto sweepAll = [&] {
                for (int32_t p = 0; p < P.nPartitions; ++p)
                {
                    int32_t const pb = P.Pptr[p], pe = P.Pptr[p + 1];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
                    for (int32_t kk = pb; kk < pe; ++kk)
                        solve_vertex(P, P.Padj[kk], xt.data(), xtilde.data(), x, sdt, sdt2);
                }
            };
            if (P.acceleration == 2)
                orc::anderson_solve(P, x, nV, iterations, sweepAll);
            // NesterovIntegrator::Solve (sim/vbd/NesterovIntegrator.cpp:16-43): x_0 is the solve's
            // start (never updated); for k > start, y = x + beta (x - x_0) before the sweep and
            // x = y - (x - x_0)/L after it, then lambda and beta advance.
            std::vector<Real> neX0, neY;
            Real neLambda = 0, neBeta = 0;
            if (P.acceleration == 3)
            {
                neX0.assign(x, x + size_t(nV) * 3);
                neY.assign(size_t(nV) * 3, 0);
            }
            if (P.acceleration == 4)
                broyden(P, xt.data(), xtilde.data(), x, sdt, sdt2, iterations, nthreads);
            if (P.acceleration == 5 && !P.tr_curved)
            {
                size_t const entry = 4 * (size_t(step) * size_t(substeps) + size_t(s)) * size_t(iterations);
                orc::trust_region_solve(P, x, nV, iterations, sweepAll,
                                        [&] { return orc_objective(&P, x, xtilde.data(), sdt); },
                                        P.tr_forced ? P.tr_forced + entry : nullptr, P.tr_log ? P.tr_log + entry : nullptr);
            }
            // The curved trust-region path (TrustRegionIntegrator.cu:167-263) never moves x off the
            // VBD iterates: its constraint solve returns 0, so t = clamp(t*, FLT_MIN, 0) is at the
            // lower bound, no accelerated step is tried and every iteration is a plain VBD sweep.
            bool const plainLoop = !(P.acceleration == 2 || P.acceleration == 4 || (P.acceleration == 5 && !P.tr_curved));
            for (int32_t k = 0; k < (plainLoop ? iterations : 0); ++k)
            {
                bool const neActive = P.acceleration == 3 && P.nesterov_start < k;
                if (neActive)
                    for (size_t q = 0; q < size_t(nV) * 3; ++q)
                        neY[q] = x[q] + neBeta * (x[q] - neX0[q]);
                // RunVbdIteration (Integrator.cpp:73-87): colours in sequence, vertices of a
                // colour in parallel.
                for (int32_t p = 0; p < P.nPartitions; ++p)
                {
                    int32_t const b = P.Pptr[p], e = P.Pptr[p + 1];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
                    for (int32_t kk = b; kk < e; ++kk)
                        solve_vertex(P, P.Padj[kk], xt.data(), xtilde.data(), x, sdt, sdt2);
                }
                if (neActive)
                {
                    Real const alpha = Real(1) / P.nesterov_L;
                    for (size_t q = 0; q < size_t(nV) * 3; ++q)
                        x[q] = neY[q] - alpha * (x[q] - neX0[q]);
                    Real const lk = neLambda;
                    neLambda      = (1 + std::sqrt(1 + 4 * neLambda * neLambda)) / 2;
                    neBeta        = (lk - 1) / neLambda;
                }
                if (P.acceleration == 1)
                {
                    omega = orc_chebyshev_omega(k, rho2, omega, P.chebyshev_formula);
#pragma omp parallel for num_threads(nthreads) schedule(static)
                    for (int64_t q = 0; q < int64_t(nV) * 3; ++q)
                    {
                        if (k > 1)
                            x[q] = omega * (x[q] - xkm2[q]) + xkm2[q];
                        xkm2[q] = xkm1[q];
                        xkm1[q] = x[q];
                    }
                }
            }
            // IntegrateVelocity (Kernels.h:121-129); GPU UpdateBdfState keeps the old velocity.
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (int64_t q = 0; q < int64_t(nV) * 3; ++q)
            {
                if (vprev)
                    vprev[q] = v[q];
                v[q] = (x[q] - xt[q]) / sdt;
            }
        }
    return 0;
}

// Backward-Euler objective and gradient (sim/vbd/Integrator.cpp:138-200):
//   f(x) = 1/2 (x - xtilde)^T M (x - xtilde) + dt^2 sum_e wg_e Psi(F_e)
double orc_objective(orc_problem const* Pp, double const* x, double const* xtilde, double dt)
{
    orc_problem const& P = *Pp;
    Real Ek              = 0;
    for (int32_t i = 0; i < P.nV; ++i)
        for (int d = 0; d < 3; ++d)
        {
            Real const dx = x[3 * i + d] - xtilde[3 * i + d];
            Ek += 0.5 * P.m[i] * dx * dx;
        }
    Real Ep = 0;
    for (int32_t e = 0; e < P.nT; ++e)
    {
        int32_t const* t  = P.T + 4 * e;
        double const* GPe = P.GP + 12 * e;
        Real F[9]         = {0};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                for (int r = 0; r < 3; ++r)
                    F[3 * d + r] += x[3 * t[a] + r] * GPe[3 * a + d];
        Ep += P.wg[e] * snh_eval(F, P.mu[e], P.lambda[e]);
    }
    return Ek + dt * dt * Ep;
}

void orc_gradient(orc_problem const* Pp, double const* x, double const* xtilde, double dt, double* grad)
{
    orc_problem const& P = *Pp;
    for (int32_t i = 0; i < P.nV; ++i)
        for (int d = 0; d < 3; ++d)
            grad[3 * i + d] = P.m[i] * (x[3 * i + d] - xtilde[3 * i + d]);
    for (int32_t e = 0; e < P.nT; ++e)
    {
        int32_t const* t  = P.T + 4 * e;
        double const* GPe = P.GP + 12 * e;
        Real F[9]         = {0};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                for (int r = 0; r < 3; ++r)
                    F[3 * d + r] += x[3 * t[a] + r] * GPe[3 * a + d];
        Real gF[9];
        snh_grad(F, P.mu[e], P.lambda[e], gF);
        // fem::GradientWrtDofs: dPsi/dx_a = gF (as 3x3, column-major) * GP(a,:)^T
        for (int a = 0; a < 4; ++a)
            for (int r = 0; r < 3; ++r)
            {
                Real s = 0;
                for (int d = 0; d < 3; ++d)
                    s += gF[3 * d + r] * GPe[3 * a + d];
                grad[3 * t[a] + r] += dt * dt * P.wg[e] * s;
            }
    }
}

// One vertex solve on explicit inputs, for comparison with the reference's kernels.
// xe: 3 x 4 column-major positions per incidence (n incidences), GPs: n x 12, il, wg, mu, lambda.
void orc_vertex_solve(
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
    Real H[9] = {0}, g[3] = {0};
    for (int32_t q = 0; q < n; ++q)
    {
        double const* x4  = xe + 12 * q;
        double const* GPe = GPs + 12 * q;
        Real F[9]         = {0};
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d)
                for (int r = 0; r < 3; ++r)
                    F[3 * d + r] += x4[3 * a + r] * GPe[3 * a + d];
        Real gF[9], HF[81];
        snh_grad_hessian(F, mus[q], lambdas[q], gF, HF);
        for (int kj = 0; kj < 3; ++kj)
            for (int ki = 0; ki < 3; ++ki)
            {
                Real const s = wgs[q] * GPe[3 * il[q] + ki] * GPe[3 * il[q] + kj];
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c)
                        H[3 * c + r] += s * HF[(3 * ki + r) * 9 + (3 * kj + c)];
            }
        for (int k = 0; k < 3; ++k)
            for (int r = 0; r < 3; ++r)
                g[r] += wgs[q] * GPe[3 * il[q] + k] * gF[3 * k + r];
    }
    Real const D = kD / sdt;
    Real gd[3];
    for (int r = 0; r < 3; ++r)
    {
        Real hx = 0;
        for (int c = 0; c < 3; ++c)
            hx += H[3 * c + r] * (xi[c] - xti[c]);
        gd[r] = g[r] + D * hx;
    }
    for (int k = 0; k < 9; ++k)
        H[k] *= Real(1) + D;
    Real const K = mi / sdt2;
    for (int r = 0; r < 3; ++r)
    {
        H[3 * r + r] += K;
        gd[r] += K * (xi[r] - xtildei[r]);
    }
    for (int r = 0; r < 3; ++r)
        gout[r] = gd[r];
    for (int k = 0; k < 9; ++k)
        Hout[k] = H[k];
    if (std::abs(det3(H)) <= detHZero)
        return;
    Real Hi[9];
    inv3(H, Hi);
    for (int r = 0; r < 3; ++r)
    {
        Real dx = 0;
        for (int c = 0; c < 3; ++c)
            dx += Hi[3 * c + r] * gd[c];
        xi[r] -= dx;
    }
}

// ---- Adjoint (no reference counterpart) ----------------------------------------------------
//
// Reverse-mode derivative of orc_run for strategies Position, Inertia and KineticEnergyMinimum,
// without acceleration or damping.  Every vertex update x_o' = x_o - H^-1 g (g, H at the state
// before the update) is reversed with w = H^-1 u (u: adjoint of x_o') and the applied step
// delta = x_o - x_o': the adjoints of the inputs are u e_o - grad phi with phi = w.(g - H delta),
// w and delta held fixed.  Per tet, grad_F phi_e = wg [d2Psi:A - lambda ((cof:B) D_A + (cof:A) D_B)]
// with A = w g_o^T, B = delta g_o^T, d2Psi the 9x9 Stable Neo-Hookean Hessian above and
// D_A = d(cof F : A)/dF = J (tr(F^-1 A) F^-T - (F^-1 A F^-1)^T).  Sweeps are reversed colour by
// colour; the state each update saw is rebuilt from the iterates recorded per iteration.
//
// x0, v0: the start state (nV x 3); xbar, vbar (nV x 3): on entry dL/dx, dL/dv of the state after
// nsteps, on return of the start state.  dlogmu, dloglambda (nT): dL/dlog(mu), dL/dlog(lambda)
// added to.  Returns 0, or 2 for unsupported settings.
int orc_adjoint(
    orc_problem const* Pp,
    double const* x0,
    double const* v0,
    double const* vprev0,
    double dt,
    int32_t iterations,
    int32_t substeps,
    int32_t nsteps,
    double* xbar,
    double* vbar,
    double* vprevbar,
    double* dlogmu,
    double* dloglambda)
{
    orc_problem const& P = *Pp;
    if ((P.acceleration != 0 && P.acceleration != 1) || P.strategy < 0 || P.strategy > 4 || substeps < 1 ||
        iterations < 0 || nsteps < 0)
        return 2;
    bool const cheb      = P.acceleration == 1;
    bool const gpuSem    = P.semantics == 1;
    int32_t const nV     = P.nV;
    size_t const n3      = size_t(nV) * 3;
    int32_t const N      = nsteps * substeps;
    Real const h = dt / Real(substeps), h2 = h * h;
    Real const D = P.kD / h;
    int32_t const K = iterations;
    // Chebyshev weights of the iterations (the same recurrence as the forward).
    std::vector<Real> omega(size_t(std::max(K, 1)), 1);
    {
        Real om = 0;
        for (int32_t k = 0; k < K; ++k)
            omega[size_t(k)] = om = orc_chebyshev_omega(k, P.rho * P.rho, om, P.chebyshev_formula);
    }
    // Colour of every vertex (-1: pinned, never solved).
    std::vector<int32_t> colour(size_t(nV), -1);
    for (int32_t p = 0; p < P.nPartitions; ++p)
        for (int32_t kk = P.Pptr[p]; kk < P.Pptr[p + 1]; ++kk)
            colour[P.Padj[kk]] = p;
    // Forward: the state at the start of every substep (positions, velocities, previous velocities).
    std::vector<Real> xs(size_t(N + 1) * n3), vs(size_t(N + 1) * n3), ps(size_t(N + 1) * n3);
    std::copy(x0, x0 + n3, xs.begin());
    std::copy(v0, v0 + n3, vs.begin());
    std::copy(vprev0, vprev0 + n3, ps.begin());
    // Recorded substep: ys[k + 1] = y_k, the iterate after iteration k (ys[0] = the initial guess,
    // y_{-1}); raws[k] = the raw sweep result of iteration k (equal to y_k without Chebyshev).
    std::vector<Real> xt(n3), xtilde(n3), ys(size_t(K + 1) * n3), raws(size_t(std::max(K, 1)) * n3),
        hinv(size_t(K) * size_t(nV) * 9);
    auto substep = [&](int32_t t, bool record) {
        Real const* xa = xs.data() + size_t(t) * n3;
        Real const* va = vs.data() + size_t(t) * n3;
        Real const* pa = ps.data() + size_t(t) * n3;
        std::vector<Real> x(xa, xa + n3), km1(n3), km2(n3);
        std::copy(xa, xa + n3, xt.begin());
        for (int32_t i = 0; i < nV; ++i)
        {
            for (int d = 0; d < 3; ++d)
                xtilde[3 * i + d] = xt[3 * i + d] + h * va[3 * i + d] + h2 * P.aext[3 * i + d];
            Real const* vtm1 = (gpuSem ? pa : va) + 3 * size_t(i);
            initial_positions(&xt[3 * size_t(i)], vtm1, va + 3 * size_t(i), P.aext + 3 * size_t(i), h, h2, P.strategy,
                              &x[3 * size_t(i)]);
        }
        if (record)
            std::copy(x.begin(), x.end(), ys.begin());
        km1 = x;
        km2 = x;
        for (int32_t k = 0; k < K; ++k)
        {
            for (int32_t p = 0; p < P.nPartitions; ++p)
            {
#pragma omp parallel for schedule(dynamic, 64)
                for (int32_t kk = P.Pptr[p]; kk < P.Pptr[p + 1]; ++kk)
                {
                    int32_t const i = P.Padj[kk];
                    solve_vertex(P, i, xt.data(), xtilde.data(), x.data(), h, h2,
                                 record ? &hinv[(size_t(k) * nV + i) * 9] : nullptr);
                }
            }
            if (record)
                std::copy(x.begin(), x.end(), raws.begin() + size_t(k) * n3);
            if (cheb)
                for (size_t q = 0; q < n3; ++q)
                {
                    if (k > 1)
                        x[q] = omega[size_t(k)] * (x[q] - km2[q]) + km2[q];
                    km2[q] = km1[q];
                    km1[q] = x[q];
                }
            if (record)
                std::copy(x.begin(), x.end(), ys.begin() + size_t(k + 1) * n3);
        }
        if (!record)
        {
            Real* xn = xs.data() + size_t(t + 1) * n3;
            Real* vn = vs.data() + size_t(t + 1) * n3;
            Real* pn = ps.data() + size_t(t + 1) * n3;
            for (size_t q = 0; q < n3; ++q)
            {
                xn[q] = x[q];
                vn[q] = (x[q] - xt[q]) / h;
                pn[q] = va[q];
            }
        }
    };
    for (int32_t t = 0; t < N; ++t)
        substep(t, false);
    // Reverse.
    std::vector<Real> ubar(n3), xtbar(n3), xsbar(n3), yp(n3), ypp(n3);
    Real const s1 = P.strategy == 0 ? Real(0) : Real(1);
    for (int32_t t = N - 1; t >= 0; --t)
    {
        substep(t, true);
        Real const* va = vs.data() + size_t(t) * n3;
        Real const* pa = ps.data() + size_t(t) * n3;
        for (size_t q = 0; q < n3; ++q)
        {
            ubar[q]  = xbar[q] + vbar[q] / h;
            xtbar[q] = 0;
            xsbar[q] = 0;
            yp[q]    = 0;
            ypp[q]   = 0;
        }
        for (int32_t k = K - 1; k >= 0; --k)
        {
            // Chebyshev: y_k = omega (raw_k - y_{k-2}) + y_{k-2} for k > 1.  ubar holds the
            // adjoint of y_k once yp (earlier contributions to it) is added; it is split into the
            // raw iterate's adjoint and a contribution to y_{k-2} (ypp, two iterations back).
            if (cheb)
            {
                Real const c1 = k > 1 ? omega[size_t(k)] : Real(1), c2 = k > 1 ? 1 - omega[size_t(k)] : Real(0);
                for (size_t q = 0; q < n3; ++q)
                {
                    Real const yc = yp[q] + ubar[q];
                    ubar[q]       = c1 * yc;
                    yp[q]         = ypp[q];
                    ypp[q]        = c2 * yc;
                }
            }
            Real const* Xk   = raws.data() + size_t(k) * n3; // lower colours: this iteration's results
            Real const* Xkm1 = ys.data() + size_t(k) * n3;   // own and higher colours: y_{k-1}
            for (int32_t p = P.nPartitions - 1; p >= 0; --p)
            {
#pragma omp parallel for schedule(dynamic, 32)
                for (int32_t kk = P.Pptr[p]; kk < P.Pptr[p + 1]; ++kk)
                {
                    int32_t const o = P.Padj[kk];
                    Real const* Hi  = &hinv[(size_t(k) * nV + o) * 9];
                    Real w[3], delta[3];
                    Real const u[3] = {ubar[3 * o], ubar[3 * o + 1], ubar[3 * o + 2]};
                    for (int r = 0; r < 3; ++r)
                    {
                        w[r] = Hi[r] * u[0] + Hi[3 + r] * u[1] + Hi[6 + r] * u[2];
                        // Applied step delta = x_o - x_o' (zero when the step was skipped); with
                        // damping the elastic part of the Newton system sees (1 + D) delta - D (x_o - xt_o).
                        Real const dl = Xkm1[3 * o + r] - Xk[3 * o + r];
                        delta[r]      = (1 + D) * dl - D * (Xkm1[3 * o + r] - xt[3 * o + r]);
                    }
                    if (Hi[0] == 0 && Hi[4] == 0 && Hi[8] == 0)
                        continue; // the Newton step was skipped: x_o' = x_o, nothing else depends on it
                    Real own[3] = {0, 0, 0};
                    for (int32_t n = P.GVGp[o]; n < P.GVGp[o + 1]; ++n)
                    {
                        int32_t const e   = P.GVGe[n];
                        int32_t const il  = P.GVGilocal[n];
                        int32_t const* tv = P.T + 4 * e;
                        double const* GPe = P.GP + 12 * e;
                        Real F[9] = {0};
                        for (int a = 0; a < 4; ++a)
                        {
                            int32_t const va2 = tv[a];
                            Real const* src   = (a == il) ? Xkm1 : (colour[va2] < p ? Xk : Xkm1);
                            for (int d = 0; d < 3; ++d)
                                for (int r = 0; r < 3; ++r)
                                    F[3 * d + r] += src[3 * va2 + r] * GPe[3 * a + d];
                        }
                        Real const mu = P.mu[e], la = P.lambda[e], wg = P.wg[e];
                        Real gF[9], HF[81];
                        snh_grad_hessian(F, mu, la, gF, HF);
                        Real const* go = GPe + 3 * il;
                        Real A[9], B[9];
                        for (int c = 0; c < 3; ++c)
                            for (int r = 0; r < 3; ++r)
                            {
                                A[3 * c + r] = go[c] * w[r];
                                B[3 * c + r] = go[c] * delta[r];
                            }
                        Real C[9];
                        cofactor(F, C);
                        Real const J = det3(F);
                        Real cA = 0, cB = 0, FA = 0;
                        for (int q = 0; q < 9; ++q)
                        {
                            cA += C[q] * A[q];
                            cB += C[q] * B[q];
                            FA += F[q] * A[q];
                        }
                        Real Fi[9];
                        inv3(F, Fi);
                        // D_X = J (tr(F^-1 X) F^-T - (F^-1 X F^-1)^T)
                        auto dJ2 = [&](Real const* Xm, Real* Dm) {
                            Real FX[9] = {0}, FXF[9] = {0};
                            for (int c = 0; c < 3; ++c)
                                for (int r = 0; r < 3; ++r)
                                    for (int q = 0; q < 3; ++q)
                                        FX[3 * c + r] += Fi[3 * q + r] * Xm[3 * c + q];
                            for (int c = 0; c < 3; ++c)
                                for (int r = 0; r < 3; ++r)
                                    for (int q = 0; q < 3; ++q)
                                        FXF[3 * c + r] += FX[3 * q + r] * Fi[3 * c + q];
                            Real const tr = FX[0] + FX[4] + FX[8];
                            for (int c = 0; c < 3; ++c)
                                for (int r = 0; r < 3; ++r)
                                    Dm[3 * c + r] = J * (tr * Fi[3 * r + c] - FXF[3 * r + c]);
                        };
                        Real DA[9], DB[9];
                        dJ2(A, DA);
                        dJ2(B, DB);
                        Real M[9];
                        for (int i9 = 0; i9 < 9; ++i9)
                        {
                            Real HA = 0;
                            for (int j9 = 0; j9 < 9; ++j9)
                                HA += HF[i9 * 9 + j9] * A[j9];
                            M[i9] = wg * (HA - la * (cB * DA[i9] + cA * DB[i9]));
                        }
                        Real wd = 0, gg = 0;
                        for (int r = 0; r < 3; ++r)
                        {
                            wd += w[r] * delta[r];
                            gg += go[r] * go[r];
                        }
                        dlogmu[e] -= wg * mu * (FA - cA - gg * wd);
                        dloglambda[e] -= wg * la * ((J - 1) * cA - cA * cB);
                        for (int a = 0; a < 4; ++a)
                        {
                            Real gphi[3];
                            for (int r = 0; r < 3; ++r)
                                gphi[r] = M[r] * GPe[3 * a] + M[3 + r] * GPe[3 * a + 1] + M[6 + r] * GPe[3 * a + 2];
                            if (a == il)
                            {
                                for (int r = 0; r < 3; ++r)
                                    own[r] += gphi[r];
                                continue;
                            }
                            int32_t const va2 = tv[a];
                            for (int r = 0; r < 3; ++r)
                            {
#pragma omp atomic
                                ubar[3 * va2 + r] -= gphi[r];
                            }
                        }
                    }
                    // Inertia K w (K = m/h^2); damping D H_e w with H_e w = (u - K w) / (1 + D)
                    // (H w = u for the full Newton matrix (1 + D) H_e + K I).
                    Real const Km = P.m[o] / h2;
                    for (int r = 0; r < 3; ++r)
                    {
                        Real const dHw = D * (u[r] - Km * w[r]) / (1 + D);
                        ubar[3 * o + r] -= Km * w[r] + dHw + own[r];
                        xtbar[3 * o + r] += Km * w[r];
                        xsbar[3 * o + r] += dHw;
                    }
                }
            }
        }
        if (cheb)
            for (size_t q = 0; q < n3; ++q)
                ubar[q] += yp[q];
        // The initial guess x0 = xt + s1 h v + h^2 a_t(v, vtm1) a and xtilde = xt + h v + h^2 a;
        // v_end = (x_end - xt) / h; with GPU semantics the substep also passes v on as the next
        // vtm1 (vprev_end = v).
        for (int32_t i = 0; i < nV; ++i)
        {
            Real const* vv = va + 3 * size_t(i);
            Real const* a  = P.aext + 3 * size_t(i);
            Real const* vm = (gpuSem ? pa : va) + 3 * size_t(i);
            Real const an2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
            Real dAv[3] = {0, 0, 0}, dAvm[3] = {0, 0, 0}; // d a_t / d v, d a_t / d vtm1
            if (an2 != 0 && P.strategy == 3 && gpuSem)
            {
                Real dd = 0;
                for (int d = 0; d < 3; ++d)
                    dd += ((vv[d] - vm[d]) / h) * a[d];
                Real const s = dd / an2;
                if (s > 0 && s < 1)
                    for (int d = 0; d < 3; ++d)
                    {
                        dAv[d]  = a[d] / (h * an2);
                        dAvm[d] = -a[d] / (h * an2);
                    }
            }
            else if (an2 != 0 && P.strategy == 4)
            {
                Real const nv = std::sqrt(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
                Real const vn = nv + std::numeric_limits<Real>::min();
                Real va2 = 0;
                for (int d = 0; d < 3; ++d)
                    va2 += vv[d] * a[d];
                Real const s = va2 / (vn * an2);
                if (nv > 0 && std::abs(s) < 1)
                {
                    Real const sg = s > 0 ? Real(1) : (s < 0 ? Real(-1) : Real(0));
                    for (int d = 0; d < 3; ++d)
                        dAv[d] = sg * (a[d] / vn - va2 * vv[d] / (vn * vn * nv)) / an2;
                }
            }
            Real au = 0;
            for (int d = 0; d < 3; ++d)
                au += a[d] * ubar[3 * size_t(i) + d];
            for (int d = 0; d < 3; ++d)
            {
                size_t const q = 3 * size_t(i) + d;
                Real const vb  = vbar[q];
                Real const pb  = vprevbar[q];
                xbar[q]        = -vb / h + ubar[q] + xtbar[q] + xsbar[q];
                vbar[q]        = s1 * h * ubar[q] + h * xtbar[q] + h2 * au * dAv[d] + (gpuSem ? pb : Real(0));
                vprevbar[q]    = h2 * au * dAvm[d];
            }
        }
    }
    return 0;
}

int32_t orc_num_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
