// Per-vertex VBD arithmetic shared by the CUDA kernels and the host-side self-check entry point.
//
// The reference evaluates, for every incident tetrahedron of vertex i, the full 9x9 Stable
// Neo-Hookean Hessian (physics/StableNeoHookeanEnergy.h:1168-1325) and contracts it with the
// shape-function-gradient row w = GP(ilocal, :) (sim/vbd/Kernels.h:131-171).  With
//   Psi(F) = mu/2 (|F|^2 - 3) + lambda/2 (det F - alpha)^2,  alpha = 1 + mu/lambda,
// that contraction has a closed form:
//   g_i += wg (mu F w + lambda (J - alpha) cof(F) w)
//   H_i += wg (mu |w|^2 I + lambda c c^T),   c = cof(F) w
// because the lambda (J - alpha) d2J/dF2 term is antisymmetric in the column pair (a, b) of F
// while w_a w_b is symmetric, so it contracts to zero.  The host self-check (pbgb_debug_vertex_block)
// lets the tests compare this against the oracle's full 9x9 contraction.
#pragma once

#if defined(__CUDACC__)
#define PBGB_HD __host__ __device__ __forceinline__
#else
#define PBGB_HD inline
#endif

#include <cmath>

namespace pbgb {

// Accumulated elastic derivatives of one vertex: gradient g, the scalar s = sum mu' |w|^2 and the
// symmetric matrix C = sum lambda' c c^T stored as (xx, xy, xz, yy, yz, zz).
template <class T>
struct VertexBlock
{
    T g[3];
    T s;
    T C[6];
};

template <class T>
PBGB_HD void zero(VertexBlock<T>& b)
{
    b.g[0] = b.g[1] = b.g[2] = T(0);
    b.s                      = T(0);
    for (int k = 0; k < 6; ++k)
        b.C[k] = T(0);
}

// Shape-function gradients of the three corners a_0, a_1, a_2 of a linear tet other than the
// solved corner o, from the rest edge vectors e[k] = X_{a_k} - X_o: they are the rows of
// [e0 e1 e2]^-1 (the reference solves the same system by LU, fem/ShapeFunctions.h:267-296), and
// grad N_o = -(G0 + G1 + G2).
template <class T>
PBGB_HD void rest_gradients(T const (&e)[3][3], T (&G)[3][3])
{
    G[0][0] = e[1][1] * e[2][2] - e[1][2] * e[2][1];
    G[0][1] = e[1][2] * e[2][0] - e[1][0] * e[2][2];
    G[0][2] = e[1][0] * e[2][1] - e[1][1] * e[2][0];
    G[1][0] = e[2][1] * e[0][2] - e[2][2] * e[0][1];
    G[1][1] = e[2][2] * e[0][0] - e[2][0] * e[0][2];
    G[1][2] = e[2][0] * e[0][1] - e[2][1] * e[0][0];
    G[2][0] = e[0][1] * e[1][2] - e[0][2] * e[1][1];
    G[2][1] = e[0][2] * e[1][0] - e[0][0] * e[1][2];
    G[2][2] = e[0][0] * e[1][1] - e[0][1] * e[1][0];
    T const inv = T(1) / (e[0][0] * G[0][0] + e[0][1] * G[0][1] + e[0][2] * G[0][2]);
    for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c)
            G[k][c] *= inv;
}

// Adds one tetrahedron's contribution to its solved corner o.
//   d[k] = x_{a_k} - x_o and G[k] = grad N_{a_k} for the three other corners (any order);
//   muw, law: wg*mu and wg*lambda; alpha = 1 + mu/lambda.
// F = sum_a x_a grad N_a^T = sum_k d[k] G[k]^T because the gradients sum to zero.
template <class T>
PBGB_HD void accumulate_tet(VertexBlock<T>& b, T const (&d)[3][3], T const (&G)[3][3], T muw, T law, T alpha)
{
    T f[3][3]; // f[c][r] = F(r, c)
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            f[c][r] = d[0][r] * G[0][c] + d[1][r] * G[1][c] + d[2][r] * G[2][c];
    T w[3];
    for (int c = 0; c < 3; ++c)
        w[c] = -(G[0][c] + G[1][c] + G[2][c]);
    // Cofactor columns k0 = f1 x f2, k1 = f2 x f0, k2 = f0 x f1;  J = f0 . k0.
    T k[3][3];
    k[0][0] = f[1][1] * f[2][2] - f[1][2] * f[2][1];
    k[0][1] = f[1][2] * f[2][0] - f[1][0] * f[2][2];
    k[0][2] = f[1][0] * f[2][1] - f[1][1] * f[2][0];
    k[1][0] = f[2][1] * f[0][2] - f[2][2] * f[0][1];
    k[1][1] = f[2][2] * f[0][0] - f[2][0] * f[0][2];
    k[1][2] = f[2][0] * f[0][1] - f[2][1] * f[0][0];
    k[2][0] = f[0][1] * f[1][2] - f[0][2] * f[1][1];
    k[2][1] = f[0][2] * f[1][0] - f[0][0] * f[1][2];
    k[2][2] = f[0][0] * f[1][1] - f[0][1] * f[1][0];
    T const J = f[0][0] * k[0][0] + f[0][1] * k[0][1] + f[0][2] * k[0][2];
    T c[3], Fw[3];
    for (int r = 0; r < 3; ++r)
    {
        c[r]  = w[0] * k[0][r] + w[1] * k[1][r] + w[2] * k[2][r];
        Fw[r] = w[0] * f[0][r] + w[1] * f[1][r] + w[2] * f[2][r];
    }
    T const sl = law * (J - alpha);
    for (int r = 0; r < 3; ++r)
        b.g[r] += muw * Fw[r] + sl * c[r];
    b.s += muw * (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    b.C[0] += law * c[0] * c[0];
    b.C[1] += law * c[0] * c[1];
    b.C[2] += law * c[0] * c[2];
    b.C[3] += law * c[1] * c[1];
    b.C[4] += law * c[1] * c[2];
    b.C[5] += law * c[2] * c[2];
}

// Finishes the vertex: Rayleigh damping (sim/vbd/Kernels.h:179-191), inertia (:310-322) and the
// 3x3 Newton step with the near-singular skip (:329-339).  Updates x in place; returns false when
// the step was skipped.
template <class T>
PBGB_HD bool newton_update(
    VertexBlock<T> const& b,
    T const* xt,
    T const* xtilde,
    T m,
    T h,
    T h2,
    T kD,
    T detHZero,
    T* x,
    T* gout = nullptr,
    T* Hout = nullptr)
{
    // H = s I + C (symmetric; xx xy xz yy yz zz)
    T H[6] = {b.C[0] + b.s, b.C[1], b.C[2], b.C[3] + b.s, b.C[4], b.C[5] + b.s};
    T g[3] = {b.g[0], b.g[1], b.g[2]};
    if (kD != T(0))
    {
        T const D  = kD / h;
        T const e0 = x[0] - xt[0], e1 = x[1] - xt[1], e2 = x[2] - xt[2];
        g[0] += D * (H[0] * e0 + H[1] * e1 + H[2] * e2);
        g[1] += D * (H[1] * e0 + H[3] * e1 + H[4] * e2);
        g[2] += D * (H[2] * e0 + H[4] * e1 + H[5] * e2);
        T const s = T(1) + D;
        for (int q = 0; q < 6; ++q)
            H[q] *= s;
    }
    T const K = m / h2;
    H[0] += K;
    H[3] += K;
    H[5] += K;
    g[0] += K * (x[0] - xtilde[0]);
    g[1] += K * (x[1] - xtilde[1]);
    g[2] += K * (x[2] - xtilde[2]);
    if (gout)
        for (int r = 0; r < 3; ++r)
            gout[r] = g[r];
    if (Hout)
    {
        Hout[0] = H[0], Hout[1] = H[1], Hout[2] = H[2];
        Hout[3] = H[1], Hout[4] = H[3], Hout[5] = H[4];
        Hout[6] = H[2], Hout[7] = H[4], Hout[8] = H[5];
    }
    // Adjugate of the symmetric H.
    T const a00 = H[3] * H[5] - H[4] * H[4];
    T const a01 = H[2] * H[4] - H[1] * H[5];
    T const a02 = H[1] * H[4] - H[2] * H[3];
    T const a11 = H[0] * H[5] - H[2] * H[2];
    T const a12 = H[1] * H[2] - H[0] * H[4];
    T const a22 = H[0] * H[3] - H[1] * H[1];
    T const det = H[0] * a00 + H[1] * a01 + H[2] * a02;
    if (!(fabs(det) > detHZero))
        return false;
    T const inv = T(1) / det;
    x[0] -= inv * (a00 * g[0] + a01 * g[1] + a02 * g[2]);
    x[1] -= inv * (a01 * g[0] + a11 * g[1] + a12 * g[2]);
    x[2] -= inv * (a02 * g[0] + a12 * g[1] + a22 * g[2]);
    return true;
}

// Initial guess of the block-coordinate solve (sim/vbd/Kernels.h:39-94).  `tiny` is the smallest
// normal number of T (the reference adds std::numeric_limits<T>::min() to |v|).
template <class T>
PBGB_HD void initial_position(
    T const* xt,
    T const* vtm1,
    T const* vt,
    T const* a,
    T dt,
    T dt2,
    int strategy,
    T tiny,
    T* x)
{
    T at = T(1);
    if (strategy == 0)
        at = T(0), dt = T(0);
    else if (strategy == 1)
        at = T(0);
    else if (strategy >= 3)
    {
        T const an2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        at          = T(0);
        if (an2 != T(0))
        {
            if (strategy == 3)
            {
                T const dot = ((vt[0] - vtm1[0]) / dt) * a[0] + ((vt[1] - vtm1[1]) / dt) * a[1] +
                              ((vt[2] - vtm1[2]) / dt) * a[2];
                T const q = dot / an2;
                at        = q < T(0) ? T(0) : (q > T(1) ? T(1) : q);
            }
            else
            {
                T const vn  = sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]) + tiny;
                T const dot = (vt[0] / vn) * a[0] + (vt[1] / vn) * a[1] + (vt[2] / vn) * a[2];
                T const q   = fabs(dot / an2);
                at          = q > T(1) ? T(1) : q;
            }
        }
    }
    for (int r = 0; r < 3; ++r)
        x[r] = xt[r] + dt * vt[r] + dt2 * at * a[r];
}

// Chebyshev weight (sim/vbd/Kernels.h:96-102).  formula 0 reproduces the reference's expression
// as written, `4/4 - rho2*omega`; formula 1 is the textbook recurrence 4/(4 - rho2*omega).
template <class T>
PBGB_HD T chebyshev_omega(int k, T rho2, T omega, int formula)
{
    if (k == 0)
        return T(1);
    if (k == 1)
        return T(2) / (T(2) - rho2);
    return formula == 0 ? T(1) - rho2 * omega : T(4) / (T(4) - rho2 * omega);
}

} // namespace pbgb
