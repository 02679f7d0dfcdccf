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

// Rest-state constants of one tetrahedron for the vertex solves of its four corners, so that an
// incidence needs only the current positions (the sweep's form of the closed-form block above).
// With G_a = grad N_a (rows of the reference's GP), for corner o and its other corners a_m =
// (o + 1 + m) & 3 and d_m = x_{a_m} - x_o:
//   F w      = sum_m (G_{a_m} . w) d_m,                 w = G_o,
//   cof(F) w = dJ/dx_o = -gamma_o n,  J = gamma_o (d_0 . n),  n = (d_1 - d_0) x (d_2 - d_0),
// where gamma_o = 1 / det[X_{a_0} - X_o, X_{a_1} - X_o, X_{a_2} - X_o] = (-1)^o gamma_0 (a cyclic
// shift of the four corners is an odd permutation) and gamma_0 = det[G_1; G_2; G_3].  So with
// p = sigma n, sigma = sqrt(lambda') |gamma_0| and kappa_o = (-1)^o alpha sqrt(lambda') sign(gamma_0)
// (lambda' = wg lambda, mu' = wg mu, alpha = 1 + mu/lambda):
//   g_o += sum_m b_{o a_m} d_m + (kappa_o - d_0 . p) p,   C_o += p p^T,   s_o += -sum_m b_{o a_m}
// with b_ab = mu' G_a . G_b (mu' |w|^2 = -sum_m b_{o a_m} because the G_a sum to zero).  The record
// holds b01 b02 b03 b12 b13 b23, sigma, kappa_0: 32 bytes, shared by the four corners.
struct TetStiffness
{
    float b[6];
    float sigma;
    float kappa;
};

// The record's eight words in FP64 (b01 b02 b03 b12 b13 b23 sigma kappa_0) from a tet's
// shape-function gradients G4 (row-major 4 x 3, row a = grad N_a), quadrature weight and Lame
// coefficients.
PBGB_HD void tet_stiffness_words(double const* G4, double wg, double mu, double lambda, double (&w)[8])
{
    auto dot = [&](int a, int c) {
        return G4[3 * a] * G4[3 * c] + G4[3 * a + 1] * G4[3 * c + 1] + G4[3 * a + 2] * G4[3 * c + 2];
    };
    double const* g1 = G4 + 3;
    double const* g2 = G4 + 6;
    double const* g3 = G4 + 9;
    double const gamma0 = g1[0] * (g2[1] * g3[2] - g2[2] * g3[1]) - g1[1] * (g2[0] * g3[2] - g2[2] * g3[0]) +
                          g1[2] * (g2[0] * g3[1] - g2[1] * g3[0]);
    double const mup = wg * mu, lap = wg * lambda, alpha = 1.0 + mu / lambda;
    double const rl  = sqrt(lap);
    w[0] = mup * dot(0, 1);
    w[1] = mup * dot(0, 2);
    w[2] = mup * dot(0, 3);
    w[3] = mup * dot(1, 2);
    w[4] = mup * dot(1, 3);
    w[5] = mup * dot(2, 3);
    w[6] = rl * fabs(gamma0);
    w[7] = gamma0 < 0.0 ? -alpha * rl : alpha * rl;
}

// The FP32 record (each word rounded once).
PBGB_HD TetStiffness tet_stiffness(double const* G4, double wg, double mu, double lambda)
{
    double w[8];
    tet_stiffness_words(G4, wg, mu, lambda, w);
    TetStiffness r{};
    for (int k = 0; k < 6; ++k)
        r.b[k] = float(w[k]);
    r.sigma = float(w[6]);
    r.kappa = float(w[7]);
    return r;
}

// The three b_{o a_m} of corner o (m = 0, 1, 2) and kappa_o, from the record's words.
template <class T>
PBGB_HD void corner_stiffness(T const (&b)[6], T kappa0, int o, T& b0, T& b1, T& b2, T& kappa)
{
    // o = 0: (01, 02, 03); o = 1: (12, 13, 01); o = 2: (23, 02, 12); o = 3: (03, 13, 23).
    b0    = o == 0 ? b[0] : (o == 1 ? b[3] : (o == 2 ? b[5] : b[2]));
    b1    = o == 0 ? b[1] : (o == 1 ? b[4] : (o == 2 ? b[1] : b[4]));
    b2    = o == 0 ? b[2] : (o == 1 ? b[0] : (o == 2 ? b[3] : b[5]));
    kappa = (o & 1) ? -kappa0 : kappa0;
}

// Adds one incidence to the vertex block (the sweep's arithmetic; see TetStiffness).
//   d[m] = x_{a_m} - x_o in the corner order (o + 1 + m) & 3.
template <class T>
PBGB_HD void accumulate_incidence(VertexBlock<T>& b, T const (&d)[3][3], T b0, T b1, T b2, T sigma, T kappa)
{
    T u[3], v[3];
    for (int r = 0; r < 3; ++r)
    {
        u[r] = d[1][r] - d[0][r];
        v[r] = d[2][r] - d[0][r];
    }
    T const p[3] = {sigma * (u[1] * v[2] - u[2] * v[1]), sigma * (u[2] * v[0] - u[0] * v[2]),
                    sigma * (u[0] * v[1] - u[1] * v[0])};
    T const coef = kappa - (d[0][0] * p[0] + d[0][1] * p[1] + d[0][2] * p[2]);
    for (int r = 0; r < 3; ++r)
        b.g[r] += b0 * d[0][r] + b1 * d[1][r] + b2 * d[2][r] + coef * p[r];
    b.s -= b0 + b1 + b2;
    b.C[0] += p[0] * p[0];
    b.C[1] += p[0] * p[1];
    b.C[2] += p[0] * p[2];
    b.C[3] += p[1] * p[1];
    b.C[4] += p[1] * p[2];
    b.C[5] += p[2] * p[2];
}

// Elastic block with Rayleigh damping (sim/vbd/Kernels.h:179-191): H = s I + C, g from the
// accumulated block; damping adds (kD/h) H (x - xt) to g and scales H by 1 + kD/h.
// H is symmetric (xx xy xz yy yz zz).
template <class T>
PBGB_HD void elastic_system(VertexBlock<T> const& b, T const* xt, T const* x, T h, T kD, T* H, T* g)
{
    H[0] = b.C[0] + b.s, H[1] = b.C[1], H[2] = b.C[2];
    H[3] = b.C[3] + b.s, H[4] = b.C[4], H[5] = b.C[5] + b.s;
    g[0] = b.g[0], g[1] = b.g[1], g[2] = b.g[2];
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
}

// Inertia (sim/vbd/Kernels.h:310-322) and the 3x3 Newton step with the near-singular skip
// (:329-339).  Updates x in place; returns false when the step was skipped.  dxOut (optional): the
// applied increment -H^-1 g (zero when skipped).
template <class T>
PBGB_HD bool inertia_solve(
    T* H,
    T* g,
    T const* xtilde,
    T m,
    T h2,
    T detHZero,
    T* x,
    T* gout  = nullptr,
    T* Hout  = nullptr,
    T* dxOut = nullptr)
{
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
    {
        if (dxOut)
            dxOut[0] = dxOut[1] = dxOut[2] = T(0);
        return false;
    }
    T const inv = T(1) / det;
    T const d0  = inv * (a00 * g[0] + a01 * g[1] + a02 * g[2]);
    T const d1  = inv * (a01 * g[0] + a11 * g[1] + a12 * g[2]);
    T const d2  = inv * (a02 * g[0] + a12 * g[1] + a22 * g[2]);
    x[0] -= d0;
    x[1] -= d1;
    x[2] -= d2;
    if (dxOut)
    {
        dxOut[0] = -d0;
        dxOut[1] = -d1;
        dxOut[2] = -d2;
    }
    return true;
}

// Finishes a vertex without contact: damping, inertia and the Newton step.
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
    T H[6], g[3];
    elastic_system(b, xt, x, h, kD, H, g);
    return inertia_solve(H, g, xtilde, m, h2, detHZero, x, gout, Hout);
}

// Vertex-triangle contact (sim/vbd/Kernels.h:215-302 of the reference): penalty 1/2 muC d^2 on the
// signed distance d = min(0, (xv - xb) . n) to the triangle's plane when xv projects inside the
// triangle, plus IPC's smoothed friction (epsv * dt) in the tangent basis (xf1 - xf0, n x (xf1 -
// xf0)).  The basis vectors are not normalised, as in the reference.  Adds to g and H
// (symmetric, xx xy xz yy yz zz); returns the energy.
//   xtv, xv: vertex at t and now; xtf, xf: triangle corners at t and now (3 x 3, corner-major).
template <class T>
PBGB_HD T vertex_triangle_contact(
    T const* xtv,
    T const* xv,
    T const (&xtf)[3][3],
    T const (&xf)[3][3],
    T dt,
    T muC,
    T muF,
    T epsv,
    T epsilon,
    T* g,
    T* H)
{
    T e0[3], e1[3], n[3];
    for (int r = 0; r < 3; ++r)
    {
        e0[r] = xf[1][r] - xf[0][r];
        e1[r] = xf[2][r] - xf[0][r];
    }
    n[0]            = e0[1] * e1[2] - e0[2] * e1[1];
    n[1]            = e0[2] * e1[0] - e0[0] * e1[2];
    n[2]            = e0[0] * e1[1] - e0[1] * e1[0];
    T const dblArea = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (dblArea <= T(1e-8))
        return T(0);
    for (int r = 0; r < 3; ++r)
        n[r] /= dblArea;
    // Projection of xv on the triangle's plane, and its barycentric coordinates.
    T const t = n[0] * (xv[0] - xf[0][0]) + n[1] * (xv[1] - xf[0][1]) + n[2] * (xv[2] - xf[0][2]);
    T ap[3];
    for (int r = 0; r < 3; ++r)
        ap[r] = (xv[r] - t * n[r]) - xf[0][r];
    T const d00   = e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2];
    T const d01   = e0[0] * e1[0] + e0[1] * e1[1] + e0[2] * e1[2];
    T const d11   = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    T const d20   = ap[0] * e0[0] + ap[1] * e0[1] + ap[2] * e0[2];
    T const d21   = ap[0] * e1[0] + ap[1] * e1[1] + ap[2] * e1[2];
    T const denom = d00 * d11 - d01 * d01;
    T const bv    = (d11 * d20 - d01 * d21) / denom;
    T const bw    = (d00 * d21 - d01 * d20) / denom;
    T const bu    = T(1) - bv - bw;
    bool const inside = bu >= T(0) && bu <= T(1) && bv >= T(0) && bv <= T(1) && bw >= T(0) && bw <= T(1);
    if (!inside)
        return T(0);
    T xb[3], xtb[3];
    for (int r = 0; r < 3; ++r)
    {
        xb[r]  = xf[0][r] * bu + xf[1][r] * bv + xf[2][r] * bw;
        xtb[r] = xtf[0][r] * bu + xtf[1][r] * bv + xtf[2][r] * bw;
    }
    T dn = (xv[0] - xb[0]) * n[0] + (xv[1] - xb[1]) * n[1] + (xv[2] - xb[2]) * n[2];
    T const d      = dn < T(0) ? dn : T(0);
    T const lambda = muC * d;
    T E            = T(0.5) * lambda * d;
    for (int r = 0; r < 3; ++r)
        g[r] += lambda * n[r];
    H[0] += muC * n[0] * n[0];
    H[1] += muC * n[0] * n[1];
    H[2] += muC * n[0] * n[2];
    H[3] += muC * n[1] * n[1];
    H[4] += muC * n[1] * n[2];
    H[5] += muC * n[2] * n[2];
    // Friction in the (e0, n x e0) basis on the relative tangential displacement.
    T b1[3];
    b1[0] = n[1] * e0[2] - n[2] * e0[1];
    b1[1] = n[2] * e0[0] - n[0] * e0[2];
    b1[2] = n[0] * e0[1] - n[1] * e0[0];
    T dx[3];
    for (int r = 0; r < 3; ++r)
        dx[r] = (xv[r] - xtv[r]) - (xb[r] - xtb[r]);
    T const u0      = e0[0] * dx[0] + e0[1] * dx[1] + e0[2] * dx[2];
    T const u1      = b1[0] * dx[0] + b1[1] * dx[1] + b1[2] * dx[2];
    T const unorm   = sqrt(u0 * u0 + u1 * u1) + epsilon;
    T const epsvh   = epsv * dt;
    T const muFlam  = muF * fabs(lambda);
    T const y       = unorm / epsvh;
    T const f1      = y < T(1) ? T(2) * y - y * y : T(1);
    T const s       = muFlam * f1 / unorm;
    for (int r = 0; r < 3; ++r)
        g[r] += s * (e0[r] * u0 + b1[r] * u1);
    H[0] += s * (e0[0] * e0[0] + b1[0] * b1[0]);
    H[1] += s * (e0[0] * e0[1] + b1[0] * b1[1]);
    H[2] += s * (e0[0] * e0[2] + b1[0] * b1[2]);
    H[3] += s * (e0[1] * e0[1] + b1[1] * b1[1]);
    H[4] += s * (e0[1] * e0[2] + b1[1] * b1[2]);
    H[5] += s * (e0[2] * e0[2] + b1[2] * b1[2]);
    T const un2 = unorm * unorm;
    E += muFlam * (T(1) / T(3) * epsvh + un2 / epsvh - un2 * unorm / (T(3) * epsvh * epsvh));
    return E;
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

// Derivatives of initial_position's acceleration factor a_t (x0 = xt + dt vt + dt^2 a_t a) with
// respect to vt and vtm1 on the branch the forward took: AdaptiveVbd's clamp((vt - vtm1)/dt . a /
// |a|^2, 0, 1) inside (0, 1), AdaptivePbat's min(|vt . a| / (|vt| |a|^2), 1) below 1 and away from
// vt = 0 (where the factor jumps and has no derivative).  Zero otherwise (constant factors, clamped
// branches).
template <class T>
PBGB_HD void initial_position_factor_derivatives(
    T const* vtm1, T const* vt, T const* a, T dt, int strategy, T tiny, T* dAv, T* dAvm)
{
    for (int r = 0; r < 3; ++r)
        dAv[r] = dAvm[r] = T(0);
    T const an2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    if (an2 == T(0))
        return;
    if (strategy == 3)
    {
        T const dot = ((vt[0] - vtm1[0]) / dt) * a[0] + ((vt[1] - vtm1[1]) / dt) * a[1] +
                      ((vt[2] - vtm1[2]) / dt) * a[2];
        T const q = dot / an2;
        if (q > T(0) && q < T(1))
            for (int r = 0; r < 3; ++r)
            {
                dAv[r]  = a[r] / (dt * an2);
                dAvm[r] = -a[r] / (dt * an2);
            }
    }
    else if (strategy == 4)
    {
        T const nv  = sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
        T const vn  = nv + tiny;
        T const va  = vt[0] * a[0] + vt[1] * a[1] + vt[2] * a[2];
        T const q   = va / (vn * an2);
        if (nv > T(0) && fabs(q) < T(1))
        {
            T const sg = q > T(0) ? T(1) : (q < T(0) ? T(-1) : T(0));
            for (int r = 0; r < 3; ++r)
                dAv[r] = sg * (a[r] / vn - va * vt[r] / (vn * vn * nv)) / an2;
        }
    }
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

// Reverse of one vertex's Newton update, restricted to one incident tetrahedron.
//
// The forward update of vertex o is x_o' = x_o - H^-1 g with g, H the vertex's gradient and 3x3
// block at the state before the update.  With w = H^-1 u (u: adjoint of x_o') and the applied step
// delta = x_o - x_o', the adjoint of every input of the update is minus the gradient of
//   phi = w . (g - H delta)        (w and delta held fixed),
// plus u itself for x_o.  One tetrahedron contributes
//   phi_e = wg [P(F):A - mu |g_o|^2 (w.delta) - lambda (cof F : A)(cof F : B)],
//   A = w g_o^T, B = delta g_o^T, P = mu F + lambda (J - alpha) cof F,
// and its gradient with respect to F is
//   M = wg [mu A + lambda (cof:A)(cof - D_B) + lambda (J - alpha - cof:B) D_A],
// where D_A = d(cof F : A)/dF.  For a rank-one A = a g^T the columns of D_A are
//   g1 (a x f2) + g2 (f1 x a),  g0 (f2 x a) + g2 (a x f0),  g0 (a x f1) + g1 (f0 x a).
// The third derivative of det F contracted with A and B vanishes because A and B share the row
// vector g_o, so no other term appears.  The gradient of phi_e with respect to corner a_k is M G[k];
// for o it is M g_o = -(sum of the three), which the caller accumulates.
//
// The material sensitivities are proportional to the stress, a small difference of O(1) terms at
// small strain: with the displacement gradient D = F - I = sum_k (d[k] - e[k]) G[k]^T (the edge
// differences are exact in floating point for nearby points), they are formed from
//   J - 1 = tr D + (sum of the principal 2x2 minors of D) + det D,
//   F - cof F = D + D^T - tr(D) I - cof D,
// and lambda (J - alpha) = lambda (J - 1) - mu, so nothing cancels.
//
//   d[k] = x_{a_k} - x_o, e[k] = X_{a_k} - X_o (rest), G[k] = grad N_{a_k} (as in accumulate_tet),
//   evaluated before the update;
//   w, delta: see above; muw, law: wg*mu, wg*lambda (alpha = 1 + mu/lambda is implied).
//   c[k]: d(phi_e)/d(x_{a_k}).
//   dlogmu, dloglambda: d(phi_e)/d(log mu), d(phi_e)/d(log lambda), with alpha = 1 + mu/lambda
//   varying with both.
// Column c of D_a = d(cof F : a g_o^T)/dF (closed form by cross products).
template <class T>
PBGB_HD void adjoint_dcol(T const (&f)[3][3], T const (&go)[3], T const* a, int c, T* out)
{
    int const c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    T u[3], v[3];
    u[0] = a[1] * f[c2][2] - a[2] * f[c2][1]; // a x f_{c+2}
    u[1] = a[2] * f[c2][0] - a[0] * f[c2][2];
    u[2] = a[0] * f[c2][1] - a[1] * f[c2][0];
    v[0] = f[c1][1] * a[2] - f[c1][2] * a[1]; // f_{c+1} x a
    v[1] = f[c1][2] * a[0] - f[c1][0] * a[2];
    v[2] = f[c1][0] * a[1] - f[c1][1] * a[0];
    for (int r = 0; r < 3; ++r)
        out[r] = go[c1] * u[r] + go[c2] * v[r];
}

// The part of adjoint_tet that does not depend on w: everything formed from the positions, the
// rest state and delta.  Split off so that a kernel can form it while it waits for w.
template <class T>
struct AdjointTetPre
{
    T G[3][3];  // rest gradients of the other corners
    T f[3][3];  // F by columns
    T go[3];    // -(G[0] + G[1] + G[2]), the solved corner's gradient
    T k[3][3];  // cofactor columns
    T dB[3][3]; // D_B columns: d(cof F : B)/dF for B = delta g_o^T
    T cg[3];    // (cof F) g_o
    T sg[3];    // (F - cof F) g_o in the displacement-gradient form
    T Jm1, cB, gg;
};

template <class T>
PBGB_HD void adjoint_tet_prepare(T const (&d)[3][3], T const (&e)[3][3], T const (&G)[3][3], T const* delta, AdjointTetPre<T>& q)
{
    for (int m = 0; m < 3; ++m)
        for (int r = 0; r < 3; ++r)
            q.G[m][r] = G[m][r];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            q.f[c][r] = d[0][r] * G[0][c] + d[1][r] * G[1][c] + d[2][r] * G[2][c];
    for (int c = 0; c < 3; ++c)
        q.go[c] = -(G[0][c] + G[1][c] + G[2][c]);
    q.k[0][0] = q.f[1][1] * q.f[2][2] - q.f[1][2] * q.f[2][1];
    q.k[0][1] = q.f[1][2] * q.f[2][0] - q.f[1][0] * q.f[2][2];
    q.k[0][2] = q.f[1][0] * q.f[2][1] - q.f[1][1] * q.f[2][0];
    q.k[1][0] = q.f[2][1] * q.f[0][2] - q.f[2][2] * q.f[0][1];
    q.k[1][1] = q.f[2][2] * q.f[0][0] - q.f[2][0] * q.f[0][2];
    q.k[1][2] = q.f[2][0] * q.f[0][1] - q.f[2][1] * q.f[0][0];
    q.k[2][0] = q.f[0][1] * q.f[1][2] - q.f[0][2] * q.f[1][1];
    q.k[2][1] = q.f[0][2] * q.f[1][0] - q.f[0][0] * q.f[1][2];
    q.k[2][2] = q.f[0][0] * q.f[1][1] - q.f[0][1] * q.f[1][0];
    // Displacement gradient D[col][row].
    T D[3][3];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            D[c][r] = (d[0][r] - e[0][r]) * G[0][c] + (d[1][r] - e[1][r]) * G[1][c] + (d[2][r] - e[2][r]) * G[2][c];
    // cof D (columns D1 x D2, D2 x D0, D0 x D1), J - 1 and F - cof F.
    T cd[3][3];
    for (int c = 0; c < 3; ++c)
    {
        T const* u = D[(c + 1) % 3];
        T const* v = D[(c + 2) % 3];
        cd[c][0] = u[1] * v[2] - u[2] * v[1];
        cd[c][1] = u[2] * v[0] - u[0] * v[2];
        cd[c][2] = u[0] * v[1] - u[1] * v[0];
    }
    T const trD  = D[0][0] + D[1][1] + D[2][2];
    T const min2 = (D[0][0] * D[1][1] - D[1][0] * D[0][1]) + (D[0][0] * D[2][2] - D[2][0] * D[0][2]) +
                   (D[1][1] * D[2][2] - D[2][1] * D[1][2]);
    T const detD = D[0][0] * cd[0][0] + D[0][1] * cd[0][1] + D[0][2] * cd[0][2];
    q.Jm1        = trD + min2 + detD;
    for (int r = 0; r < 3; ++r)
    {
        q.cg[r] = q.go[0] * q.k[0][r] + q.go[1] * q.k[1][r] + q.go[2] * q.k[2][r];
        T acc   = T(0);
        for (int c = 0; c < 3; ++c)
            acc += q.go[c] * (D[c][r] + D[r][c] - cd[c][r] - (c == r ? trD : T(0)));
        q.sg[r] = acc;
    }
    q.cB = delta[0] * q.cg[0] + delta[1] * q.cg[1] + delta[2] * q.cg[2];
    q.gg = q.go[0] * q.go[0] + q.go[1] * q.go[1] + q.go[2] * q.go[2];
    for (int c = 0; c < 3; ++c)
        adjoint_dcol(q.f, q.go, delta, c, q.dB[c]);
}

// The part of adjoint_tet that depends on w.
template <class T>
PBGB_HD void adjoint_tet_finish(AdjointTetPre<T> const& q, T const* w, T const* delta, T muw, T law, T (&c)[3][3], T& dlogmu, T& dloglambda)
{
    T const cA  = w[0] * q.cg[0] + w[1] * q.cg[1] + w[2] * q.cg[2];
    T const FmC = w[0] * q.sg[0] + w[1] * q.sg[1] + w[2] * q.sg[2];
    T const wd  = w[0] * delta[0] + w[1] * delta[1] + w[2] * delta[2];
    dlogmu      = muw * (FmC - q.gg * wd);
    dloglambda  = law * (q.Jm1 * cA - cA * q.cB);
    T const sA  = law * (q.Jm1 - q.cB) - muw;
    T const sC  = law * cA;
    T M[3][3]; // M[col][row]
    for (int col = 0; col < 3; ++col)
    {
        T dA[3];
        adjoint_dcol(q.f, q.go, w, col, dA);
        for (int r = 0; r < 3; ++r)
            M[col][r] = muw * q.go[col] * w[r] + sC * (q.k[col][r] - q.dB[col][r]) + sA * dA[r];
    }
    for (int m = 0; m < 3; ++m)
        for (int r = 0; r < 3; ++r)
            c[m][r] = M[0][r] * q.G[m][0] + M[1][r] * q.G[m][1] + M[2][r] * q.G[m][2];
}

template <class T>
PBGB_HD void adjoint_tet(
    T const (&d)[3][3],
    T const (&e)[3][3],
    T const (&G)[3][3],
    T const* w,
    T const* delta,
    T muw,
    T law,
    T (&c)[3][3],
    T& dlogmu,
    T& dloglambda)
{
    AdjointTetPre<T> q;
    adjoint_tet_prepare(d, e, G, delta, q);
    adjoint_tet_finish(q, w, delta, muw, law, c, dlogmu, dloglambda);
}

} // namespace pbgb
