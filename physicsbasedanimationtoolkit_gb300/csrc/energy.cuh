// Backward-Euler objective terms shared by the objective/gradient kernels and the trust-region
// reductions, so every objective value on the device comes from the same arithmetic.
//   f(x) = sum_i 1/2 m_i |x_i - xtilde_i|^2 + dt^2 sum_e wg_e Psi(F_e)        (sim/vbd/Integrator.cpp:138-165)
// Per-entity terms are formed from FP32 positions with FP64 products; sums are FP64.
#pragma once

#include "vbd_kernels.cuh"
#include "vbd_math.cuh"

namespace pbgb {

__device__ __forceinline__ double warp_sum(double v)
{
    for (int off = 16; off > 0; off >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Tet geometry helper: deformation gradient F (columns f[c]) of tet e, the shape-function
// gradients of its 4 corners (G4[a]) and its material scalars.
__device__ __forceinline__ void tet_F(EnergyParams const& p, int e, float f[3][3], int4& t, float G4[4][3], float4& mat)
{
    TetRecord const& r = p.tets[e];
    uint4 const tu     = r.v;
    t   = make_int4(int(tu.x & kIndexMask), int(tu.y & kIndexMask), int(tu.z & kIndexMask), int(tu.w & kIndexMask));
    mat = r.mat;
    int const vid[4] = {t.x, t.y, t.z, t.w};
    float4 const X0 = p.X[vid[0]], x0 = p.x[vid[0]];
    float d[3][3], E[3][3], G[3][3];
    for (int m = 0; m < 3; ++m)
    {
        float4 const Xa = p.X[vid[m + 1]], xa = p.x[vid[m + 1]];
        d[m][0] = xa.x - x0.x, d[m][1] = xa.y - x0.y, d[m][2] = xa.z - x0.z;
        E[m][0] = Xa.x - X0.x, E[m][1] = Xa.y - X0.y, E[m][2] = Xa.z - X0.z;
    }
    rest_gradients(E, G);
    for (int c = 0; c < 3; ++c)
    {
        for (int rr = 0; rr < 3; ++rr)
            f[c][rr] = d[0][rr] * G[0][c] + d[1][rr] * G[1][c] + d[2][rr] * G[2][c];
        G4[0][c] = -(G[0][c] + G[1][c] + G[2][c]);
        G4[1][c] = G[0][c];
        G4[2][c] = G[1][c];
        G4[3][c] = G[2][c];
    }
}

// Displacement gradient D = F - I of tet e, D[c][r] = dF_rc, formed from the corner
// displacements u_a = x_a - X_a (for a near-rest tet these FP32 differences are exact), and the
// tet's material scalars.
__device__ __forceinline__ void tet_D(EnergyParams const& p, int e, float D[3][3], float4& mat)
{
    TetRecord const& r = p.tets[e];
    uint4 const tu     = r.v;
    mat                = r.mat;
    int const vid[4]   = {int(tu.x & kIndexMask), int(tu.y & kIndexMask), int(tu.z & kIndexMask), int(tu.w & kIndexMask)};
    float4 const X0 = p.X[vid[0]], x0 = p.x[vid[0]];
    float const u0[3] = {x0.x - X0.x, x0.y - X0.y, x0.z - X0.z};
    float du[3][3], E[3][3], G[3][3];
    for (int m = 0; m < 3; ++m)
    {
        float4 const Xa = p.X[vid[m + 1]], xa = p.x[vid[m + 1]];
        du[m][0] = (xa.x - Xa.x) - u0[0], du[m][1] = (xa.y - Xa.y) - u0[1], du[m][2] = (xa.z - Xa.z) - u0[2];
        E[m][0] = Xa.x - X0.x, E[m][1] = Xa.y - X0.y, E[m][2] = Xa.z - X0.z;
    }
    rest_gradients(E, G);
    for (int c = 0; c < 3; ++c)
        for (int rr = 0; rr < 3; ++rr)
            D[c][rr] = du[0][rr] * G[0][c] + du[1][rr] * G[1][c] + du[2][rr] * G[2][c];
}

// Contribution of entity j to f: vertex j's inertia (j < nV) plus tet j's weighted elastic energy
// (j < nT) less its rest-state value, which the caller adds once as dt^2 p.restEnergy.
// mat = (wg mu, wg lambda, 1 + mu/lambda, .) per tet.  With D = F - I and c = mu/lambda,
//   Psi = mu/2 (2 tr D + |D|^2) + lambda/2 (J - 1 - c)^2
//       = lambda c^2 / 2 + mu/2 (2 tr D + |D|^2) + lambda (J - 1) ((J - 1)/2 - c),
//   J - 1 = tr D + (sum of D's principal 2x2 minors) + det D,
// so every term left scales with the strain and keeps its relative precision in FP32 (relative
// error ~1e-7 of the strain energy, not of the rest-state constant); the sum is FP64.  GB300's
// FP64 rate is a small fraction of its FP32 rate, so FP64 is kept to the accumulation.
// The two FP32 parts of entry j: the inertial term of vertex j (kin, 0 past nV) and the elastic
// term of tet j before its dt^2 factor (elas, 0 past nT).
__device__ __forceinline__ void objective_parts(EnergyParams const& p, int j, float& kin, float& elas)
{
    kin  = 0.f;
    elas = 0.f;
    if (j < p.nV)
    {
        float4 const x = p.x[j], y = p.xtilde[j];
        float const dx = x.x - y.x, dy = x.y - y.y, dz = x.z - y.z;
        kin            = 0.5f * p.m[j] * (dx * dx + dy * dy + dz * dz);
    }
    if (j < p.nT)
    {
        float D[3][3];
        float4 mat;
        tet_D(p, j, D, mat);
        float const tr = D[0][0] + D[1][1] + D[2][2];
        float n2       = 0.f;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r)
                n2 += D[c][r] * D[c][r];
        float const minors = (D[0][0] * D[1][1] - D[0][1] * D[1][0]) + (D[0][0] * D[2][2] - D[0][2] * D[2][0]) +
                             (D[1][1] * D[2][2] - D[1][2] * D[2][1]);
        float const detD = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) -
                           D[1][0] * (D[0][1] * D[2][2] - D[0][2] * D[2][1]) +
                           D[2][0] * (D[0][1] * D[1][2] - D[0][2] * D[1][1]);
        float const Jm1 = tr + minors + detD;
        float const c   = mat.z - 1.f;
        elas            = mat.y * Jm1 * (0.5f * Jm1 - c) + 0.5f * mat.x * (2.f * tr + n2);
    }
}

__device__ __forceinline__ double objective_term(EnergyParams const& p, int j)
{
    float kin, elas;
    objective_parts(p, j, kin, elas);
    double acc = 0.0;
    if (j < p.nV)
        acc += double(kin);
    if (j < p.nT)
        acc += p.dt2 * double(elas);
    return acc;
}

} // namespace pbgb
