// Anderson-accelerated VBD on the device (reference: pbat::sim::vbd::AndersonIntegrator,
// sim/vbd/AndersonIntegrator.cpp:24-57, and gpu/impl/vbd/AndersonIntegrator.cu:36-105).
//
// After VBD iteration k >= 1 of a substep, with G_k = x and F_k = G_k - x_{k-1}, column
// (k-1) mod m of the window receives DG = G_k - G_{k-1} and DF = F_k - F_{k-1}, and
// x = G_k - DG alpha with alpha the minimum-norm minimiser of |DF alpha - F_k| over the
// mk = min(m, k) filled columns.  Layout and kernels:
//   window kernel: one streaming pass that forms the new column and, per block, the FP64 partial
//       dot products DF_j . DF_new (j < mk) and DF_new . F_k in a fixed reduction order (since
//       F_k = F_{k-1} + DF_new, DF_j . F_k = DF_j . F_{k-1} + DF_j . DF_new for the unchanged
//       columns, so only the new column needs its own product with F_k);
//   solve kernel (one block): sums the block partials in order, refreshes row and column
//       (k-1) mod m of the persistent FP64 Gram matrix DF^T DF, and solves
//       (DF^T DF + eps I) alpha = DF^T F_k by Cholesky, eps = 1e-10 of the largest diagonal entry;
//   update kernel: x = G_k - DG alpha.
// F_k is taken from the increments the sweep applied (x_k - x_{k-1} vertex by vertex, each free
// vertex moving once per iteration), so it keeps FP32 relative precision when it is far smaller than
// the positions.
// The reference's CPU integrator uses a complete orthogonal decomposition with threshold 1e-10 and
// its GPU integrator a Householder QR whose zero pivots are replaced by a tiny value; all give the
// same alpha when DF is well conditioned.  When it is not, the ridge damps the directions below eps
// towards zero as the CPU's minimum-norm solution does, where a QR with patched pivots can return
// arbitrarily large coefficients.
//
// Broyden-accelerated VBD (sim/vbd/BroydenIntegrator.cpp:41-80) runs on the same window: with
// VBD(f_k) = -(the iteration's increments), its G_{k-m} VBD(Delta f) columns are -DF, and its
// iterate-difference columns X_j (x_k - x_{k-1}, pre-sweep iterates) are kept in DG.  gamma solves
// min |DF gamma - F_k| by the reference's least-squares conjugate gradient (Eigen's CGLS, zero
// initial guess, at most max(1, m - k) iterations, relative tolerance 1e-10), run here on the
// normal equations with the FP64 Gram matrix (the same iterates in exact arithmetic), and
// x <- x - (X + DF) gamma.  The update kernel also writes the next X column,
// x_{k+1} - x_k = F_k - (X + DF) gamma, without cancelling against the positions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pbgb {

int constexpr kAndersonMaxWindow = 16;

struct AndersonParams
{
    float4* __restrict__ x;
    float4* xh; // with contact: the two-buffer sweep's copy of the iterate, updated with x (or null)
    float4 const* __restrict__ step; // the last VBD iteration's increments: F_k = step
    float4* __restrict__ Gkm1; // last un-accelerated iterate G_{k-1}
    float4* __restrict__ Fkm1; // last residual F_{k-1}
    float4* __restrict__ DF;   // m columns of n float4 (column j at j * n)
    float4* __restrict__ DG;
    double* __restrict__ partials; // per window block: mk dots DF_j . DF_new, then DF_new . F_k
    double* __restrict__ gram;     // m x m, row-major
    double* __restrict__ rhs;      // m: DF_j . F_k
    double* __restrict__ alpha;    // m
    int32_t n;
    int32_t m;
    int32_t dkl; // column written this iteration
    int32_t mk;  // filled columns
    int32_t broyden;  // 0: Anderson, 1: Broyden
    int32_t maxIters; // Broyden: conjugate-gradient iterations of this solve
    int32_t next;     // Broyden: X column the update writes for the next iteration (-1: none)
};

int anderson_window_blocks(int32_t n);

// After iteration 0: G_{k-1} = x, F_{k-1} = the iteration's increments (Broyden: the first X
// column = the increments, F_{k-1} = the increments).
cudaError_t launch_anderson_start(AndersonParams const& p, cudaStream_t s);
cudaError_t launch_anderson_window(AndersonParams const& p, cudaStream_t s);
cudaError_t launch_anderson_solve(AndersonParams const& p, cudaStream_t s);
cudaError_t launch_anderson_update(AndersonParams const& p, cudaStream_t s);

} // namespace pbgb
