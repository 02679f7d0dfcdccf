// Anderson-accelerated VBD on the device (reference: pbat::sim::vbd::AndersonIntegrator,
// sim/vbd/AndersonIntegrator.cpp:24-57, and gpu/impl/vbd/AndersonIntegrator.cu:36-105).
//
// After VBD iteration k >= 1 of a substep, with G_k = x and F_k = G_k - x_{k-1}, column
// (k-1) mod m of the window receives DG = G_k - G_{k-1} and DF = F_k - F_{k-1}, and
// x = G_k - DG alpha with alpha the minimum-norm minimiser of |DF alpha - F_k| over the
// mk = min(m, k) filled columns.  Layout and kernels:
//   window kernel: one streaming pass that forms the new column and, per block, the FP64 partial
//       dot products DF_j . DF_new and DF_j . F_k (j < mk) in a fixed reduction order;
//   solve kernel (one block): sums the block partials in order, refreshes row and column
//       (k-1) mod m of the persistent FP64 Gram matrix DF^T DF, and solves the mk x mk system by a
//       Jacobi eigen-decomposition (pseudo-inverse over eigenvalues above 1e-14 of the largest);
//   update kernel: x = G_k - DG alpha.
// F_k is taken from the increments the sweep applied (x_k - x_{k-1} vertex by vertex, each free
// vertex moving once per iteration), so it keeps FP32 relative precision when it is far smaller than
// the positions.
// The reference's CPU integrator uses a complete orthogonal decomposition with threshold 1e-10 and
// its GPU integrator a Householder QR whose zero pivots are replaced by a tiny value; both give the
// same alpha when DF has full rank, and the pseudo-inverse gives the CPU's minimum-norm solution
// when it does not.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pbgb {

int constexpr kAndersonMaxWindow = 16;

struct AndersonParams
{
    float4* __restrict__ x;
    float4 const* __restrict__ step; // the last VBD iteration's increments: F_k = step
    float4* __restrict__ Gkm1; // last un-accelerated iterate G_{k-1}
    float4* __restrict__ Fkm1; // last residual F_{k-1}
    float4* __restrict__ DF;   // m columns of n float4 (column j at j * n)
    float4* __restrict__ DG;
    double* __restrict__ partials; // per window block: mk dots with DF_new, then mk dots with F_k
    double* __restrict__ gram;     // m x m, row-major
    double* __restrict__ alpha;    // m
    int32_t n;
    int32_t m;
    int32_t dkl; // column written this iteration
    int32_t mk;  // filled columns
};

int anderson_window_blocks(int32_t n);

// After iteration 0: G_{k-1} = x, F_{k-1} = the iteration's increments.
cudaError_t launch_anderson_start(AndersonParams const& p, cudaStream_t s);
cudaError_t launch_anderson_window(AndersonParams const& p, cudaStream_t s);
cudaError_t launch_anderson_solve(AndersonParams const& p, cudaStream_t s);
cudaError_t launch_anderson_update(AndersonParams const& p, cudaStream_t s);

} // namespace pbgb
