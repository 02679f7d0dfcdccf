// Adjoint of the VBD step (no reference counterpart: the reference has no differentiation).
//
// A recorded substep keeps, for iterations k = 0..K, the iterate X_k after iteration k (X_0: the
// initial guess) and, per iteration and solved vertex, the inverse of the vertex's 3x3 Newton
// matrix.  Reversing the substep runs the colour sweeps backwards (iterations K..1, colours last
// to first).  Reversing colour c of iteration k is the same block sweep on the transposed system:
// every vertex o of the colour forms w = H^-1 u from its adjoint u, then each incident tet adds
// -d(phi)/dx to the adjoints of its three other corners (atomics: those belong to other colours)
// and to o's own, with phi = w . (g - H delta) (adjoint_tet in vbd_math.cuh).  The state a vertex
// saw before its update is rebuilt from the tape by the colour rank bits of the tet record: a
// corner of lower rank from X_k, one of higher rank (and o itself) from X_{k-1}.
//
// Supported forward settings: no acceleration, no damping, no contact, initial guess Position,
// Inertia or KineticEnergyMinimum (the others depend on the previous velocity through clamps).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_kernels.cuh"

namespace pbgb {

struct AdjointSweepParams
{
    float4 const* __restrict__ xk;   // X_k
    float4 const* __restrict__ xkm1; // X_{k-1}
    float4 const* __restrict__ X;    // rest positions
    TetRecord const* __restrict__ tets;
    int32_t const* __restrict__ solve;
    int32_t const* __restrict__ incPtr;
    uint32_t const* __restrict__ inc;
    float4 const* __restrict__ tape; // inverse Newton matrices of iteration k (2 float4 per entry)
    float const* __restrict__ m;     // lumped masses
    float4* __restrict__ ubar;       // adjoint of the positions (in: after the colour, out: before)
    float4* __restrict__ xtbar;      // adjoint of the inertial target, accumulated
    // Per tet, accumulated in FP64: each is a sum over every iteration of terms that largely
    // cancel (about 4 x iterations x steps of them), which FP32 accumulation does not resolve.
    double* __restrict__ dlogmu;
    double* __restrict__ dloglambda;
    int32_t begin;
    int32_t end;
    float h2;
};

// pdl: programmatic dependent launch (the kernel waits before reading the adjoints).
cudaError_t launch_adjoint_sweep(AdjointSweepParams const& p, int lanes, int block, bool pdl, cudaStream_t s);

// Start of a reversed substep: ubar = xbar + vbar / h (v = (x - xt)/h), xtbar = 0.
//   xbar, vbar: n x 3 adjoints of the substep's end positions and velocities.
cudaError_t launch_adjoint_begin(int32_t n, float const* xbar, float const* vbar, float4* ubar, float4* xtbar, float h, cudaStream_t s);

// End of a reversed substep: the adjoints of the substep's start positions and velocities, in
// place of xbar and vbar.  With xtilde = xt + h v + h^2 a and the initial guess
// x0 = xt + s1 h v + s2 h^2 a (s1 = 0 for Position, 1 otherwise):
//   xbar <- -vbar / h + ubar + xtbar,   vbar <- s1 h ubar + h xtbar.
cudaError_t launch_adjoint_end(int32_t n, float* xbar, float* vbar, float4 const* ubar, float4 const* xtbar, float h, float s1, cudaStream_t s);

} // namespace pbgb
