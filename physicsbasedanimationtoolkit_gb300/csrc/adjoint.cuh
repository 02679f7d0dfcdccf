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
// Rayleigh damping (D = kD / h) makes the Newton matrix (1 + D) H_e + K I and adds D H_e (x_o - xt_o)
// to the gradient, so the tet terms use delta' = (1 + D) delta - D (x_o - xt_o), the own vertex
// loses D H_e w = D (u - K w) / (1 + D) more, and xt_o gains it.  Chebyshev (y_k = omega (raw_k -
// y_{k-2}) + y_{k-2}) is reversed by splitting each iterate's adjoint between its raw sweep result
// and the iterate two back (launch_adjoint_cheb_mix), the reversed sweep reading raw_k for lower
// colours and y_{k-1} for its own and higher colours.  The initial guess enters through
// launch_adjoint_end, including the derivative of the adaptive guesses' acceleration factor on the
// branch the forward took.
//
// Not supported: contact, Anderson, Nesterov, Broyden and trust-region acceleration.
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
    // Damping: D = kD / h (0: none), xs = the substep's start positions, xsbar = their adjoint
    // through the damping term (accumulated).
    float4 const* __restrict__ xs;
    float4* __restrict__ xsbar;
    float D;
    int32_t begin;
    int32_t end;
    float h2;
};

// pdl: programmatic dependent launch (the kernel waits before reading the adjoints).
cudaError_t launch_adjoint_sweep(AdjointSweepParams const& p, int lanes, int block, bool pdl, cudaStream_t s);

// Start of a reversed substep: ubar = xbar + vbar / h (v = (x - xt)/h), xtbar = xsbar = 0, and the
// Chebyshev carries yp = ypp = 0 (nullable).
cudaError_t launch_adjoint_begin(int32_t n, float const* xbar, float const* vbar, float4* ubar, float4* xtbar, float4* xsbar,
                                 float4* yp, float4* ypp, float h, cudaStream_t s);

// Before reversing Chebyshev iteration k: y = yp + ubar (the complete adjoint of y_k), ubar = c1 y
// (raw_k's), yp = ypp (y_{k-1}'s so far), ypp = c2 y (y_{k-2}'s); c1 = omega_k, c2 = 1 - omega_k for
// k > 1, else 1 and 0.
cudaError_t launch_adjoint_cheb_mix(int32_t n, float4* ubar, float4* yp, float4* ypp, float c1, float c2, cudaStream_t s);

// End of a reversed substep: the adjoints of the substep's start positions, velocities and
// previous velocities, in place of xbar, vbar and pbar (n x 3 each).  With xtilde = xt + h v + h^2 a,
// the initial guess x0 = xt + s1 h v + h^2 a_t(v, vtm1) a (vtm1: the previous velocity with GPU
// semantics, v otherwise) and the next previous velocity = v (GPU semantics):
//   xbar <- -vbar/h + ubar + xtbar + xsbar
//   vbar <- s1 h ubar + h xtbar + h^2 (a . ubar) da_t/dv + [GPU] pbar
//   pbar <- h^2 (a . ubar) da_t/dvtm1
// v0, p0, a: the substep's start velocities, previous velocities and external accelerations.
cudaError_t launch_adjoint_end(int32_t n, float* xbar, float* vbar, float* pbar, float4 const* ubar, float4 const* xtbar,
                               float4 const* xsbar, float4 const* v0, float4 const* p0, float4 const* a, float h,
                               int32_t strategy, int32_t gpuSemantics, cudaStream_t s);

} // namespace pbgb
