// Device kernels of the VBD step.  Layout in HBM (all arrays of the whole, possibly batched,
// system; indices global):
//
//   x, xt, xtilde, v, aext, vprev : float4 per vertex (xyz, w unused except xt.w = lumped mass)
//   tv    : int4   per tet   — the 4 vertex indices
//   tg    : 3 float4 per tet — (GP row 1, wg*mu), (GP row 2, wg*lambda), (GP row 3, alpha)
//           where GP row 0 = -(rows 1+2+3) and alpha = 1 + mu/lambda
//   solve : free vertices, colour-major; inside a colour sorted by decreasing degree
//   incPtr: offsets of each solved vertex's incidences; inc: (tet << 2 | local index), tets
//           ascending
//
// A tet record is 64 B and is read by each of its 4 vertices in 4 different colour passes of an
// iteration; the record table stays L2-resident for meshes whose table fits in L2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_math.cuh"

namespace pbgb {

struct SweepParams
{
    float4* __restrict__ x;
    float4 const* __restrict__ xt;     // .w = lumped mass
    float4 const* __restrict__ xtilde; // inertial target
    int4 const* __restrict__ tv;
    float4 const* __restrict__ tg;
    int32_t const* __restrict__ solve;
    int32_t const* __restrict__ incPtr;
    uint32_t const* __restrict__ inc;
    int32_t begin;
    int32_t end;
    float h;
    float h2;
    float kD;
    float detHZero;
};

struct SubstepParams
{
    float4* __restrict__ x;
    float4* __restrict__ xt;
    float4* __restrict__ xtilde;
    float4* __restrict__ v;
    float4 const* __restrict__ aext;
    float4* __restrict__ vprev;
    float const* __restrict__ m;
    int32_t* __restrict__ flags;
    int32_t n;
    float h;
    float h2;
    int32_t strategy;
    int32_t gpuSemantics;
};

struct ChebyshevParams
{
    float4* __restrict__ x;
    float4* __restrict__ xkm1;
    float4* __restrict__ xkm2;
    int32_t n;
    int32_t k;
    float omega;
};

struct EnergyParams
{
    float4 const* __restrict__ x;
    float4 const* __restrict__ xtilde;
    float const* __restrict__ m;
    int4 const* __restrict__ tv;
    float4 const* __restrict__ tg;
    int32_t nV;
    int32_t nT;
    double dt2;
    double* __restrict__ out; // objective: out[0]; gradient: 3 x nV
};

// Launchers (defined in vbd_kernels.cu).  Each returns the launch status.
cudaError_t launch_sweep(SweepParams const& p, int lanes, int block, cudaStream_t s);
cudaError_t launch_begin_substep(SubstepParams const& p, cudaStream_t s);
cudaError_t launch_end_substep(SubstepParams const& p, cudaStream_t s);
cudaError_t launch_chebyshev(ChebyshevParams const& p, cudaStream_t s);
cudaError_t launch_objective(EnergyParams const& p, cudaStream_t s);
cudaError_t launch_gradient(EnergyParams const& p, cudaStream_t s);
cudaError_t launch_pack3(float const* in3, float4* out4, int32_t n, cudaStream_t s);
cudaError_t launch_unpack3(float4 const* in4, float* out3, int32_t n, cudaStream_t s);

} // namespace pbgb
