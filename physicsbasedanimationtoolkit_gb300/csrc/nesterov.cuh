// Nesterov-accelerated VBD on the device (reference: pbat::sim::vbd::NesterovIntegrator,
// sim/vbd/NesterovIntegrator.cpp:16-43; the reference has it on the CPU only).  With x_0 the
// iterate at the start of the solve, alpha = 1/L and the scalars lambda, beta of the reference's
// recurrence, every iteration k > start does
//   y = x + beta (x - x_0)          before the colour sweeps,
//   x = y - alpha (x - x_0)         after them
// (x_0 stays the solve's start as in the reference).  Both are streaming kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pbgb {

cudaError_t launch_nesterov_extrapolate(int32_t n, float4 const* x, float4 const* x0, float4* y, float beta, cudaStream_t s);
cudaError_t launch_nesterov_update(int32_t n, float4* x, float4 const* x0, float4 const* y, float alpha, cudaStream_t s);

} // namespace pbgb
