// Nesterov acceleration kernels (see nesterov.cuh).
#include "nesterov.cuh"

namespace pbgb {

namespace {

__global__ void nesterov_extrapolate_kernel(int32_t n, float4 const* __restrict__ x, float4 const* __restrict__ x0, float4* __restrict__ y, float beta)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 const a = x[i], o = x0[i];
    y[i]           = make_float4(a.x + beta * (a.x - o.x), a.y + beta * (a.y - o.y), a.z + beta * (a.z - o.z), 0.f);
}

__global__ void nesterov_update_kernel(int32_t n, float4* __restrict__ x, float4 const* __restrict__ x0, float4 const* __restrict__ y, float alpha)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 const a = x[i], o = x0[i], b = y[i];
    x[i]           = make_float4(b.x - alpha * (a.x - o.x), b.y - alpha * (a.y - o.y), b.z - alpha * (a.z - o.z), 0.f);
}

inline int blocks_of(int64_t n)
{
    return int((n + 255) / 256);
}

} // namespace

cudaError_t launch_nesterov_extrapolate(int32_t n, float4 const* x, float4 const* x0, float4* y, float beta, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    nesterov_extrapolate_kernel<<<blocks_of(n), 256, 0, s>>>(n, x, x0, y, beta);
    return cudaGetLastError();
}

cudaError_t launch_nesterov_update(int32_t n, float4* x, float4 const* x0, float4 const* y, float alpha, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    nesterov_update_kernel<<<blocks_of(n), 256, 0, s>>>(n, x, x0, y, alpha);
    return cudaGetLastError();
}

} // namespace pbgb
