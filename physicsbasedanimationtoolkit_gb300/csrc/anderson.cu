// Anderson acceleration kernels (see anderson.cuh).
#include "anderson.cuh"

namespace pbgb {

namespace {

int constexpr kWindowThreads = 256;

__device__ __forceinline__ double dot3(float4 a, float4 b)
{
    return double(a.x) * double(b.x) + double(a.y) * double(b.y) + double(a.z) * double(b.z);
}

__global__ void anderson_start_kernel(AndersonParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    p.Gkm1[i] = p.x[i];
    p.Fkm1[i] = p.step[i];
}

// One vertex per thread; 2 mk FP64 partial sums reduced per block (warp shuffles, then the warps'
// sums in order), written to partials[block * 2 m + t].
__global__ void __launch_bounds__(kWindowThreads) anderson_window_kernel(AndersonParams p)
{
    __shared__ double warpSums[kWindowThreads / 32][2 * kAndersonMaxWindow];
    int const i  = blockIdx.x * blockDim.x + threadIdx.x;
    int const mk = p.mk;
    // Dots with the new column (accA) and with F_k (accB); indices known at compile time so that
    // the accumulators stay in registers.
    double accA[kAndersonMaxWindow], accB[kAndersonMaxWindow];
#pragma unroll
    for (int t = 0; t < kAndersonMaxWindow; ++t)
        accA[t] = accB[t] = 0.0;
    if (i < p.n)
    {
        float4 const g  = p.x[i];
        float4 const f  = p.step[i];
        float4 const gp = p.Gkm1[i];
        float4 const fp = p.Fkm1[i];
        float4 const dg = make_float4(g.x - gp.x, g.y - gp.y, g.z - gp.z, 0.f);
        float4 const df = make_float4(f.x - fp.x, f.y - fp.y, f.z - fp.z, 0.f);
        size_t const n  = size_t(p.n);
        p.DG[size_t(p.dkl) * n + i] = dg;
        p.DF[size_t(p.dkl) * n + i] = df;
        p.Gkm1[i]                   = g;
        p.Fkm1[i]                   = f;
#pragma unroll
        for (int j = 0; j < kAndersonMaxWindow; ++j)
            if (j < mk)
            {
                float4 const c = j == p.dkl ? df : p.DF[size_t(j) * n + i];
                accA[j]        = dot3(c, df);
                accB[j]        = dot3(c, f);
            }
    }
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < kAndersonMaxWindow; ++t)
        if (t < mk)
        {
            double a = accA[t], c = accB[t];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
            {
                a += __shfl_xor_sync(0xffffffffu, a, off);
                c += __shfl_xor_sync(0xffffffffu, c, off);
            }
            if (lane == 0)
            {
                warpSums[warp][t]      = a;
                warpSums[warp][mk + t] = c;
            }
        }
    __syncthreads();
    if (threadIdx.x < 2 * mk)
    {
        double v = 0.0;
        for (int w = 0; w < kWindowThreads / 32; ++w)
            v += warpSums[w][threadIdx.x];
        p.partials[size_t(blockIdx.x) * 2 * p.m + threadIdx.x] = v;
    }
}

// One block: the 2 mk sums over the window blocks in order, the Gram row/column update and the
// mk x mk minimum-norm least-squares solve by cyclic Jacobi rotations (thread 0).
__global__ void anderson_solve_kernel(AndersonParams p, int nblocks)
{
    __shared__ double sums[2 * kAndersonMaxWindow];
    int const mk = p.mk, m = p.m, t = threadIdx.x;
    if (t < 2 * mk)
    {
        double v = 0.0;
        for (int b = 0; b < nblocks; ++b)
            v += p.partials[size_t(b) * 2 * m + t];
        sums[t] = v;
    }
    __syncthreads();
    if (t != 0)
        return;
    for (int j = 0; j < mk; ++j)
    {
        p.gram[j * m + p.dkl] = sums[j];
        p.gram[p.dkl * m + j] = sums[j];
    }
    double G[kAndersonMaxWindow][kAndersonMaxWindow], V[kAndersonMaxWindow][kAndersonMaxWindow];
    for (int i = 0; i < mk; ++i)
        for (int j = 0; j < mk; ++j)
        {
            G[i][j] = p.gram[i * m + j];
            V[i][j] = i == j ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 64; ++sweep)
    {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < mk; ++i)
            for (int j = 0; j < mk; ++j)
                if (i == j)
                    diag += G[i][j] * G[i][j];
                else
                    off += G[i][j] * G[i][j];
        if (off <= 1e-30 * diag || off == 0.0)
            break;
        for (int a = 0; a < mk; ++a)
            for (int b = a + 1; b < mk; ++b)
            {
                if (G[a][b] == 0.0)
                    continue;
                double const theta = (G[b][b] - G[a][a]) / (2.0 * G[a][b]);
                double const tn    = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double const c     = 1.0 / sqrt(tn * tn + 1.0), sn = tn * c;
                for (int k = 0; k < mk; ++k)
                {
                    double const gka = G[k][a], gkb = G[k][b];
                    G[k][a]          = c * gka - sn * gkb;
                    G[k][b]          = sn * gka + c * gkb;
                }
                for (int k = 0; k < mk; ++k)
                {
                    double const gak = G[a][k], gbk = G[b][k];
                    G[a][k]          = c * gak - sn * gbk;
                    G[b][k]          = sn * gak + c * gbk;
                }
                for (int k = 0; k < mk; ++k)
                {
                    double const vka = V[k][a], vkb = V[k][b];
                    V[k][a]          = c * vka - sn * vkb;
                    V[k][b]          = sn * vka + c * vkb;
                }
            }
    }
    double lmax = 0.0;
    for (int i = 0; i < mk; ++i)
        lmax = fmax(lmax, G[i][i]);
    double al[kAndersonMaxWindow];
    for (int j = 0; j < mk; ++j)
        al[j] = 0.0;
    for (int e = 0; e < mk; ++e)
    {
        double const l = G[e][e];
        if (!(l > 1e-14 * lmax))
            continue;
        double proj = 0.0;
        for (int i = 0; i < mk; ++i)
            proj += V[i][e] * sums[mk + i];
        for (int j = 0; j < mk; ++j)
            al[j] += V[j][e] * proj / l;
    }
    for (int j = 0; j < mk; ++j)
        p.alpha[j] = al[j];
}

__global__ void anderson_update_kernel(AndersonParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    float4 u       = p.x[i];
    size_t const n = size_t(p.n);
    for (int j = 0; j < p.mk; ++j)
    {
        float const a  = float(p.alpha[j]);
        float4 const d = p.DG[size_t(j) * n + i];
        u.x -= a * d.x;
        u.y -= a * d.y;
        u.z -= a * d.z;
    }
    u.w    = 0.f;
    p.x[i] = u;
}

inline int blocks_of(int64_t n, int b)
{
    return int((n + b - 1) / b);
}

} // namespace

int anderson_window_blocks(int32_t n)
{
    return blocks_of(n > 0 ? n : 1, kWindowThreads);
}

cudaError_t launch_anderson_start(AndersonParams const& p, cudaStream_t s)
{
    if (p.n <= 0)
        return cudaSuccess;
    anderson_start_kernel<<<blocks_of(p.n, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_anderson_window(AndersonParams const& p, cudaStream_t s)
{
    if (p.mk < 1 || p.mk > kAndersonMaxWindow || p.m > kAndersonMaxWindow || p.dkl < 0 || p.dkl >= p.m)
        return cudaErrorInvalidValue;
    anderson_window_kernel<<<anderson_window_blocks(p.n), kWindowThreads, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_anderson_solve(AndersonParams const& p, cudaStream_t s)
{
    anderson_solve_kernel<<<1, 64, 0, s>>>(p, anderson_window_blocks(p.n));
    return cudaGetLastError();
}

cudaError_t launch_anderson_update(AndersonParams const& p, cudaStream_t s)
{
    if (p.n <= 0)
        return cudaSuccess;
    anderson_update_kernel<<<blocks_of(p.n, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

} // namespace pbgb
