// Anderson acceleration kernels (see anderson.cuh).
#include "anderson.cuh"
#include "dfloat.cuh"

namespace pbgb {

namespace {

int constexpr kWindowThreads = 256;
int constexpr kWindowVerticesPerThread = 4;

__global__ void anderson_start_kernel(AndersonParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    if (p.broyden)
        p.DG[i] = p.step[i]; // X_0 = x_1 - x_0: iteration 0 is a plain sweep
    else
        p.Gkm1[i] = p.x[i];
    p.Fkm1[i] = p.step[i];
}

// kWindowVerticesPerThread vertices per thread (grid-stride); the mk + 1 products are carried as
// double-float sums (exact products, compensated additions on the FP32 pipe), reduced over the
// warp in the same form, converted to FP64 once per warp, and the warps' sums added in order:
// partials[block * 2 m + t].
__global__ void __launch_bounds__(kWindowThreads) anderson_window_kernel(AndersonParams p)
{
    __shared__ double warpSums[kWindowThreads / 32][2 * kAndersonMaxWindow];
    int const mk = p.mk;
    // Dots with the new column (accA, indices known at compile time so that the accumulators stay
    // in registers) and the new column's dot with F_k (accF).
    DFloat accA[kAndersonMaxWindow], accF = {0.f, 0.f};
#pragma unroll
    for (int t = 0; t < kAndersonMaxWindow; ++t)
        accA[t] = {0.f, 0.f};
    size_t const n = size_t(p.n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x)
    {
        float4 const f  = p.step[i];
        float4 const fp = p.Fkm1[i];
        float4 const df = make_float4(f.x - fp.x, f.y - fp.y, f.z - fp.z, 0.f);
        if (!p.broyden)
        {
            // Broyden's X column was written by the previous update.
            float4 const g              = p.x[i];
            float4 const gp             = p.Gkm1[i];
            p.DG[size_t(p.dkl) * n + i] = make_float4(g.x - gp.x, g.y - gp.y, g.z - gp.z, 0.f);
            p.Gkm1[i]                   = g;
        }
        p.DF[size_t(p.dkl) * n + i] = df;
        p.Fkm1[i]                   = f;
#pragma unroll
        for (int j = 0; j < kAndersonMaxWindow; ++j)
            if (j < mk)
                accA[j] = df_add(accA[j], df_dot3(j == p.dkl ? df : p.DF[size_t(j) * n + i], df));
        accF = df_add(accF, df_dot3(df, f));
    }
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < kAndersonMaxWindow; ++t)
        if (t < mk)
        {
            DFloat const a = df_warp_sum(accA[t]);
            if (lane == 0)
                warpSums[warp][t] = df_to_double(a);
        }
    accF = df_warp_sum(accF);
    if (lane == 0)
        warpSums[warp][mk] = df_to_double(accF);
    __syncthreads();
    if (threadIdx.x < mk + 1)
    {
        double v = 0.0;
        for (int w = 0; w < kWindowThreads / 32; ++w)
            v += warpSums[w][threadIdx.x];
        p.partials[size_t(blockIdx.x) * 2 * p.m + threadIdx.x] = v;
    }
}

int constexpr kSolveThreads = 256;

// One block: the 2 mk sums over the window blocks (each thread a strided set of blocks, then a
// fixed reduction tree: deterministic), the Gram row/column update and the mk x mk ridge-
// regularised solve by Cholesky (thread 0, matrices in shared memory; the few FP64 divisions and
// square roots of a Cholesky keep this latency-bound single thread short).
__global__ void __launch_bounds__(kSolveThreads) anderson_solve_kernel(AndersonParams p, int nblocks)
{
    __shared__ double warpSums[kSolveThreads / 32][2 * kAndersonMaxWindow];
    __shared__ double sums[2 * kAndersonMaxWindow];
    __shared__ double G[kAndersonMaxWindow][kAndersonMaxWindow];
    __shared__ double V[kAndersonMaxWindow][kAndersonMaxWindow];
    int const mk = p.mk, m = p.m, t = threadIdx.x;
    double acc[kAndersonMaxWindow + 1];
#pragma unroll
    for (int j = 0; j <= kAndersonMaxWindow; ++j)
        acc[j] = 0.0;
    for (int b = t; b < nblocks; b += kSolveThreads)
    {
        double const* row = p.partials + size_t(b) * 2 * m;
#pragma unroll
        for (int j = 0; j <= kAndersonMaxWindow; ++j)
            if (j <= mk)
                acc[j] += row[j];
    }
    int const lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int j = 0; j <= kAndersonMaxWindow; ++j)
        if (j <= mk)
        {
            double a = acc[j];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
                a += __shfl_xor_sync(0xffffffffu, a, off);
            if (lane == 0)
                warpSums[warp][j] = a;
        }
    __syncthreads();
    if (t <= mk)
    {
        double v = 0.0;
        for (int w = 0; w < kSolveThreads / 32; ++w)
            v += warpSums[w][t];
        sums[t] = v;
    }
    __syncthreads();
    if (t != 0)
        return;
    // Gram row/column dkl; right-hand side: the new column's product directly, the others updated.
    double const fnew = sums[mk];
    for (int j = 0; j < mk; ++j)
    {
        p.gram[j * m + p.dkl] = sums[j];
        p.gram[p.dkl * m + j] = sums[j];
        p.rhs[j]              = j == p.dkl ? fnew : p.rhs[j] + sums[j];
    }
    for (int j = 0; j < mk; ++j)
        sums[mk + j] = p.rhs[j];
    if (p.broyden)
    {
        // Eigen's LeastSquaresConjugateGradient (IdentityPreconditioner, zero initial guess) on
        // min |DF gamma - F_k|, written on the normal equations: the normal residual
        // DF^T (F_k - DF gamma) starts at b = DF^T F_k and drops by a (DF^T DF) p per step.
        double* gam = &V[0][0];
        double* nr  = &V[1][0];
        double* pv  = &V[2][0];
        double* Ap  = &V[3][0];
        double rhsNorm2 = 0.0;
        for (int j = 0; j < mk; ++j)
        {
            gam[j] = 0.0;
            nr[j]  = sums[mk + j];
            pv[j]  = nr[j];
            rhsNorm2 += nr[j] * nr[j];
        }
        double const threshold = 1e-20 * rhsNorm2; // tolerance 1e-10, squared
        if (rhsNorm2 > 0.0)
        {
            double absNew = rhsNorm2;
            for (int it = 0; it < p.maxIters; ++it)
            {
                double pAp = 0.0;
                for (int i = 0; i < mk; ++i)
                {
                    double v = 0.0;
                    for (int j = 0; j < mk; ++j)
                        v += p.gram[i * m + j] * pv[j];
                    Ap[i] = v;
                    pAp += pv[i] * v;
                }
                double const a = absNew / pAp;
                double rn2     = 0.0;
                for (int j = 0; j < mk; ++j)
                {
                    gam[j] += a * pv[j];
                    nr[j] -= a * Ap[j];
                    rn2 += nr[j] * nr[j];
                }
                if (rn2 < threshold)
                    break;
                double const beta = rn2 / absNew;
                absNew            = rn2;
                for (int j = 0; j < mk; ++j)
                    pv[j] = nr[j] + beta * pv[j];
            }
        }
        for (int j = 0; j < mk; ++j)
            p.alpha[j] = gam[j];
        return;
    }
    // (G + eps I) alpha = b by Cholesky, eps = 1e-10 of the largest diagonal entry: the exact
    // least-squares solution where DF is well conditioned, directions far below eps damped to zero.
    double dmax = 0.0;
    for (int i = 0; i < mk; ++i)
        dmax = fmax(dmax, p.gram[i * m + i]);
    double const eps = 1e-10 * dmax + 1e-300;
    for (int i = 0; i < mk; ++i)
        for (int j = 0; j <= i; ++j)
            G[i][j] = p.gram[i * m + j] + (i == j ? eps : 0.0);
    for (int j = 0; j < mk; ++j)
    {
        double d = G[j][j];
        for (int k = 0; k < j; ++k)
            d -= G[j][k] * G[j][k];
        d          = d > eps ? d : eps;
        double const r = sqrt(d);
        G[j][j]        = r;
        V[0][j]        = 1.0 / r; // reciprocal pivots
        for (int i = j + 1; i < mk; ++i)
        {
            double v = G[i][j];
            for (int k = 0; k < j; ++k)
                v -= G[i][k] * G[j][k];
            G[i][j] = v * V[0][j];
        }
    }
    // L y = b, then L^T alpha = y (alpha into sums[0..mk)).
    for (int i = 0; i < mk; ++i)
    {
        double v = sums[mk + i];
        for (int k = 0; k < i; ++k)
            v -= G[i][k] * sums[k];
        sums[i] = v * V[0][i];
    }
    for (int i = mk - 1; i >= 0; --i)
    {
        double v = sums[i];
        for (int k = i + 1; k < mk; ++k)
            v -= G[k][i] * sums[k];
        sums[i] = v * V[0][i];
    }
    for (int j = 0; j < mk; ++j)
        p.alpha[j] = sums[j];
}

__global__ void anderson_update_kernel(AndersonParams p)
{
    // The coefficients once per block in FP32 (the update itself is FP32).
    __shared__ float alpha[kAndersonMaxWindow];
    if (threadIdx.x < p.mk)
        alpha[threadIdx.x] = float(p.alpha[threadIdx.x]);
    __syncthreads();
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    float4 u       = p.x[i];
    size_t const n = size_t(p.n);
    if (p.broyden)
    {
        // x <- x - (X + DF) gamma; the next X column is this iteration's total move.
        float cx = 0.f, cy = 0.f, cz = 0.f;
        for (int j = 0; j < p.mk; ++j)
        {
            float const a   = alpha[j];
            float4 const X  = p.DG[size_t(j) * n + i];
            float4 const Df = p.DF[size_t(j) * n + i];
            cx += a * (X.x + Df.x);
            cy += a * (X.y + Df.y);
            cz += a * (X.z + Df.z);
        }
        p.x[i] = make_float4(u.x - cx, u.y - cy, u.z - cz, 0.f);
        if (p.xh)
            p.xh[i] = p.x[i];
        if (p.next >= 0)
        {
            float4 const f               = p.step[i];
            p.DG[size_t(p.next) * n + i] = make_float4(f.x - cx, f.y - cy, f.z - cz, 0.f);
        }
        return;
    }
    for (int j = 0; j < p.mk; ++j)
    {
        float const a  = alpha[j];
        float4 const d = p.DG[size_t(j) * n + i];
        u.x -= a * d.x;
        u.y -= a * d.y;
        u.z -= a * d.z;
    }
    u.w    = 0.f;
    p.x[i] = u;
    if (p.xh)
        p.xh[i] = u;
}

inline int blocks_of(int64_t n, int b)
{
    return int((n + b - 1) / b);
}

} // namespace

int anderson_window_blocks(int32_t n)
{
    return blocks_of(n > 0 ? n : 1, kWindowThreads * kWindowVerticesPerThread);
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
    anderson_solve_kernel<<<1, kSolveThreads, 0, s>>>(p, anderson_window_blocks(p.n));
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
