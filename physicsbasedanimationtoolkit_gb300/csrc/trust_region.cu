// Trust-region accelerated VBD kernels (see trust_region.cuh).
#include "trust_region.cuh"
#include "dfloat.cuh"
#include "energy.cuh"

#include <cfloat>

namespace pbgb {

namespace {

int constexpr kTrustBlock = 256;
double constexpr kTrustZero = 1e-6; // the reference's step-bound tolerance

inline int trust_blocks(int64_t n)
{
    int64_t g = (n + kTrustBlock - 1) / kTrustBlock;
    if (g > kTrustMaxBlocks)
        g = kTrustMaxBlocks;
    return g < 1 ? 1 : int(g);
}

// Sum over the block in a fixed order; the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double warps[kTrustBlock / 32];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0)
        warps[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32)
    {
        r = threadIdx.x < (blockDim.x >> 5) ? warps[threadIdx.x] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Block total from one FP64 value per warp (valid in lane 0), added over the warps in order; the
// result is valid in thread 0.
__device__ __forceinline__ double block_sum_of_warps(double w)
{
    __shared__ double warps[kTrustBlock / 32];
    if ((threadIdx.x & 31) == 0)
        warps[threadIdx.x >> 5] = w;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < int(blockDim.x >> 5); ++k)
            r += warps[k];
    return r;
}

// Publishes this block's partial; returns the grid total in thread 0 of the last block to finish
// (true there), summed over the partials in block order.  Other blocks return false.
__device__ bool grid_sum_last(TrustParams const& p, double blockTotal, double& total)
{
    __shared__ bool last;
    if (threadIdx.x == 0)
    {
        p.partials[blockIdx.x] = blockTotal;
        __threadfence();
        unsigned int const done = atomicAdd(&p.state->ticket, 1u);
        last                    = done == gridDim.x - 1;
    }
    __syncthreads();
    if (!last)
        return false;
    __threadfence();
    double v = 0.0;
    for (int b = threadIdx.x; b < int(gridDim.x); b += blockDim.x)
        v += __ldcg(p.partials + b);
    total = block_sum(v);
    if (threadIdx.x == 0)
        p.state->ticket = 0u;
    return true;
}

// Minimiser of m(t) = a t^2 + b t + c (TrustRegionIntegrator.cu:400-430), the reference's float
// thresholds kept: FLT_MIN as zero, FLT_MAX as infinity.
__device__ double model_optimal_step(double const aQ[3])
{
    double const zero = FLT_MIN, inf = FLT_MAX;
    if (fabs(aQ[0]) > zero)
        return aQ[0] > zero ? -aQ[1] / (2.0 * aQ[0]) : inf;
    if (fabs(aQ[1]) > zero)
        return aQ[1] > 0.0 ? -inf : inf;
    return 0.0;
}

// std::clamp(v, lo, hi) as min(max(v, lo), hi).
__device__ __forceinline__ double clamp_std(double v, double lo, double hi)
{
    double const m = (v < lo) ? lo : v;
    return (hi < m) ? hi : m;
}

__global__ void trust_begin_kernel(TrustParams p, int32_t k)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 2 && i < p.nV)
        p.xkm1[i] = p.x[i];
    if (i != 0)
        return;
    TrustState& S = *p.state;
    if (k >= 2)
    {
        // ConstructModel: translate so that t_k = 0 and solve Q aQ = (f_{k-2}, f_{k-1}, f_k) with
        // Q's rows (t^2, t, 1); with t_k = 0 its last row gives c = f_k.
        S.tkm2 -= S.tk;
        S.tkm1 -= S.tk;
        S.tk = 0.0;
        double const a = S.tkm2, b = S.tkm1;
        double const r0 = S.fkm2 - S.fk, r1 = S.fkm1 - S.fk;
        double const det = a * a * b - b * b * a; // | a^2 a ; b^2 b |
        S.aQ[0] = (r0 * b - r1 * a) / det;
        S.aQ[1] = (a * a * r1 - b * b * r0) / det;
        S.aQ[2] = S.fk;
    }
    // UpdateIterates (scalars; x_{k-1} is copied above when it is used).
    S.fkm2 = S.fkm1;
    S.fkm1 = S.fk;
    S.tkm2 = S.tkm1;
    S.tkm1 = S.tk;
}

__global__ void trust_step_size_kernel(TrustParams p, int32_t entry)
{
    // |x - x_{k-1}|^2 as double-float sums (exact differences and squares; see dfloat.cuh).
    DFloat acc = {0.f, 0.f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.nV; i += gridDim.x * blockDim.x)
    {
        float4 const a = p.x[i], b = p.xkm1[i];
        acc = df_add(acc, df_sq_diff(a.x, b.x));
        acc = df_add(acc, df_sq_diff(a.y, b.y));
        acc = df_add(acc, df_sq_diff(a.z, b.z));
    }
    DFloat const sum = df_warp_sum(acc); // all lanes shuffle; lane 0 converts
    double const w   = (threadIdx.x & 31) == 0 ? df_to_double(sum) : 0.0;
    double total     = 0.0;
    if (!grid_sum_last(p, block_sum_of_warps(w), total) || threadIdx.x != 0)
        return;
    TrustState& S    = *p.state;
    double const dx2 = total;
    // The radius is never smaller than the VBD step, so the stretched step can improve on it.
    if (S.R2 < dx2 + kTrustZero)
        S.R2 = p.tau * p.tau * dx2;
    double const lower = 1.0, upper = sqrt(S.R2 / dx2);
    double const t     = clamp_std(model_optimal_step(S.aQ), lower, upper);
    S.t                = t;
    S.upper            = upper;
    S.tryStep          = !(fabs(t - lower) < kTrustZero);
    S.accepted         = 0;
    S.rollback         = 0;
    S.needObjective    = 0;
    if (!S.tryStep)
    {
        // Rejected without a try: shrink the radius, keep the VBD iterate.
        S.R2 /= p.tau * p.tau;
        S.needObjective = 1;
        S.tk            = S.tkm1 + 1.0;
    }
    double* L = p.log + size_t(kTrustLogFields) * size_t(entry);
    L[0]      = t;
    L[1]      = __longlong_as_double(0x7ff8000000000000ll); // NaN: no ratio unless a step is tried
    L[2]      = S.R2;
    L[3]      = S.tryStep ? 1.0 : 0.0;
}

__global__ void trust_apply_kernel(TrustParams p, bool rollback)
{
    TrustState const& S = *p.state;
    if (!(rollback ? S.rollback : S.tryStep))
        return;
    double const t = S.t;
    int const i    = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.nV)
        return;
    float4 const a = p.x[i], b = p.xkm1[i];
    double const s = rollback ? 1.0 / t : t;
    float4 const u = make_float4(float(double(b.x) + s * (double(a.x) - b.x)), float(double(b.y) + s * (double(a.y) - b.y)),
                                 float(double(b.z) + s * (double(a.z) - b.z)), a.w);
    p.x[i] = u;
    if (p.xh)
        p.xh[i] = u;
}

// Contact energy of active vertex av[q] (TrustRegionIntegrator.cu:310-350): the area-scaled
// penalty over its listed triangles and vertex_triangle_contact's energy for each, at the current
// positions against those at t.
__device__ DFloat contact_energy(TrustParams const& p, int q)
{
    DFloat e = {0.f, 0.f};
    int const i = p.cV[p.av[q]];
    float sumfa = 0.f;
    int32_t f[8];
    for (int c = 0; c < 8; ++c)
    {
        f[c] = p.fc[i * 8 + c];
        if (f[c] >= 0)
            sumfa += p.FA[f[c]];
    }
    if (!(sumfa > 0.f))
        return e;
    float const kC     = p.XVA[i] * p.muC / sumfa;
    float4 const xti4  = p.xt[i], xi4 = p.x[i];
    float const xti[3] = {xti4.x, xti4.y, xti4.z}, xi[3] = {xi4.x, xi4.y, xi4.z};
    for (int c = 0; c < 8; ++c)
    {
        if (f[c] < 0)
            continue;
        int4 const t   = p.cF[f[c]];
        int const v[3] = {t.x, t.y, t.z};
        float xtf[3][3], xf[3][3];
        for (int k = 0; k < 3; ++k)
        {
            float4 const a = p.xt[v[k]], b = p.x[v[k]];
            xtf[k][0] = a.x, xtf[k][1] = a.y, xtf[k][2] = a.z;
            xf[k][0] = b.x, xf[k][1] = b.y, xf[k][2] = b.z;
        }
        float g[3] = {0.f, 0.f, 0.f}, H[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        e = df_add(e, vertex_triangle_contact(xti, xi, xtf, xf, p.h, kC * p.FA[f[c]], p.muF, p.epsv, FLT_EPSILON, g, H));
    }
    return e;
}

__global__ void trust_objective_kernel(TrustParams p, TrustObjectivePhase phase, int32_t k, int32_t entry)
{
    TrustState& S = *p.state;
    if ((phase == kTrustTrial && !S.tryStep) || (phase == kTrustFinal && !S.needObjective))
        return;
    // FP32 terms (energy.cuh objective_parts) summed as double-float values: the inertial and
    // contact terms in accV, the elastic terms in accT (scaled by dt^2 once per warp, in FP64).
    DFloat accV = {0.f, 0.f}, accT = {0.f, 0.f};
    int const n = p.energy.nV > p.energy.nT ? p.energy.nV : p.energy.nT;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    {
        float kin, elas;
        objective_parts(p.energy, j, kin, elas);
        accV = df_add(accV, kin);
        accT = df_add(accT, elas);
    }
    if (p.nActive)
    {
        int const na = *p.nActive;
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < na; q += gridDim.x * blockDim.x)
            accV = df_add(accV, contact_energy(p, q));
    }
    DFloat const sv = df_warp_sum(accV), st = df_warp_sum(accT); // all lanes shuffle; lane 0 converts
    double w        = (threadIdx.x & 31) == 0 ? df_to_double(sv) + p.energy.dt2 * df_to_double(st) : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        w += p.energy.dt2 * p.energy.restEnergy;
    double f = 0.0;
    if (!grid_sum_last(p, block_sum_of_warps(w), f) || threadIdx.x != 0)
        return;
    switch (phase)
    {
        case kTrustInitial:
            S.fk = f;
            S.fkm1 = S.fkm2 = 0.0;
            S.tk            = -1.0;
            S.tkm1 = S.tkm2 = 0.0;
            S.R2            = 0.0;
            break;
        case kTrustPlain:
        {
            S.fk      = f;
            S.tk      = double(k);
            double* L = p.log + size_t(kTrustLogFields) * size_t(entry);
            L[0]      = 0.0;
            L[1]      = __longlong_as_double(0x7ff8000000000000ll);
            L[2]      = S.R2;
            L[3]      = 0.0;
            break;
        }
        case kTrustTrial:
        {
            S.fk               = f;
            double const t     = S.t;
            double const mNext = S.aQ[0] * t * t + S.aQ[1] * t + S.aQ[2];
            // m(0) = f_{k-1}: the predicted decrease against the actual one.
            double const rho = (S.fkm1 - f) / (S.fkm1 - mNext);
            S.accepted       = rho > p.eta;
            if (S.accepted)
            {
                if ((S.upper - t) < kTrustZero)
                    S.R2 *= p.tau * p.tau;
                S.tk = t;
            }
            else
            {
                S.R2 /= p.tau * p.tau;
                S.rollback      = 1;
                S.needObjective = 1;
                S.tk            = S.tkm1 + 1.0;
            }
            double* L = p.log + size_t(kTrustLogFields) * size_t(entry);
            L[1]      = rho;
            L[2]      = S.R2;
            L[3]      = S.accepted ? 3.0 : 1.0;
            break;
        }
        case kTrustFinal: S.fk = f; break;
    }
}

} // namespace

cudaError_t launch_trust_begin(TrustParams const& p, int32_t k, cudaStream_t s)
{
    int const g = k >= 2 ? int((int64_t(p.nV) + kTrustBlock - 1) / kTrustBlock) : 1;
    trust_begin_kernel<<<g < 1 ? 1 : g, kTrustBlock, 0, s>>>(p, k);
    return cudaGetLastError();
}

cudaError_t launch_trust_step_size(TrustParams const& p, int32_t entry, cudaStream_t s)
{
    trust_step_size_kernel<<<trust_blocks(p.nV), kTrustBlock, 0, s>>>(p, entry);
    return cudaGetLastError();
}

cudaError_t launch_trust_apply(TrustParams const& p, bool rollback, cudaStream_t s)
{
    int const g = int((int64_t(p.nV) + kTrustBlock - 1) / kTrustBlock);
    if (g < 1)
        return cudaSuccess;
    trust_apply_kernel<<<g, kTrustBlock, 0, s>>>(p, rollback);
    return cudaGetLastError();
}

cudaError_t launch_trust_objective(TrustParams const& p, TrustObjectivePhase phase, int32_t k, int32_t entry, cudaStream_t s)
{
    int const n = p.energy.nV > p.energy.nT ? p.energy.nV : p.energy.nT;
    trust_objective_kernel<<<trust_blocks(n), kTrustBlock, 0, s>>>(p, phase, k, entry);
    return cudaGetLastError();
}

} // namespace pbgb
