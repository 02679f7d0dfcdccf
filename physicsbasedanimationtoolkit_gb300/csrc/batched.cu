// The persistent batched step (see batched.cuh for the work items and the progress argument).
#include "batched.cuh"
#include "sweep_device.cuh"

#include <climits>

namespace pbgb {

namespace {

__device__ __forceinline__ int32_t load_acquire(int32_t const* q)
{
    int32_t v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(q) : "memory");
    return v;
}

__device__ __forceinline__ void add_release(int32_t* q, int32_t v)
{
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(q), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits until *counter >= need.  Returns false when the wait gave up (time limit, or another
// block's wait gave up before): then flags[1] and the abort flag are set.  At most 2^24 polls in
// any case, so the loop ends even if the timer stood still.
__device__ bool wait_for(BatchedStepParams const& p, int32_t const* counter, int32_t need)
{
    if (load_acquire(counter) >= need)
        return true;
    unsigned long long const t0 = global_ns();
    unsigned sleep              = 32;
    for (int poll = 0; poll < (1 << 24); ++poll)
    {
        if (load_acquire(counter) >= need)
            return true;
        if (*reinterpret_cast<int32_t const volatile*>(p.control + 1) != 0)
            return false;
        if (static_cast<long long>(global_ns() - t0) > p.waitNs)
            break;
        __nanosleep(sleep);
        sleep = sleep < 1024 ? 2 * sleep : sleep;
    }
    atomicOr(p.flags + 1, 1);
    atomicExch(p.control + 1, 1);
    return false;
}

// Colour sweep of solve entries [begin, end) by the whole block: sub-tiles of blockDim / L vertices,
// each staged and solved like staged_sweep_kernel (the same arithmetic in the same order), with the
// block's positions read through L2.  The incidence loop keeps two incidences' records in flight
// (this one's and the next two's loads overlap its arithmetic): the batch's incidence records
// stream from DRAM, and one record ahead per lane left too few bytes in flight per SM.  (Loading
// the records evict-first, ld.global.cs, doubled the DRAM reads of a 256-mesh step: a record's
// sector left L2 before the neighbouring lanes had read their parts of it.)
template <int L, bool CHEB>
__device__ __forceinline__ void sweep_tile(SweepParams const& p, int begin, int end, float4* slab)
{
    int const per  = int(blockDim.x) / L;
    int const lane = int(threadIdx.x) & (L - 1);
    for (int f = begin; f < end; f += per)
    {
        int const s      = f + int(threadIdx.x) / L;
        bool const valid = s < end;
        int const nb0    = __ldg(p.nbrPtr + f);
        VertexBlock<float> b;
        zero(b);
        int i       = 0;
        float xi[3] = {0.f, 0.f, 0.f};
        int k = 0, k1 = 0, n0 = 0, n1 = 0, base = 0;
        uint2 q0 = make_uint2(0u, 0u), q1 = q0;
        float4 st0 = make_float4(0.f, 0.f, 0.f, 0.f), st1 = st0;
        if (valid)
        {
            i    = __ldg(p.solve + s);
            n0   = __ldg(p.nbrPtr + s);
            n1   = __ldg(p.nbrPtr + s + 1);
            base = n0 - nb0;
            k1   = __ldg(p.incPtr + s + 1);
            k    = __ldg(p.incPtr + s) + lane;
            if (k < k1)
            {
                q0  = __ldg(p.incPack + k);
                st0 = __ldg(p.stiff + k);
            }
            if (k + L < k1)
            {
                q1  = __ldg(p.incPack + k + L);
                st1 = __ldg(p.stiff + k + L);
            }
            load3(Mem<true>::ld((CHEB ? p.hprev : p.x) + i), xi);
            for (int j = n0 + lane; j < n1; j += L)
            {
                uint32_t const a  = __ldg(p.nbr + j);
                float4 const* src = p.x;
                if (CHEB && !(a >> 31))
                    src = p.hprev;
                slab[base + j - n0] = Mem<true>::ld(src + (a & kIndexMask));
            }
        }
        __syncwarp();
        if (valid)
        {
            for (; k < k1; k += L)
            {
                uint2 q2   = make_uint2(0u, 0u);
                float4 st2 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k + 2 * L < k1)
                {
                    q2  = __ldg(p.incPack + k + 2 * L);
                    st2 = __ldg(p.stiff + k + 2 * L);
                }
                float d[3][3];
#pragma unroll
                for (int m = 0; m < 3; ++m)
                {
                    float4 const xa = slab[base + int((q0.x >> (8 * m)) & 0xFFu)];
                    d[m][0] = xa.x - xi[0];
                    d[m][1] = xa.y - xi[1];
                    d[m][2] = xa.z - xi[2];
                }
                accumulate_incidence(b, d, st0.x, st0.y, st0.z, __uint_as_float(q0.y), st0.w);
                q0  = q1;
                st0 = st1;
                q1  = q2;
                st1 = st2;
            }
        }
        finish_vertex<L, CHEB, false, false, true>(p, b, valid, lane, i, s, xi);
        if (f + per < end)
            __syncthreads(); // the next sub-tile reuses the slab
    }
}

template <int L, bool CHEB>
__global__ void __launch_bounds__(256, 4) batched_step_kernel(BatchedStepParams p)
{
    extern __shared__ float4 slab[];
    __shared__ int32_t sItem;
    __shared__ int32_t sSkip;
    int32_t next = 0;
    if (threadIdx.x == 0)
        next = atomicAdd(p.control, 1);
    for (;;)
    {
        if (threadIdx.x == 0)
        {
            int32_t const it = next;
            sItem            = it;
            sSkip            = 0;
            if (it < p.nItems)
            {
                next            = atomicAdd(p.control, 1); // taken now, used after this item
                int4 const a    = __ldg(&p.items[it].a);
                int32_t const n = it == p.poison ? INT_MAX : __ldg(&p.items[it].b.x);
                if (!wait_for(p, p.done + a.x, n))
                    sSkip = 1;
            }
        }
        __syncthreads();
        int32_t const it = sItem;
        if (it >= p.nItems)
            break;
        int4 const a = __ldg(&p.items[it].a);
        if (!sSkip)
        {
            int const kind = a.y & 3;
            if (kind == kBatchSweep)
            {
                SweepParams q = p.sweep;
                if constexpr (CHEB)
                {
                    int const kk = a.y >> 2;
                    q.k          = kk;
                    q.omega      = __ldg(p.omega + kk);
                    q.hprev      = (kk + 1) & 1 ? p.H1 : p.H0;
                    q.hcur       = kk & 1 ? p.H1 : p.H0;
                }
                sweep_tile<L, CHEB>(q, a.z, a.w, slab);
            }
            else if (kind == kBatchBegin)
            {
                for (int v = a.z + int(threadIdx.x); v < a.w; v += int(blockDim.x))
                    begin_substep_vertex<true>(p.sub, v);
            }
            else
            {
                for (int v = a.z + int(threadIdx.x); v < a.w; v += int(blockDim.x))
                    end_substep_vertex<true>(p.sub, v);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            __threadfence();
            add_release(p.done + a.x, 1);
        }
    }
}

template <int L, bool CHEB>
cudaError_t launch_l(BatchedStepParams const& p, int block, int grid, size_t smem, cudaStream_t s)
{
    batched_step_kernel<L, CHEB><<<grid, block, smem, s>>>(p);
    return cudaGetLastError();
}

template <bool CHEB>
cudaError_t launch_c(BatchedStepParams const& p, int lanes, int block, int grid, size_t smem, cudaStream_t s)
{
    switch (lanes)
    {
        case 1: return launch_l<1, CHEB>(p, block, grid, smem, s);
        case 2: return launch_l<2, CHEB>(p, block, grid, smem, s);
        case 4: return launch_l<4, CHEB>(p, block, grid, smem, s);
        case 8: return launch_l<8, CHEB>(p, block, grid, smem, s);
        case 16: return launch_l<16, CHEB>(p, block, grid, smem, s);
        case 32: return launch_l<32, CHEB>(p, block, grid, smem, s);
        default: return cudaErrorInvalidValue;
    }
}

template <bool CHEB>
void const* kernel_of(int lanes)
{
    switch (lanes)
    {
        case 1: return reinterpret_cast<void const*>(batched_step_kernel<1, CHEB>);
        case 2: return reinterpret_cast<void const*>(batched_step_kernel<2, CHEB>);
        case 4: return reinterpret_cast<void const*>(batched_step_kernel<4, CHEB>);
        case 8: return reinterpret_cast<void const*>(batched_step_kernel<8, CHEB>);
        case 16: return reinterpret_cast<void const*>(batched_step_kernel<16, CHEB>);
        case 32: return reinterpret_cast<void const*>(batched_step_kernel<32, CHEB>);
        default: return nullptr;
    }
}

} // namespace

cudaError_t launch_batched_step(BatchedStepParams const& p, int lanes, int block, int grid, size_t smem, bool chebyshev, cudaStream_t s)
{
    if (p.nItems <= 0)
        return cudaSuccess;
    if (grid < 1 || block < 32 || block > 256 || block % lanes != 0 || smem > kStagedMaxBytes || !p.items ||
        !p.control || !p.done || !p.flags || !p.sweep.stiff || !p.sweep.incPack || !p.sweep.nbrPtr || (chebyshev && (!p.H0 || !p.H1 || !p.omega)))
        return cudaErrorInvalidValue;
    return chebyshev ? launch_c<true>(p, lanes, block, grid, smem, s) : launch_c<false>(p, lanes, block, grid, smem, s);
}

int batched_step_blocks_per_sm(int lanes, int block, size_t smem, bool chebyshev)
{
    void const* k = chebyshev ? kernel_of<true>(lanes) : kernel_of<false>(lanes);
    if (!k)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t prepare_batched_step()
{
    int const lanes[] = {1, 2, 4, 8, 16, 32};
    for (bool cheb : {false, true})
        for (int L : lanes)
        {
            void const* k = cheb ? kernel_of<true>(L) : kernel_of<false>(L);
            cudaError_t const e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStagedMaxBytes));
            if (e != cudaSuccess)
                return e;
        }
    return cudaSuccess;
}

} // namespace pbgb
