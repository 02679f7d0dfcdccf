// LBVH kernels (sm_103a).  See lbvh.cuh.
#include "lbvh.cuh"

#include <algorithm>

namespace pbgb {

namespace {

int constexpr kSortThreads = 256;
int constexpr kSortRounds  = 16; // a tile is kSortRounds * kSortThreads consecutive keys
int constexpr kTile        = kSortThreads * kSortRounds;
int constexpr kBuckets     = 256;
int constexpr kWarps       = kSortThreads / 32;
static_assert(kBuckets == kSortThreads, "the scatter scans the tile's digit counts one digit per thread");

inline int tiles_for(int32_t n)
{
    return (n + kTile - 1) / kTile;
}

// Morton code of box i's centre normalised by the scene box.  The arithmetic order of the
// reference (gpu/impl/geometry/Morton.cu:40: (0.5*(b+e) - wmin)/(wmax - wmin)) is kept with
// explicitly rounded operations so that no multiply-add is contracted.
__device__ __forceinline__ float normalised(float b, float e, float lo, float ext)
{
    return __fdiv_rn(__fsub_rn(__fmul_rn(0.5f, __fadd_rn(b, e)), lo), ext);
}

__device__ __forceinline__ uint32_t quantise(float c)
{
    // min(max(c * 1024, 0), 1023), truncated (geometry/Morton.h:73-79).
    float q = __fmul_rn(c, 1024.f);
    q       = fminf(fmaxf(q, 0.f), 1023.f);
    return static_cast<uint32_t>(q);
}

// Also copies each box into one 32-byte record (lower, upper), so that the box pass gathers one
// sector per leaf where it would read two half-used ones from the two input arrays.
__global__ void morton_kernel(int32_t n, float4 const* __restrict__ lo, float4 const* __restrict__ hi, float3 wmin, float3 ext, uint32_t* __restrict__ codes, int32_t* __restrict__ inds, float4* __restrict__ packed)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 const b = lo[i], e = hi[i];
    packed[2 * size_t(i)]     = b;
    packed[2 * size_t(i) + 1] = e;
    uint32_t const x = quantise(normalised(b.x, e.x, wmin.x, ext.x));
    uint32_t const y = quantise(normalised(b.y, e.y, wmin.y, ext.y));
    uint32_t const z = quantise(normalised(b.z, e.z, wmin.z, ext.z));
    codes[i]         = expand_bits(x) * 4u + expand_bits(y) * 2u + expand_bits(z);
    inds[i]          = i;
}

// --- stable LSD radix sort, 8-bit digits ------------------------------------------------------
// Pass = count digits per tile -> exclusive scan (digit-major, so tiles keep their order inside a
// digit) -> scatter with each key's rank inside its tile (radix_scatter_kernel), in which equal
// digits keep their input order, so every pass is stable.

__global__ void radix_count_kernel(uint32_t const* __restrict__ keys, int32_t n, int shift, uint32_t* __restrict__ counts, int tiles)
{
    __shared__ uint32_t hist[kBuckets];
    int const tile = blockIdx.x;
    for (int d = threadIdx.x; d < kBuckets; d += blockDim.x)
        hist[d] = 0;
    __syncthreads();
    int const base = tile * kTile;
    // All of the thread's keys are loaded before the first addition, so the loads overlap.
    uint32_t d[kSortRounds];
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r)
    {
        int const i = base + r * kSortThreads + threadIdx.x;
        d[r]        = i < n ? (keys[i] >> shift) & 0xFFu : uint32_t(kBuckets);
    }
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r)
        if (d[r] < uint32_t(kBuckets))
            atomicAdd(&hist[d[r]], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < kBuckets; d += blockDim.x)
        counts[size_t(d) * tiles + tile] = hist[d];
}

// Exclusive scan of the digit counters, in place.  Each block scans kScanItems consecutive
// counters: loaded coalesced into shared memory (padded one word per 32 so that both the strided
// and the contiguous accesses are free of bank conflicts), kScanPer consecutive counters per
// thread, thread totals scanned with warp shuffles, stored back coalesced; the block's total goes
// to `sums`.  The block totals are scanned the same way (recursively) and added back.
int constexpr kScanThreads = 256;
int constexpr kScanPer     = 8;
int constexpr kScanItems   = kScanThreads * kScanPer;

__device__ __forceinline__ int scan_pad(int i)
{
    return i + (i >> 5);
}

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(uint32_t* __restrict__ a, int64_t total, uint32_t* __restrict__ sums)
{
    __shared__ uint32_t sh[kScanItems + kScanItems / 32];
    __shared__ uint32_t warpTotal[kScanThreads / 32];
    int64_t const base = int64_t(blockIdx.x) * kScanItems;
    int const t        = threadIdx.x;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
    {
        int const i      = t + j * kScanThreads;
        int64_t const g  = base + i;
        sh[scan_pad(i)] = g < total ? a[g] : 0u;
    }
    __syncthreads();
    uint32_t v[kScanPer];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
    {
        v[j] = sh[scan_pad(t * kScanPer + j)];
        sum += v[j];
    }
    int const lane = t & 31, warp = t >> 5;
    uint32_t inc   = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
        uint32_t const y = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off)
            inc += y;
    }
    if (lane == 31)
        warpTotal[warp] = inc;
    __syncthreads();
    uint32_t run = inc - sum;
    for (int w = 0; w < warp; ++w)
        run += warpTotal[w];
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
    {
        sh[scan_pad(t * kScanPer + j)] = run;
        run += v[j];
    }
    if (t == kScanThreads - 1)
        sums[blockIdx.x] = run;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
    {
        int const i     = t + j * kScanThreads;
        int64_t const g = base + i;
        if (g < total)
            a[g] = sh[scan_pad(i)];
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_add_kernel(uint32_t* __restrict__ a, int64_t total, uint32_t const* __restrict__ sums)
{
    int64_t const base = int64_t(blockIdx.x) * kScanItems;
    uint32_t const off = sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanPer; ++j)
    {
        int64_t const g = base + threadIdx.x + j * kScanThreads;
        if (g < total)
            a[g] += off;
    }
}

// Scratch words the scan of `total` counters needs for its block totals (all levels).
int64_t scan_tmp_size(int64_t total)
{
    int64_t words = 0;
    while (total > 1)
    {
        total = (total + kScanItems - 1) / kScanItems;
        words += total;
    }
    return words + 1;
}

cudaError_t exclusive_scan(uint32_t* a, int64_t total, uint32_t* tmp, cudaStream_t s)
{
    int64_t const nb = (total + kScanItems - 1) / kScanItems;
    if (nb <= 0)
        return cudaSuccess;
    scan_blocks_kernel<<<unsigned(nb), kScanThreads, 0, s>>>(a, total, tmp);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || nb == 1)
        return e;
    if ((e = exclusive_scan(tmp, nb, tmp + nb, s)) != cudaSuccess)
        return e;
    scan_add_kernel<<<unsigned(nb), kScanThreads, 0, s>>>(a, total, tmp);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(kSortThreads, 3) radix_scatter_kernel(
    uint32_t const* __restrict__ kin,
    int32_t const* __restrict__ vin,
    uint32_t* __restrict__ kout,
    int32_t* __restrict__ vout,
    int32_t n,
    int shift,
    uint32_t const* __restrict__ offsets,
    int tiles)
{
    // The tile is first ordered by digit in shared memory (stably), then each digit's run is
    // written to its global range, so consecutive threads write consecutive addresses.  Warp w
    // ranks its own kSortRounds * 32 consecutive keys of the tile in one pass (round r, lane l:
    // key w * kSortRounds * 32 + r * 32 + l): a key's rank among its warp's equal digits is the
    // warp's running count of the digit before the round plus its peers in lower lanes; the lowest
    // peer then adds the group to the count.  One block scan over
    // (digit, warp) turns the warps' counts into each warp's first position per digit, so the
    // tile needs three block barriers whatever its rounds.
    __shared__ uint32_t skey[kTile];
    __shared__ int32_t sval[kTile];
    __shared__ uint32_t wcount[kWarps][kBuckets]; // the warp's count per digit, then its first position
    __shared__ uint32_t localStart[kBuckets];
    __shared__ uint32_t warpTotal[kWarps];
    int const tile = blockIdx.x;
    int const t    = threadIdx.x;
    int const lane = t & 31;
    int const warp = t >> 5;
    for (int q = t; q < kWarps * kBuckets; q += blockDim.x)
        (&wcount[0][0])[q] = 0;
    __syncthreads();
    int const base = tile * kTile + warp * (kSortRounds * 32) + lane;
    uint32_t key[kSortRounds];
    uint32_t rank[kSortRounds]; // rank among the warp's equal digits, bits 8..; digit, bits 0..7
    unsigned const lanesBelow = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r)
    {
        int const i = base + r * 32;
        key[r]      = i < n ? kin[i] : 0u;
    }
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r)
    {
        bool const valid     = base + r * 32 < n;
        uint32_t const d     = valid ? (key[r] >> shift) & 0xFFu : uint32_t(kBuckets);
        // Lanes with the same digit: nine ballots, one per bit of d (bit 8 marks the lanes past n);
        // on this GPU they cost less than one __match_any_sync.
        unsigned peers = 0xffffffffu;
#pragma unroll
        for (int bit = 0; bit < 9; ++bit)
        {
            unsigned const m = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
            peers &= ((d >> bit) & 1u) ? m : ~m;
        }
        unsigned const below = __popc(peers & lanesBelow);
        uint32_t const before = valid ? wcount[warp][d] : 0u;
        rank[r]              = ((before + below) << 8) | (d & 0xFFu);
        __syncwarp();
        if (valid && below == 0)
            wcount[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Digit t: the tile's exclusive prefix over digits (kBuckets == kSortThreads), then each warp's
    // first position for the digit.
    {
        uint32_t cw[kWarps];
        uint32_t c = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w)
        {
            cw[w] = wcount[w][t];
            c += cw[w];
        }
        uint32_t inc = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1)
        {
            uint32_t const y = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off)
                inc += y;
        }
        if (lane == 31)
            warpTotal[warp] = inc;
        __syncthreads();
        uint32_t start = inc - c;
        for (int w = 0; w < warp; ++w)
            start += warpTotal[w];
        localStart[t] = start;
#pragma unroll
        for (int w = 0; w < kWarps; ++w)
        {
            wcount[w][t] = start;
            start += cw[w];
        }
    }
    __syncthreads();
    // The values are read only now (coalesced, like the keys), which keeps them out of registers
    // across the ranking.
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r)
    {
        int const i = base + r * 32;
        if (i < n)
        {
            uint32_t const pos = wcount[warp][rank[r] & 0xFFu] + (rank[r] >> 8);
            skey[pos]          = key[r];
            sval[pos]          = vin[i];
        }
    }
    __syncthreads();
    int const first = tile * kTile;
    int const count = n - first < kTile ? n - first : kTile;
    for (int j = t; j < count; j += kSortThreads)
    {
        uint32_t const k = skey[j];
        uint32_t const d = (k >> shift) & 0xFFu;
        uint32_t const g = offsets[size_t(d) * tiles + tile] + (uint32_t(j) - localStart[d]);
        kout[g]          = k;
        vout[g]          = sval[j];
    }
}

// --- Karras hierarchy (gpu/impl/geometry/Bvh.cu:24-114) -------------------------------------------

// The sorted keys (code, index) the binary radix tree is built over.
struct SortedKeys
{
    uint32_t const* __restrict__ code;
    int32_t n;
};

__global__ void karras_kernel(SortedKeys K, int32_t* __restrict__ child, int32_t* __restrict__ parent, int32_t* __restrict__ rightmost, int32_t* __restrict__ first)
{
    int32_t const i = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t const n = K.n;
    if (i >= n - 1)
        return;
    int32_t const leafBegin = n - 1;
    // delta(j): the length of the common prefix of keys i and j, the index bits breaking ties of
    // equal codes, -1 outside [0, n); key i is held in a register (the searches only vary j).
    uint32_t const ci = K.code[i];
    auto delta = [&](int32_t j) -> int {
        if (uint32_t(j) >= uint32_t(n))
            return -1;
        uint32_t const x = ci ^ K.code[j];
        return x ? __clz(x) : 32 + __clz(uint32_t(i) ^ uint32_t(j));
    };
    // Direction of the range and a lower bound on its common prefix.
    int32_t const d    = (delta(i + 1) - delta(i - 1)) > 0 ? 1 : -1;
    int const dmin     = delta(i - d);
    int32_t lmax       = 2;
    while (delta(i + lmax * d) > dmin)
        lmax <<= 1;
    int32_t l = 0;
    do
    {
        lmax >>= 1;
        if (delta(i + (l + lmax) * d) > dmin)
            l += lmax;
    } while (lmax > 1);
    int32_t const j   = i + l * d;
    int const dnode   = delta(j);
    int32_t s         = 0;
    int32_t t         = l;
    do
    {
        t = (t + 1) >> 1;
        if (delta(i + (s + t) * d) > dnode)
            s += t;
    } while (t > 1);
    int32_t const gamma = i + s * d + (d < 0 ? d : 0);
    int32_t const lo    = i < j ? i : j;
    int32_t const hi    = i < j ? j : i;
    int32_t const lc    = lo == gamma ? leafBegin + gamma : gamma;
    int32_t const rc    = hi == gamma + 1 ? leafBegin + gamma + 1 : gamma + 1;
    child[2 * i]         = lc;
    child[2 * i + 1]     = rc;
    parent[lc]           = i;
    parent[rc]           = i;
    rightmost[2 * i]     = leafBegin + gamma;
    rightmost[2 * i + 1] = leafBegin + hi;
    first[i]             = lo;
}

__device__ __forceinline__ float4 fmin4(float4 a, float4 b)
{
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.f);
}
__device__ __forceinline__ float4 fmax4(float4 a, float4 b)
{
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.f);
}

// Atomic add with release semantics at device scope: the caller's earlier stores are visible to
// a thread that reads the counter's new value and then acquires (acquire_fence).
__device__ __forceinline__ int atomic_add_release(int32_t* p, int v)
{
    int old;
    asm volatile("atom.release.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Together with the preceding atomic read of the counter, an acquire: the stores released by the
// thread whose addition was read are visible after it.
__device__ __forceinline__ void acquire_fence()
{
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

// Leaf boxes in sorted order and the bottom-up internal boxes (gpu/impl/geometry/Bvh.cu:175-229).
// Thread s gathers leaf s's box, writes the leaf's record, then climbs: the first thread to reach a
// node stops; the second unites the box it carries in registers with its sibling's record (written
// by the first thread before its counter update) and continues.  Min and max are exact and
// commutative, so the boxes do not depend on which child's thread goes on.
//
// A block owns kBoxLeaves consecutive sorted leaves [L, R].  A node whose leaf range lies inside
// [L, R] has its index inside it too (a Karras node is an end of its range), so its visit counter
// is a shared-memory word and the arrival order needs only block-scope fences; its record lands in
// the block's own window of the node array (the second arrival sets the node's visits entry to 2).
// The first node whose range reaches past [L, R] and all its ancestors use device-scope counters
// (visits) with a releasing add and an acquire by the second arrival, whose sibling record may
// come from another block.  Over both phases a climb takes at most 64 levels; deeper trees raise
// kBvhErrDepth instead of looping on.
// Leaves per block of the box pass: 256 measured faster than 1,024 on 4.19M boxes (0.79 against
// 0.87 ms per build): more blocks in flight overlap one block's leaf gathers with another's climbs.
int constexpr kBoxLeaves = 256;

// Shared memory of boxes_kernel: the block's part of the topology (read once, coalesced), the
// arrival counters, and the boxes of its leaves and of its internal nodes, so that a climb inside
// the block touches global memory only to store the records.
struct BoxesSmem
{
    static int constexpr K = kBoxLeaves;
    float4 leaf[2 * K];    // leaf s - L: lower, upper
    float4 box[2 * K];     // internal node p - L (inside nodes only)
    int2 child[K];         // internal node p - L
    int32_t parent[K];     // internal node p - L
    int32_t leafParent[K]; // leaf s - L
    int32_t first[K];      // internal node p - L: its first and last leaf
    int32_t last[K];
    int32_t arrivals[K];
};

// packed (nullable): the boxes as 32-byte records (lower, upper) in input order, read instead of
// lo and hi.
__global__ void __launch_bounds__(kBoxLeaves, 2048 / kBoxLeaves) boxes_kernel(int32_t n, BvhBuffers B, float4 const* __restrict__ lo, float4 const* __restrict__ hi, float4 const* __restrict__ packed)
{
    int constexpr K = kBoxLeaves;
    __shared__ BoxesSmem S;
    int32_t const L         = int32_t(blockIdx.x) * K;
    int32_t const R         = min(L + K, n) - 1;
    int32_t const t         = int32_t(threadIdx.x);
    int32_t const s         = L + t;
    int32_t const leafBegin = n - 1;
    S.arrivals[t] = 0;
    // Internal nodes with index p in [L, R] (p <= n - 2), leaves s in [L, R].
    if (L + t <= min(R, n - 2))
    {
        int32_t const q = L + t;
        S.child[t]      = reinterpret_cast<int2 const*>(B.child)[q];
        S.parent[t]     = B.parent[q];
        S.first[t]      = B.first[q];
        S.last[t]       = B.rightmost[2 * q + 1] - leafBegin;
    }
    int32_t i = 0;
    float4 bl{}, bh{};
    if (s <= R)
    {
        i  = B.inds[s];
        bl = packed ? packed[2 * size_t(i)] : lo[i];
        bh = packed ? packed[2 * size_t(i) + 1] : hi[i];
        S.leafParent[t]   = B.parent[leafBegin + s];
        S.leaf[2 * t]     = bl;
        S.leaf[2 * t + 1] = bh;
    }
    __syncthreads();
    if (s > R)
        return;
    int32_t node                  = leafBegin + s;
    B.nodes[2 * size_t(node)]     = make_float4(bl.x, bl.y, bl.z, __int_as_float(i));
    B.nodes[2 * size_t(node) + 1] = make_float4(bh.x, bh.y, bh.z, __int_as_float(-1));
    int32_t p = S.leafParent[t];
    int k     = 0;
    // Inside the block: a node p in [L, R] whose leaves are all in [L, R].
    for (; k < 64 && p >= 0; ++k)
    {
        if (p < L || p > R || S.first[p - L] < L || S.last[p - L] > R)
            break;
        __threadfence_block(); // this node's shared box before the arrival
        if (atomicAdd(&S.arrivals[p - L], 1) == 0)
            return;
        __threadfence_block(); // the sibling's after its arrival
        int2 const c      = S.child[p - L];
        int32_t const sib = c.x == node ? c.y : c.x;
        float4 sl, sh;
        if (sib >= leafBegin)
        {
            sl = S.leaf[2 * (sib - leafBegin - L)];
            sh = S.leaf[2 * (sib - leafBegin - L) + 1];
        }
        else
        {
            sl = S.box[2 * (sib - L)];
            sh = S.box[2 * (sib - L) + 1];
        }
        bl                         = fmin4(bl, sl);
        bh                         = fmax4(bh, sh);
        S.box[2 * (p - L)]         = bl;
        S.box[2 * (p - L) + 1]     = bh;
        B.nodes[2 * size_t(p)]     = make_float4(bl.x, bl.y, bl.z, __int_as_float(c.x));
        B.nodes[2 * size_t(p) + 1] = make_float4(bh.x, bh.y, bh.z, __int_as_float(c.y));
        B.visits[p]                = 2; // the second arrival (crossing nodes count in visits itself)
        node = p;
        p    = S.parent[p - L];
    }
    // Across blocks.
    for (; k < 64 && p >= 0; ++k)
    {
        if (atomic_add_release(&B.visits[p], 1) == 0)
            return;
        acquire_fence();
        int2 const c      = __ldcg(reinterpret_cast<int2 const*>(B.child) + p);
        int32_t const sib = c.x == node ? c.y : c.x;
        float4 const sl   = __ldcg(&B.nodes[2 * size_t(sib)]);
        float4 const sh   = __ldcg(&B.nodes[2 * size_t(sib) + 1]);
        bl                = fmin4(bl, sl);
        bh                = fmax4(bh, sh);
        __stcg(&B.nodes[2 * size_t(p)], make_float4(bl.x, bl.y, bl.z, __int_as_float(c.x)));
        __stcg(&B.nodes[2 * size_t(p) + 1], make_float4(bh.x, bh.y, bh.z, __int_as_float(c.y)));
        node = p;
        p    = B.parent[p];
    }
    if (k == 64 && p >= 0)
        atomicOr(B.flags, kBvhErrDepth);
}

__device__ __forceinline__ bool boxes_overlap(float4 const& l1, float4 const& u1, float4 const& l2, float4 const& u2)
{
    // Closed intervals on every axis (geometry/OverlapQueries.h:608-616).
    return l1.x <= u2.x && l1.y <= u2.y && l1.z <= u2.z && l2.x <= u1.x && l2.y <= u1.y && l2.z <= u1.z;
}

// Query boxes against the tree (gpu/impl/geometry/Bvh.cuh:282-345 with the overlap predicate of
// Bvh.cuh:476-588): depth-first from the root with a bounded stack.
__global__ void overlaps_kernel(BvhView V, int32_t nq, float4 const* __restrict__ qlo, float4 const* __restrict__ qhi, int32_t* __restrict__ pairs, int64_t capacity, unsigned long long* __restrict__ count, int32_t* __restrict__ flags)
{
    int const q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq || V.n < 1)
        return;
    float4 const L = qlo[q], U = qhi[q];
    int32_t const leafBegin = V.n - 1;
    int32_t stack[kBvhStack];
    int top      = 0;
    stack[top++] = 0;
    while (top > 0)
    {
        int32_t const node = stack[--top];
        float4 const nl    = node_lo(V, node);
        float4 const nh    = node_hi(V, node);
        if (!boxes_overlap(L, U, nl, nh))
            continue;
        if (node >= leafBegin)
        {
            unsigned long long const slot = atomicAdd(count, 1ull);
            if (slot < (unsigned long long)capacity)
            {
                pairs[2 * slot]     = q;
                pairs[2 * slot + 1] = node_link(nl);
            }
        }
        else
        {
            if (top + 2 > kBvhStack)
            {
                atomicOr(flags, kBvhErrStackOverflow);
                return;
            }
            stack[top++] = node_link(nl);
            stack[top++] = node_link(nh);
        }
    }
}

// Self-overlaps of the built leaves (gpu/impl/geometry/Bvh.cuh:206-281): leaf s walks the tree
// from the root and only descends into subtrees whose rightmost leaf lies after its own, so each
// unordered pair is met once, from the leaf earlier in Morton order, and reported as (its box,
// the other box).  With set != nullptr, pairs of boxes in the same set are dropped
// (gpu/geometry/Bvh.cu:91-121).
__global__ void self_overlaps_kernel(BvhView V, int32_t const* __restrict__ set, int32_t* __restrict__ pairs, int64_t capacity, unsigned long long* __restrict__ count, int32_t* __restrict__ flags)
{
    int const s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= V.n || V.n < 2)
        return;
    int32_t const leafBegin = V.n - 1;
    int32_t const leaf      = leafBegin + s;
    float4 const L = node_lo(V, leaf), U = node_hi(V, leaf);
    int32_t const bi = node_link(L);
    int32_t stack[kBvhStack];
    int top      = 0;
    stack[top++] = 0;
    while (top > 0)
    {
        int32_t const node = stack[--top];
#pragma unroll
        for (int c = 0; c < 2; ++c)
        {
            int32_t const ch = V.child[2 * node + c];
            if (V.rightmost[2 * node + c] <= leaf)
                continue;
            bool const isLeaf = ch >= leafBegin;
            float4 const cl   = node_lo(V, ch);
            float4 const cu   = node_hi(V, ch);
            if (!boxes_overlap(L, U, cl, cu))
                continue;
            if (isLeaf)
            {
                int32_t const bj = node_link(cl);
                if (set && set[bi] == set[bj])
                    continue;
                unsigned long long const slot = atomicAdd(count, 1ull);
                if (slot < (unsigned long long)capacity)
                {
                    pairs[2 * slot]     = bi;
                    pairs[2 * slot + 1] = bj;
                }
            }
            else
            {
                if (top + 1 > kBvhStack)
                {
                    atomicOr(flags, kBvhErrStackOverflow);
                    return;
                }
                stack[top++] = ch;
            }
        }
    }
}

// Boxes of simplices with k vertices each (gpu/impl/geometry/Aabb.cuh Construct): component-wise
// minimum and maximum of the corners.
__global__ void simplex_boxes_kernel(int32_t nS, int32_t k, float4 const* __restrict__ P, int32_t const* __restrict__ S, float4* __restrict__ lo, float4* __restrict__ hi)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nS)
        return;
    float4 l = P[S[size_t(i) * k]], u = l;
    for (int a = 1; a < k; ++a)
    {
        float4 const q = P[S[size_t(i) * k + a]];
        l              = make_float4(fminf(l.x, q.x), fminf(l.y, q.y), fminf(l.z, q.z), 0.f);
        u              = make_float4(fmaxf(u.x, q.x), fmaxf(u.y, q.y), fmaxf(u.z, q.z), 0.f);
    }
    lo[i] = make_float4(l.x, l.y, l.z, 0.f);
    hi[i] = make_float4(u.x, u.y, u.z, 0.f);
}

inline int blocks(int64_t n, int b)
{
    return int((n + b - 1) / b);
}

cudaError_t sort_impl(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, float3 wmin, float3 wmax, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    float3 const ext = make_float3(wmax.x - wmin.x, wmax.y - wmin.y, wmax.z - wmin.z);
    morton_kernel<<<blocks(n, 256), 256, 0, s>>>(n, lo, hi, wmin, ext, B.codes, B.inds, B.packed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    int const tiles     = tiles_for(n);
    int64_t const total = int64_t(kBuckets) * tiles;
    uint32_t* kin       = B.codes;
    uint32_t* kout      = B.codesAlt;
    int32_t* vin        = B.inds;
    int32_t* vout       = B.indsAlt;
    for (int shift = 0; shift < 32; shift += 8)
    {
        radix_count_kernel<<<tiles, kSortThreads, 0, s>>>(kin, n, shift, B.counts, tiles);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        if ((e = exclusive_scan(B.counts, total, B.scanTmp, s)) != cudaSuccess)
            return e;
        radix_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, shift, B.counts, tiles);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        uint32_t* tk = kin;
        kin          = kout;
        kout         = tk;
        int32_t* tv  = vin;
        vin          = vout;
        vout         = tv;
    }
    // Four passes: the sorted keys end in B.codes / B.inds again.
    return cudaSuccess;
}

cudaError_t boxes_impl(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, float4 const* packed, cudaStream_t s)
{
    if (n < 1)
        return cudaSuccess;
    if (n > 1)
    {
        cudaError_t const e = cudaMemsetAsync(B.visits, 0, sizeof(int32_t) * size_t(n - 1), s);
        if (e != cudaSuccess)
            return e;
    }
    boxes_kernel<<<blocks(n, kBoxLeaves), kBoxLeaves, 0, s>>>(n, B, lo, hi, packed);
    return cudaGetLastError();
}

} // namespace

int64_t bvh_build_kernels(int32_t n)
{
    if (n <= 0)
        return 0;
    // Kernels of exclusive_scan over `total` counters: one block scan per level, one add per
    // level above the last.
    auto scan = [](int64_t total) {
        int64_t k = 0;
        for (;;)
        {
            int64_t const nb = (total + kScanItems - 1) / kScanItems;
            if (nb <= 0)
                return k;
            ++k;
            if (nb == 1)
                return k;
            ++k;
            total = nb;
        }
    };
    // Morton, 4 x (count, scan, scatter), Karras (two or more boxes), boxes.
    return 1 + 4 * (2 + scan(radix_counts_size(n))) + (n > 1 ? 1 : 0) + 1;
}

int64_t bvh_refit_kernels(int32_t n)
{
    return n > 0 ? 1 : 0;
}

int64_t radix_counts_size(int32_t n)
{
    return int64_t(kBuckets) * tiles_for(n > 0 ? n : 1);
}

cudaError_t bvh_allocate(BvhBuffers& B, int32_t capacity)
{
    B          = BvhBuffers{};
    B.capacity = capacity;
    size_t const n  = size_t(capacity > 0 ? capacity : 1);
    size_t const ni = n > 1 ? n - 1 : 1;
    cudaError_t e   = cudaSuccess;
    auto get = [&](auto*& p, size_t count) {
        if (e == cudaSuccess)
            e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(*p));
    };
    get(B.codes, n);
    get(B.codesAlt, n);
    get(B.inds, n);
    get(B.indsAlt, n);
    get(B.counts, size_t(radix_counts_size(capacity)));
    get(B.scanTmp, size_t(scan_tmp_size(radix_counts_size(capacity))));
    get(B.child, 2 * ni);
    get(B.parent, 2 * n);
    get(B.rightmost, 2 * ni);
    get(B.first, ni);
    get(B.visits, ni);
    get(B.packed, 2 * n);
    get(B.nodes, 2 * (2 * n - 1));
    get(B.flags, 1);
    if (e == cudaSuccess)
        e = cudaMemset(B.flags, 0, sizeof(int32_t));
    return e;
}

void bvh_release(BvhBuffers& B)
{
    void* ptrs[] = {B.codes, B.codesAlt, B.inds, B.indsAlt, B.counts, B.scanTmp, B.child, B.parent,
                    B.rightmost, B.first, B.visits, B.packed, B.nodes, B.flags};
    for (void* p : ptrs)
        if (p)
            cudaFree(p);
    B = BvhBuffers{};
}

cudaError_t bvh_sort(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, float3 wmin, float3 wmax, cudaStream_t s)
{
    return sort_impl(B, n, lo, hi, wmin, wmax, s);
}

cudaError_t bvh_build(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, float3 wmin, float3 wmax, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    cudaError_t e = sort_impl(B, n, lo, hi, wmin, wmax, s);
    if (e != cudaSuccess)
        return e;
    // The root has no parent; every other node is the child of exactly one internal node, whose
    // Karras thread writes its parent.
    if ((e = cudaMemsetAsync(B.parent, 0xFF, sizeof(int32_t), s)) != cudaSuccess)
        return e;
    if (n > 1)
    {
        karras_kernel<<<blocks(n - 1, 256), 256, 0, s>>>(SortedKeys{B.codes, n}, B.child, B.parent, B.rightmost, B.first);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
    }
    return boxes_impl(B, n, lo, hi, B.packed, s);
}

cudaError_t bvh_refit(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    return boxes_impl(B, n, lo, hi, nullptr, s);
}

cudaError_t bvh_overlaps(
    BvhView const& V,
    int32_t nq,
    float4 const* qlo,
    float4 const* qhi,
    int32_t* pairs,
    int64_t capacity,
    unsigned long long* count,
    int32_t* flags,
    cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || nq <= 0)
        return e;
    overlaps_kernel<<<blocks(nq, 128), 128, 0, s>>>(V, nq, qlo, qhi, pairs, capacity, count, flags);
    return cudaGetLastError();
}

cudaError_t bvh_self_overlaps(
    BvhView const& V,
    int32_t const* set,
    int32_t* pairs,
    int64_t capacity,
    unsigned long long* count,
    int32_t* flags,
    cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || V.n < 2)
        return e;
    self_overlaps_kernel<<<blocks(V.n, 128), 128, 0, s>>>(V, set, pairs, capacity, count, flags);
    return cudaGetLastError();
}

cudaError_t simplex_boxes(int32_t nS, int32_t k, float4 const* P, int32_t const* S, float4* lo, float4* hi, cudaStream_t s)
{
    if (nS <= 0)
        return cudaSuccess;
    if (k < 1 || k > 4)
        return cudaErrorInvalidValue;
    simplex_boxes_kernel<<<blocks(nS, 256), 256, 0, s>>>(nS, k, P, S, lo, hi);
    return cudaGetLastError();
}

} // namespace pbgb
