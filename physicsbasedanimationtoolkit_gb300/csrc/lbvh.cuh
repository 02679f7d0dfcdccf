// Linear BVH over axis-aligned boxes (reference: pbat::gpu::impl::geometry::Bvh,
// gpu/impl/geometry/Bvh.cu:24-229 and Bvh.cuh:205-588; Morton codes gpu/impl/geometry/Morton.cu:23-44
// and geometry/Morton.h:35-80).
//
// Build = Morton codes of the box centres normalised by the scene box, a stable LSD radix sort of
// (code, box index), Karras' radix-tree hierarchy, and bottom-up internal boxes.  Node numbering
// follows the reference: internal nodes 0..n-2 (0 is the root), leaves n-1..2n-2 in sorted order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pbgb {

int constexpr kBvhStack = 64;       // traversal stack capacity (reference kStackSize)
int constexpr kBvhMaxNeighbours = 8; // nearest-neighbour ties kept per query (reference kQueueSize)

// Error bits raised on the device (read back by the host after a query or build).
int constexpr kBvhErrStackOverflow = 1;
int constexpr kBvhErrDepth        = 2;

// Node records: node k (internal 0..n-2, leaf n-1+s for sorted leaf s) is nodes[2k] = (lo.x, lo.y,
// lo.z, c0) and nodes[2k+1] = (hi.x, hi.y, hi.z, c1), c0 and c1 stored as int bits: the children of
// an internal node, and (original box index, -1) for a leaf.  A box and the node's links share one
// 32-byte sector, so a traversal step reads one sector per node.
struct BvhView
{
    int32_t n;                       // leaves
    int32_t const* __restrict__ inds; // n: original box index of sorted leaf s
    int32_t const* __restrict__ child;     // 2(n-1): child[2i], child[2i+1]
    int32_t const* __restrict__ rightmost; // 2(n-1)
    float4 const* __restrict__ nodes;      // 2(2n-1) node records
};

__device__ __forceinline__ float4 node_lo(BvhView const& V, int32_t k)
{
    return V.nodes[2 * size_t(k)];
}
__device__ __forceinline__ float4 node_hi(BvhView const& V, int32_t k)
{
    return V.nodes[2 * size_t(k) + 1];
}
// The link words of a node record: children of an internal node, (box index, -1) of a leaf.
__device__ __forceinline__ int32_t node_link(float4 const& half)
{
    return __float_as_int(half.w);
}

// Work arrays of one BVH (allocated by the owner, sized for `capacity` boxes).
struct BvhBuffers
{
    int32_t capacity;
    uint32_t* codes;    // n   sorted Morton codes
    uint32_t* codesAlt; // n   radix-sort ping-pong
    int32_t* inds;      // n   sorted original indices
    int32_t* indsAlt;   // n
    uint32_t* counts;   // 256 * tiles (radix digit counts / offsets)
    uint32_t* scanTmp;  // block totals of the counter scan (all levels)
    int32_t* child;     // 2(n-1)
    int32_t* parent;    // 2n-1
    int32_t* rightmost; // 2(n-1)
    int32_t* first;     // n-1 lowest sorted leaf of each internal node's range
    int32_t* visits;    // n-1 arrivals counted at each internal node (2 after a build or refit)
    float4* packed;     // 2n  the build's input boxes, (lower, upper) per box in input order
    float4* nodes;      // 2(2n-1) node records (BvhView)
    int32_t* flags;     // device error bits
};

// Number of uint32 digit counters the radix sort needs for n keys.
int64_t radix_counts_size(int32_t n);
// Kernel launches of bvh_build and bvh_refit for n boxes (memsets not counted).
int64_t bvh_build_kernels(int32_t n);
int64_t bvh_refit_kernels(int32_t n);

// Device arrays of a BVH for up to `capacity` boxes (bvh_release frees them; safe on partial
// allocation).
cudaError_t bvh_allocate(BvhBuffers& B, int32_t capacity);
void bvh_release(BvhBuffers& B);

// Full build from unsorted boxes lo/hi (n each) and the scene box (wmin, wmax).
cudaError_t bvh_build(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, float3 wmin, float3 wmax, cudaStream_t s);
// Only the Morton codes + stable sort (codes, inds ascending) — exposed for tests.
cudaError_t bvh_sort(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, float3 wmin, float3 wmax, cudaStream_t s);
// Recompute leaf boxes (gathered through inds) and internal boxes, topology unchanged
// (reference: VertexTriangleMixedCcdDcd::UpdateBvh + Bvh::ConstructBoxes).
cudaError_t bvh_refit(BvhBuffers const& B, int32_t n, float4 const* lo, float4 const* hi, cudaStream_t s);

// Overlapping (query, original box index) pairs, appended at pairs[2k], pairs[2k+1] for k < capacity;
// *count (device) receives the total number found (may exceed capacity).
cudaError_t bvh_overlaps(
    BvhView const& V,
    int32_t nq,
    float4 const* qlo,
    float4 const* qhi,
    int32_t* pairs,
    int64_t capacity,
    unsigned long long* count,
    int32_t* flags,
    cudaStream_t s);

// Self-overlaps of the built boxes (each unordered pair once, from the leaf earlier in Morton
// order); set (nullable, one entry per box) drops pairs within one set.  Pairs beyond capacity are
// counted, not written.
cudaError_t bvh_self_overlaps(
    BvhView const& V,
    int32_t const* set,
    int32_t* pairs,
    int64_t capacity,
    unsigned long long* count,
    int32_t* flags,
    cudaStream_t s);

// Boxes of nS simplices of k (1..4) vertices each: S[k i + a] indexes P.
cudaError_t simplex_boxes(int32_t nS, int32_t k, float4 const* P, int32_t const* S, float4* lo, float4* hi, cudaStream_t s);

// Nearest simplex to each query point (gpu/geometry/Bvh.cu PointTriangleNearestNeighbors /
// PointTetrahedronNearestNeighbors): k = 3 (triangles) or 4 (tetrahedra) vertices per simplex;
// nn[q] = the simplex the reference's callback leaves there (the last of the exact-tie list).
cudaError_t bvh_nearest_simplices(
    BvhView const& V,
    int32_t nq,
    float4 const* X,
    float4 const* P,
    int32_t const* S,
    int32_t k,
    int32_t* nn,
    int32_t* flags,
    cudaStream_t s);

inline BvhView view_of(BvhBuffers const& B, int32_t n)
{
    return BvhView{n, B.inds, B.child, B.rightmost, B.nodes};
}

// Spreads the 10 low bits of v so that bit k lands on bit 3k (shift-or form).  A 30-bit Morton
// code is expand(x) * 4 + expand(y) * 2 + expand(z) (geometry/Morton.h:35-80 of the reference).
__host__ __device__ inline uint32_t expand_bits(uint32_t v)
{
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

} // namespace pbgb
