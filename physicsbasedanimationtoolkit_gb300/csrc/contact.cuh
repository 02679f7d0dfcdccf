// Vertex-triangle contact detection for VBD (reference: pbat::gpu::impl::contact::
// VertexTriangleMixedCcdDcd, gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:51-223 and .cuh).
//
//   initialize(xt, xnext): swept vertex boxes vs a BVH over swept triangle boxes; a vertex that
//       overlaps a triangle of another body becomes active, with the squared diagonal of the joint
//       box as its nearest-neighbour search radius.
//   update(x): refit the triangle BVH to x, then up to kBvhMaxNeighbours nearest triangles of every
//       active vertex (branch and bound, ties within FLT_EPSILON kept) -> per-vertex contact list fc.
//   finalize(x): refit, nearest triangles again; a vertex stays active while it lies behind the
//       plane of its (last reported) nearest triangle.
//
// Differences kept small and on purpose: the search radius of a vertex that overlaps several
// triangles is the largest of their joint-box diagonals (the reference keeps whichever write lands
// last), and active vertices are compacted in vertex order (the reference compacts in Morton order;
// every per-vertex result is independent of that order).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lbvh.cuh"

namespace pbgb {

int constexpr kMaxContacts = 8; // per vertex (reference kMaxCollidingTrianglesPerVertex)

struct ContactMesh
{
    int32_t nV;                      // vertices of the whole system
    int32_t nSurfV;                  // collision vertices
    int32_t nF;                      // collision triangles
    int32_t const* __restrict__ V;   // nSurfV global vertex indices
    int4 const* __restrict__ F;      // nF triangles (global vertex indices, w unused)
    int32_t const* __restrict__ B;   // nV body of each vertex
};

struct ContactState
{
    BvhBuffers bvh;     // over the nF triangle boxes
    float4* tlo;        // nF triangle boxes (unsorted)
    float4* thi;
    float4* vlo;        // nSurfV swept vertex boxes
    float4* vhi;
    uint8_t* active;    // nSurfV
    float* dupper;      // nSurfV nearest-neighbour search radius (squared)
    int32_t* av;        // nSurfV active collision vertices (indices into V)
    int32_t* nActive;   // device counter
    int32_t* nn;        // nSurfV * kMaxContacts nearest triangles (-1 = none)
    int32_t* fc;        // nV * kMaxContacts contact triangles per system vertex (-1 = none)
    int32_t* flags;     // device error bits
};

// xt, xnext: float4 positions of all nV vertices.
cudaError_t contact_initialize(ContactMesh const& M, ContactState const& S, float4 const* xt, float4 const* xnext, float3 wmin, float3 wmax, cudaStream_t s);
cudaError_t contact_update(ContactMesh const& M, ContactState const& S, float4 const* x, cudaStream_t s);
cudaError_t contact_finalize(ContactMesh const& M, ContactState const& S, float4 const* x, cudaStream_t s);
// x = xt + dt v + dt^2 aext for all vertices (the prediction the active set is initialised with).
cudaError_t contact_predict(int32_t n, float4 const* xt, float4 const* v, float4 const* a, float dt, float4* xnext, cudaStream_t s);

} // namespace pbgb
