// Vertex-triangle contact detection kernels (sm_103a).  See contact.cuh.
#include "contact.cuh"

#include <cfloat>

namespace pbgb {

namespace {

__device__ __forceinline__ float3 f3(float4 const& v)
{
    return make_float3(v.x, v.y, v.z);
}
__device__ __forceinline__ float3 sub(float3 a, float3 b)
{
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float dot(float3 a, float3 b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ float3 cross(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 axpy(float s, float3 a, float3 b)
{
    return make_float3(s * a.x + b.x, s * a.y + b.y, s * a.z + b.z);
}

// Squared distance from p to triangle abc: closest point by Voronoi regions of the triangle
// (Ericson, Real-Time Collision Detection, section 5.1.5), the method the reference's
// geometry::DistanceQueries::PointTriangle uses.
__device__ float point_triangle_sqdist(float3 p, float3 a, float3 b, float3 c)
{
    float3 const ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
    float const d1 = dot(ab, ap), d2 = dot(ac, ap);
    float3 q;
    if (d1 <= 0.f && d2 <= 0.f)
        q = a;
    else
    {
        float3 const bp = sub(p, b);
        float const d3 = dot(ab, bp), d4 = dot(ac, bp);
        if (d3 >= 0.f && d4 <= d3)
            q = b;
        else
        {
            float const vc = d1 * d4 - d3 * d2;
            if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f)
                q = axpy(d1 / (d1 - d3), ab, a);
            else
            {
                float3 const cp = sub(p, c);
                float const d5 = dot(ab, cp), d6 = dot(ac, cp);
                if (d6 >= 0.f && d5 <= d6)
                    q = c;
                else
                {
                    float const vb = d5 * d2 - d1 * d6;
                    if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f)
                        q = axpy(d2 / (d2 - d6), ac, a);
                    else
                    {
                        float const va = d3 * d6 - d5 * d4;
                        if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f)
                            q = axpy((d4 - d3) / ((d4 - d3) + (d5 - d6)), sub(c, b), b);
                        else
                        {
                            float const den = 1.f / (va + vb + vc);
                            float const v = vb * den, w = vc * den;
                            q = make_float3(a.x + ab.x * v + ac.x * w, a.y + ab.y * v + ac.y * w,
                                            a.z + ab.z * v + ac.z * w);
                        }
                    }
                }
            }
        }
    }
    float3 const d = sub(p, q);
    return dot(d, d);
}

// Squared distance from p to a closed box (0 inside).
__device__ __forceinline__ float point_box_sqdist(float3 p, float4 const& lo, float4 const& hi)
{
    float const dx = p.x < lo.x ? lo.x - p.x : (p.x > hi.x ? p.x - hi.x : 0.f);
    float const dy = p.y < lo.y ? lo.y - p.y : (p.y > hi.y ? p.y - hi.y : 0.f);
    float const dz = p.z < lo.z ? lo.z - p.z : (p.z > hi.z ? p.z - hi.z : 0.f);
    return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ bool boxes_overlap(float4 const& l1, float4 const& u1, float4 const& l2, float4 const& u2)
{
    return l1.x <= u2.x && l1.y <= u2.y && l1.z <= u2.z && l2.x <= u1.x && l2.y <= u1.y && l2.z <= u1.z;
}

__global__ void predict_kernel(int32_t n, float4 const* __restrict__ xt, float4 const* __restrict__ v, float4 const* __restrict__ a, float dt, float4* __restrict__ xn)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 const x0 = xt[i], v0 = v[i], a0 = a[i];
    float const dt2 = dt * dt;
    xn[i] = make_float4(x0.x + dt * v0.x + dt2 * a0.x, x0.y + dt * v0.y + dt2 * a0.y, x0.z + dt * v0.z + dt2 * a0.z, 0.f);
}

__global__ void vertex_boxes_kernel(ContactMesh M, float4 const* __restrict__ xt, float4 const* __restrict__ xn, float4* __restrict__ lo, float4* __restrict__ hi)
{
    int const q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M.nSurfV)
        return;
    int const i     = M.V[q];
    float4 const a = xt[i], b = xn[i];
    lo[q] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.f);
    hi[q] = make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.f);
}

// Boxes of the triangles at x (and, when xn is given, swept to xn).
__global__ void triangle_boxes_kernel(ContactMesh M, float4 const* __restrict__ x, float4 const* __restrict__ xn, float4* __restrict__ lo, float4* __restrict__ hi)
{
    int const f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= M.nF)
        return;
    int4 const t      = M.F[f];
    int const c[3]    = {t.x, t.y, t.z};
    float4 l = x[c[0]], u = l;
    for (int k = 0; k < 3; ++k)
    {
        float4 const p = x[c[k]];
        l = make_float4(fminf(l.x, p.x), fminf(l.y, p.y), fminf(l.z, p.z), 0.f);
        u = make_float4(fmaxf(u.x, p.x), fmaxf(u.y, p.y), fmaxf(u.z, p.z), 0.f);
        if (xn)
        {
            float4 const r = xn[c[k]];
            l = make_float4(fminf(l.x, r.x), fminf(l.y, r.y), fminf(l.z, r.z), 0.f);
            u = make_float4(fmaxf(u.x, r.x), fmaxf(u.y, r.y), fmaxf(u.z, r.z), 0.f);
        }
    }
    lo[f] = make_float4(l.x, l.y, l.z, 0.f);
    hi[f] = make_float4(u.x, u.y, u.z, 0.f);
}

// Squared diagonal of the joint box of vertex i and triangle t over both position sets (the
// reference's nearest-neighbour search radius for the pair).
__device__ __forceinline__ float joint_box_sqdiag(int i, int4 const& t, float4 const* __restrict__ xt, float4 const* __restrict__ xn)
{
    int const c[3] = {t.x, t.y, t.z};
    float4 lo = xt[i], hi = xt[i];
    float4 pts[8];
    pts[0] = xt[i];
    pts[1] = xn[i];
    for (int k = 0; k < 3; ++k)
    {
        pts[2 + k] = xt[c[k]];
        pts[5 + k] = xn[c[k]];
    }
    for (int k = 0; k < 8; ++k)
    {
        lo = make_float4(fminf(lo.x, pts[k].x), fminf(lo.y, pts[k].y), fminf(lo.z, pts[k].z), 0.f);
        hi = make_float4(fmaxf(hi.x, pts[k].x), fmaxf(hi.y, pts[k].y), fmaxf(hi.z, pts[k].z), 0.f);
    }
    float const dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dx + dy * dy + dz * dz;
}

// Swept vertex box vs the swept-triangle BVH (gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:103-
// 136): triangles of another body activate the vertex and bound its search radius.  One thread's
// depth-first traversal (the fallback of initialize_kernel).
__device__ void initialize_serial(ContactMesh const& M, ContactState const& S, BvhView const& T, float4 const* __restrict__ xt, float4 const* __restrict__ xn, int q)
{
    int const i     = M.V[q];
    float4 const L = S.vlo[q], U = S.vhi[q];
    int32_t const leafBegin = T.n - 1;
    int32_t stack[kBvhStack];
    int top      = 0;
    stack[top++] = 0;
    float best   = 0.f;
    bool hit     = false;
    while (top > 0)
    {
        int32_t const node = stack[--top];
        float4 const nl    = node_lo(T, node);
        float4 const nh    = node_hi(T, node);
        if (!boxes_overlap(L, U, nl, nh))
            continue;
        if (node >= leafBegin)
        {
            int4 const t = M.F[node_link(nl)];
            if (M.B[i] == M.B[t.x])
                continue;
            best = fmaxf(best, joint_box_sqdiag(i, t, xt, xn));
            hit  = true;
        }
        else
        {
            if (top + 2 > kBvhStack)
            {
                atomicOr(S.flags, kBvhErrStackOverflow);
                return;
            }
            stack[top++] = node_link(nl);
            stack[top++] = node_link(nh);
        }
    }
    if (hit)
    {
        S.dupper[q] = best;
        S.active[q] = 1;
    }
}

int constexpr kInitWarps    = 4;   // warps (vertices) per block
int constexpr kInitFrontier = 512; // breadth-first frontier capacity per warp

// Warp-cooperative form of the same overlap query, one warp per collision vertex: the levels of
// the hierarchy are expanded breadth first across the lanes (the result, a maximum over the
// overlapping triangles of other bodies, does not depend on the visit order), so a vertex in a
// dense contact patch costs about the tree's depth in dependent loads instead of one thread's
// whole traversal.  A frontier overflow hands the vertex to lane 0's depth-first traversal.
__global__ void __launch_bounds__(32 * kInitWarps) initialize_kernel(ContactMesh M, ContactState S, BvhView T, float4 const* __restrict__ xt, float4 const* __restrict__ xn)
{
    __shared__ int32_t frontier[kInitWarps][2][kInitFrontier];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int const q    = blockIdx.x * kInitWarps + warp;
    if (q >= M.nSurfV || T.n < 1)
        return;
    unsigned const all = 0xffffffffu;
    int const i        = M.V[q];
    int const body     = M.B[i];
    float4 const L = S.vlo[q], U = S.vhi[q];
    int32_t const leafBegin = T.n - 1;
    int cur = 0, nf = 1;
    bool overflow = false;
    float best    = 0.f;
    bool hit      = false;
    if (lane == 0)
        frontier[warp][0][0] = 0;
    __syncwarp();
    while (nf > 0 && !overflow)
    {
        int nn = 0;
        for (int base = 0; base < nf; base += 32)
        {
            int const idx = base + lane;
            int32_t const node = idx < nf ? frontier[warp][cur][idx] : -1;
            bool push = false;
            int32_t a = -1, b = -1;
            if (node >= 0)
            {
                float4 const nl = node_lo(T, node);
                float4 const nh = node_hi(T, node);
                if (boxes_overlap(L, U, nl, nh))
                {
                    if (node < leafBegin)
                    {
                        a    = node_link(nl);
                        b    = node_link(nh);
                        push = true;
                    }
                    else
                    {
                        int4 const t = M.F[node_link(nl)];
                        if (M.B[t.x] != body)
                        {
                            best = fmaxf(best, joint_box_sqdiag(i, t, xt, xn));
                            hit  = true;
                        }
                    }
                }
            }
            unsigned const m = __ballot_sync(all, push);
            int const slot   = nn + 2 * __popc(m & ((1u << lane) - 1u));
            if (push && slot + 1 < kInitFrontier)
            {
                frontier[warp][cur ^ 1][slot]     = a;
                frontier[warp][cur ^ 1][slot + 1] = b;
            }
            nn += 2 * __popc(m);
            if (nn > kInitFrontier)
                overflow = true; // warp-uniform
        }
        __syncwarp();
        cur ^= 1;
        nf = nn;
    }
    if (overflow)
    {
        if (lane == 0)
            initialize_serial(M, S, T, xt, xn, q);
        return;
    }
    for (int off = 16; off > 0; off >>= 1)
        best = fmaxf(best, __shfl_xor_sync(all, best, off));
    bool const any = __any_sync(all, hit);
    if (lane == 0 && any)
    {
        S.dupper[q] = best;
        S.active[q] = 1;
    }
}

__global__ void compact_kernel(int32_t n, uint8_t const* __restrict__ active, int32_t* __restrict__ av, int32_t* __restrict__ count)
{
    int const q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n || !active[q])
        return;
    av[atomicAdd(count, 1)] = q;
}

// Nearest triangles of active vertex av[q] (gpu/impl/geometry/Bvh.cuh:347-474 with the contact
// callbacks of gpu/impl/contact/VertexTriangleMixedCcdDcd.cuh:109-162): the reference runs a
// depth-first branch and bound from the warm-start radius (right child first, so leaves are met in
// decreasing sorted order); triangles within FLT_EPSILON of the best are kept (at most
// kMaxContacts) and a strictly better one restarts the list.  finalize = false writes the list to
// nn, finalize = true sets active[v] from the side of the last listed triangle's plane.
//
// The list is the result of scanning the leaves in that order with the running minimum: a leaf the
// branch and bound prunes lies beyond the running bound and would change nothing.  Two passes give
// the same list with far fewer node visits when the warm-start radius is loose:
//   1. the exact nearest distance d* (closer child first, pruned by the best distance so far);
//   2. the reference-order scan, pruned by min(running bound, d* + 8 FLT_EPSILON + 16 ulp).
// The last restart of the scan has d <= d* + eps (otherwise the d* triangle would restart it
// again) and every triangle listed after it has d <= d* + 2 eps (FP32 rounding of the bounds
// widens each eps to at most an ulp of d), so the leaves pass 2 skips can
// neither restart nor join the final list, and removing them leaves the last restart and
// everything after it unchanged.
__device__ __forceinline__ float node_box_sqdist(BvhView const& T, float3 p, int32_t node)
{
    return point_box_sqdist(p, node_lo(T, node), node_hi(T, node));
}

// Writes the result of a query (see nearest_kernel).
template <bool FINALIZE>
__device__ void nearest_write(ContactMesh const& M, ContactState const& S, float4 const* __restrict__ x, int v, int i,
                              float3 p, int32_t const* list, int count)
{
    if (FINALIZE)
    {
        if (count > 0)
        {
            int4 const t     = M.F[list[count - 1]];
            float3 const a   = f3(x[t.x]);
            float3 const nrm = cross(sub(f3(x[t.y]), a), sub(f3(x[t.z]), a));
            S.active[v]      = dot(sub(p, a), nrm) < 0.f ? 1 : 0;
        }
    }
    else
    {
        for (int k = 0; k < kMaxContacts; ++k)
        {
            int32_t const f            = k < count ? list[k] : -1;
            S.nn[v * kMaxContacts + k] = f;
            S.fc[i * kMaxContacts + k] = f;
        }
    }
}

// One thread's query of active vertex av[q]: the two passes described above.
template <bool FINALIZE>
__device__ void nearest_serial(ContactMesh const& M, ContactState const& S, BvhView const& T, float4 const* __restrict__ x, int q)
{
    int const v = S.av[q];
    int const i = M.V[v];
    float3 const p = f3(x[i]);
    int const body = M.B[i];
    float const eps = FLT_EPSILON;
    float const d0  = S.dupper[v];
    int32_t const leafBegin = T.n - 1;
    int32_t stack[kBvhStack];
    float dist[kBvhStack];
    int top = 0;

    // Pass 1: d* over the triangles of other bodies within the reference's initial bound.
    float best = d0 + eps;
    bool found = false;
    stack[top]  = 0;
    dist[top++] = node_box_sqdist(T, p, 0);
    while (top > 0)
    {
        --top;
        int32_t const node = stack[top];
        if (dist[top] > best)
            continue;
        if (node < leafBegin)
        {
            int32_t const a = node_link(node_lo(T, node)), b = node_link(node_hi(T, node));
            float const da = node_box_sqdist(T, p, a), db = node_box_sqdist(T, p, b);
            if (top + 2 > kBvhStack)
            {
                atomicOr(S.flags, kBvhErrStackOverflow);
                return;
            }
            // Farther child first, so the nearer one is expanded next.
            bool const aFirst = da > db;
            int32_t const n0 = aFirst ? a : b, n1 = aFirst ? b : a;
            float const e0 = aFirst ? da : db, e1 = aFirst ? db : da;
            if (e0 <= best)
                stack[top] = n0, dist[top++] = e0;
            if (e1 <= best)
                stack[top] = n1, dist[top++] = e1;
            continue;
        }
        int4 const t = M.F[node_link(node_lo(T, node))];
        if (M.B[t.x] == body)
            continue;
        float const d = point_triangle_sqdist(p, f3(x[t.x]), f3(x[t.y]), f3(x[t.z]));
        if (d <= best)
        {
            best  = d;
            found = true;
        }
    }

    // Pass 2: the reference-order scan over the leaves that can matter.
    int32_t list[kMaxContacts];
    int count = 0;
    if (found)
    {
        // 2 eps suffices in exact arithmetic; FP32 rounding of dmin +- eps can widen each
        // tolerance to one ulp of dmin, so the cap keeps a relative and an absolute margin.
        float const cap = best * (1.f + 16.f * eps) + 8.f * eps;
        float dmin      = d0;
        top             = 0;
        stack[top++]    = 0;
        while (top > 0)
        {
            int32_t const node = stack[--top];
            float const lo     = dmin - eps;
            float const hi     = dmin + eps;
            float const bound  = fminf(hi, cap);
            float4 const nl    = node_lo(T, node);
            float4 const nh    = node_hi(T, node);
            if (point_box_sqdist(p, nl, nh) > bound)
                continue;
            if (node < leafBegin)
            {
                if (top + 2 > kBvhStack)
                {
                    atomicOr(S.flags, kBvhErrStackOverflow);
                    return;
                }
                stack[top++] = node_link(nl);
                stack[top++] = node_link(nh);
                continue;
            }
            int32_t const f = node_link(nl);
            int4 const t    = M.F[f];
            float const d   = M.B[t.x] == body ? FLT_MAX
                                               : point_triangle_sqdist(p, f3(x[t.x]), f3(x[t.y]), f3(x[t.z]));
            if (d < lo)
            {
                list[0] = f;
                count   = 1;
                dmin    = d;
            }
            else if (d <= hi && count < kMaxContacts)
                list[count++] = f;
        }
    }
    nearest_write<FINALIZE>(M, S, x, v, i, p, list, count);
}

int constexpr kNearestWarps    = 2;    // warps (queries) per block
int constexpr kNearestFrontier = 1024; // breadth-first frontier capacity per warp
int constexpr kNearestCand     = 1024; // candidate leaves per warp

struct NearestSmem
{
    int32_t frontier[2][kNearestFrontier];
    int32_t cand[kNearestCand]; // sorted leaf index
    float candD[kNearestCand];  // its squared distance (FLT_MAX: the vertex's own body)
};

// Warp-cooperative form of the same query, one warp per active vertex.  The traversal is what
// bounds the kernel: a query's loads form one dependent chain per thread, so spreading it over 32
// lanes shortens the longest chain about as many times.
//   1. breadth first, collect every leaf whose box lies within min(dupper + eps, the distance to
//      the vertex's current list plus the margin), with its triangle's squared distance (no
//      other leaf can be listed: see above);
//   2. d* = the warp minimum over other bodies; keep the candidates with d <= d* + margin (see
//      above: no other leaf can restart the scan's final list or join it);
//   3. order them by decreasing leaf index (the reference's visit order) and run its scan.
// A frontier or candidate overflow hands the query to lane 0's serial traversal.
template <bool FINALIZE>
__global__ void __launch_bounds__(32 * kNearestWarps) nearest_kernel(ContactMesh M, ContactState S, BvhView T, float4 const* __restrict__ x)
{
    extern __shared__ unsigned char nearestSmemRaw[];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    NearestSmem& sm = reinterpret_cast<NearestSmem*>(nearestSmemRaw)[warp];
    int const q     = blockIdx.x * kNearestWarps + warp;
    if (q >= *S.nActive || T.n < 1)
        return;
    unsigned const all = 0xffffffffu;
    int const v        = S.av[q];
    int const i        = M.V[v];
    float3 const p     = f3(x[i]);
    int const body     = M.B[i];
    float const eps    = FLT_EPSILON;
    float const d0     = S.dupper[v];
    // Any triangle of another body bounds d* from above; the vertex's current list (from the last
    // update) usually holds the nearest ones, so the collection can stop at that bound plus the
    // margin the scan needs instead of the warm-start radius.
    float U = FLT_MAX;
    if (lane < kMaxContacts)
    {
        int32_t const f = S.fc[i * kMaxContacts + lane];
        if (f >= 0)
        {
            int4 const t = M.F[f];
            if (M.B[t.x] != body)
                U = point_triangle_sqdist(p, f3(x[t.x]), f3(x[t.y]), f3(x[t.z]));
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        U = fminf(U, __shfl_xor_sync(all, U, off));
    float const bound = fminf(d0 + eps, U * (1.f + 16.f * eps) + 8.f * eps);
    int32_t const leafBegin = T.n - 1;

    // 1. Breadth-first collection (every leaf with d <= bound: they include all those with
    //    d <= d* + margin, as U >= d*).
    int cur = 0, nf = 1, nc = 0;
    bool overflow = false;
    if (lane == 0)
        sm.frontier[0][0] = 0;
    __syncwarp();
    while (nf > 0 && !overflow)
    {
        int nn = 0;
        for (int base = 0; base < nf; base += 32)
        {
            int const idx  = base + lane;
            int32_t node   = idx < nf ? sm.frontier[cur][idx] : -1;
            bool pushNode  = false, pushLeaf = false;
            int32_t a = -1, b = -1;
            float d        = FLT_MAX;
            if (node >= 0)
            {
                float4 const nl = node_lo(T, node);
                float4 const nh = node_hi(T, node);
                bool const near = point_box_sqdist(p, nl, nh) <= bound;
                if (node < leafBegin)
                {
                    if (near)
                    {
                        a        = node_link(nl);
                        b        = node_link(nh);
                        pushNode = true;
                    }
                }
                else
                {
                    int32_t const s = node - leafBegin;
                    if (near)
                    {
                        int4 const t = M.F[node_link(nl)];
                        d            = M.B[t.x] == body ? FLT_MAX
                                                        : point_triangle_sqdist(p, f3(x[t.x]), f3(x[t.y]), f3(x[t.z]));
                        pushLeaf = d <= bound;
                        node     = s;
                    }
                }
            }
            unsigned const mNode = __ballot_sync(all, pushNode);
            unsigned const mLeaf = __ballot_sync(all, pushLeaf);
            unsigned const below = (1u << lane) - 1u;
            int const slotN      = nn + 2 * __popc(mNode & below);
            int const slotL      = nc + __popc(mLeaf & below);
            if (pushNode && slotN + 1 < kNearestFrontier)
            {
                sm.frontier[cur ^ 1][slotN]     = a;
                sm.frontier[cur ^ 1][slotN + 1] = b;
            }
            if (pushLeaf && slotL < kNearestCand)
            {
                sm.cand[slotL]  = node;
                sm.candD[slotL] = d;
            }
            nn += 2 * __popc(mNode);
            nc += __popc(mLeaf);
            if (nn > kNearestFrontier || nc > kNearestCand)
                overflow = true; // warp-uniform
        }
        __syncwarp();
        cur ^= 1;
        nf = nn;
    }
    if (overflow)
    {
        if (lane == 0)
            nearest_serial<FINALIZE>(M, S, T, x, q);
        return;
    }

    // 2. d* and the candidates that can matter.
    float dstar = FLT_MAX;
    for (int k = lane; k < nc; k += 32)
        dstar = fminf(dstar, sm.candD[k]);
    for (int off = 16; off > 0; off >>= 1)
        dstar = fminf(dstar, __shfl_xor_sync(all, dstar, off));
    int32_t list[kMaxContacts];
    int count = 0;
    if (dstar <= d0 + eps)
    {
        float const cap = dstar * (1.f + 16.f * eps) + 8.f * eps;
        // Compact the kept candidates to the front (order does not matter yet).
        int kept = 0;
        for (int base = 0; base < nc; base += 32)
        {
            int const k      = base + lane;
            bool const keep  = k < nc && sm.candD[k] <= cap;
            int32_t const s  = keep ? sm.cand[k] : 0;
            float const dk   = keep ? sm.candD[k] : 0.f;
            unsigned const m = __ballot_sync(all, keep);
            __syncwarp();
            if (keep)
            {
                int const slot   = kept + __popc(m & ((1u << lane) - 1u));
                sm.cand[slot]    = s;
                sm.candD[slot]   = dk;
            }
            kept += __popc(m);
            __syncwarp();
        }
        // 3. The reference's scan in decreasing leaf index: repeatedly take the largest remaining.
        float dmin   = d0;
        int32_t last = INT32_MAX;
        for (int r = 0; r < kept; ++r)
        {
            int32_t bestS = -1;
            float bestD   = 0.f;
            for (int k = lane; k < kept; k += 32)
            {
                int32_t const s = sm.cand[k];
                if (s < last && s > bestS)
                {
                    bestS = s;
                    bestD = sm.candD[k];
                }
            }
            for (int off = 16; off > 0; off >>= 1)
            {
                int32_t const os = __shfl_xor_sync(all, bestS, off);
                float const od   = __shfl_xor_sync(all, bestD, off);
                if (os > bestS)
                {
                    bestS = os;
                    bestD = od;
                }
            }
            last           = bestS;
            float const lo = dmin - eps, hi = dmin + eps;
            if (bestD < lo)
            {
                list[0] = T.inds[bestS];
                count   = 1;
                dmin    = bestD;
            }
            else if (bestD <= hi && count < kMaxContacts)
                list[count++] = T.inds[bestS];
        }
    }
    if (lane == 0)
        nearest_write<FINALIZE>(M, S, x, v, i, p, list, count);
}

// Point in closed tetrahedron abcd (geometry/OverlapQueries.h:562-587): outside when strictly on
// the positive side of one of the faces (a, b, d), (b, c, d), (c, a, d), (a, c, b).
__device__ __forceinline__ bool point_in_tet(float3 p, float3 a, float3 b, float3 c, float3 d)
{
    auto outside = [&](float3 u, float3 v, float3 w) { return dot(sub(p, u), cross(sub(v, u), sub(w, u))) > 0.f; };
    return !(outside(a, b, d) || outside(b, c, d) || outside(c, a, d) || outside(a, c, b));
}

// Squared point-tetrahedron distance (geometry/DistanceQueries.h:230-249): 0 inside, else the
// nearest of the four faces.
__device__ __forceinline__ float point_tet_sqdist(float3 p, float3 a, float3 b, float3 c, float3 d)
{
    if (point_in_tet(p, a, b, c, d))
        return 0.f;
    return fminf(fminf(point_triangle_sqdist(p, a, b, d), point_triangle_sqdist(p, b, c, d)),
                 fminf(point_triangle_sqdist(p, c, a, d), point_triangle_sqdist(p, a, c, b)));
}

// Nearest simplex to each query point (gpu/impl/geometry/Bvh.cuh:347-474 with the callbacks of
// gpu/geometry/Bvh.cu:123-260): depth-first branch and bound from the root (children pushed left
// then right, so the right child is visited first), leaves pruned by their box, exact ties (eps 0)
// kept in a list of 8 in visit order; the reference's callback writes every listed simplex in turn,
// so the last one stays.  Squared distances order the candidates as distances do.
template <int K>
__global__ void nearest_simplex_kernel(BvhView V, int32_t nq, float4 const* __restrict__ X, float4 const* __restrict__ P, int32_t const* __restrict__ S, int32_t* __restrict__ nn, int32_t* __restrict__ flags)
{
    int const q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq)
        return;
    if (V.n < 1)
    {
        nn[q] = -1;
        return;
    }
    float3 const x          = f3(X[q]);
    int32_t const leafBegin = V.n - 1;
    int32_t stack[kBvhStack];
    int top      = 0;
    stack[top++] = 0;
    int32_t list[kMaxContacts];
    int count  = 0;
    float dmin = FLT_MAX;
    while (top > 0)
    {
        int32_t const node = stack[--top];
        float4 const nl    = node_lo(V, node);
        float4 const nh    = node_hi(V, node);
        if (point_box_sqdist(x, nl, nh) > dmin)
            continue;
        if (node < leafBegin)
        {
            if (top + 2 > kBvhStack)
            {
                atomicOr(flags, kBvhErrStackOverflow);
                nn[q] = -1;
                return;
            }
            stack[top++] = node_link(nl);
            stack[top++] = node_link(nh);
            continue;
        }
        int32_t const i      = node_link(nl);
        int32_t const* const c = S + size_t(i) * K;
        float const d = K == 3 ? point_triangle_sqdist(x, f3(P[c[0]]), f3(P[c[1]]), f3(P[c[2]]))
                               : point_tet_sqdist(x, f3(P[c[0]]), f3(P[c[1]]), f3(P[c[2]]), f3(P[c[K - 1]]));
        if (d < dmin)
        {
            count     = 0;
            list[count++] = i;
            dmin      = d;
        }
        else if (d <= dmin && count < kMaxContacts)
            list[count++] = i;
    }
    nn[q] = count > 0 ? list[count - 1] : -1;
}

inline int blocks(int64_t n, int b)
{
    return int((n + b - 1) / b);
}

cudaError_t refit(ContactMesh const& M, ContactState const& S, float4 const* x, cudaStream_t s)
{
    triangle_boxes_kernel<<<blocks(M.nF, 256), 256, 0, s>>>(M, x, nullptr, S.tlo, S.thi);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    return bvh_refit(S.bvh, M.nF, S.tlo, S.thi, s);
}

} // namespace

cudaError_t contact_predict(int32_t n, float4 const* xt, float4 const* v, float4 const* a, float dt, float4* xnext, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    predict_kernel<<<blocks(n, 256), 256, 0, s>>>(n, xt, v, a, dt, xnext);
    return cudaGetLastError();
}

cudaError_t contact_initialize(ContactMesh const& M, ContactState const& S, float4 const* xt, float4 const* xnext, float3 wmin, float3 wmax, cudaStream_t s)
{
    if (M.nF <= 0 || M.nSurfV <= 0)
        return cudaSuccess;
    vertex_boxes_kernel<<<blocks(M.nSurfV, 256), 256, 0, s>>>(M, xt, xnext, S.vlo, S.vhi);
    triangle_boxes_kernel<<<blocks(M.nF, 256), 256, 0, s>>>(M, xt, xnext, S.tlo, S.thi);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    if ((e = bvh_build(S.bvh, M.nF, S.tlo, S.thi, wmin, wmax, s)) != cudaSuccess)
        return e;
    initialize_kernel<<<blocks(M.nSurfV, kInitWarps), 32 * kInitWarps, 0, s>>>(M, S, view_of(S.bvh, M.nF), xt, xnext);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(S.nActive, 0, sizeof(int32_t), s)) != cudaSuccess)
        return e;
    compact_kernel<<<blocks(M.nSurfV, 256), 256, 0, s>>>(M.nSurfV, S.active, S.av, S.nActive);
    return cudaGetLastError();
}

cudaError_t contact_update(ContactMesh const& M, ContactState const& S, float4 const* x, cudaStream_t s)
{
    if (M.nF <= 0 || M.nSurfV <= 0)
        return cudaSuccess;
    cudaError_t e = refit(M, S, x, s);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(S.nn, 0xFF, sizeof(int32_t) * size_t(M.nSurfV) * kMaxContacts, s)) != cudaSuccess)
        return e;
    nearest_kernel<false><<<blocks(M.nSurfV, kNearestWarps), 32 * kNearestWarps, sizeof(NearestSmem) * kNearestWarps, s>>>(
        M, S, view_of(S.bvh, M.nF), x);
    return cudaGetLastError();
}

cudaError_t contact_finalize(ContactMesh const& M, ContactState const& S, float4 const* x, cudaStream_t s)
{
    if (M.nF <= 0 || M.nSurfV <= 0)
        return cudaSuccess;
    cudaError_t e = refit(M, S, x, s);
    if (e != cudaSuccess)
        return e;
    nearest_kernel<true><<<blocks(M.nSurfV, kNearestWarps), 32 * kNearestWarps, sizeof(NearestSmem) * kNearestWarps, s>>>(
        M, S, view_of(S.bvh, M.nF), x);
    return cudaGetLastError();
}

cudaError_t bvh_nearest_simplices(
    BvhView const& V,
    int32_t nq,
    float4 const* X,
    float4 const* P,
    int32_t const* S,
    int32_t k,
    int32_t* nn,
    int32_t* flags,
    cudaStream_t s)
{
    if (nq <= 0)
        return cudaSuccess;
    if (k == 3)
        nearest_simplex_kernel<3><<<blocks(nq, 128), 128, 0, s>>>(V, nq, X, P, S, nn, flags);
    else if (k == 4)
        nearest_simplex_kernel<4><<<blocks(nq, 128), 128, 0, s>>>(V, nq, X, P, S, nn, flags);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

} // namespace pbgb
