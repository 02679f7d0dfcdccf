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

// Swept vertex box vs the swept-triangle BVH (gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:103-
// 136): triangles of another body activate the vertex and bound its search radius.
__global__ void initialize_kernel(ContactMesh M, ContactState S, BvhView T, float4 const* __restrict__ xt, float4 const* __restrict__ xn)
{
    int const q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= M.nSurfV || T.n < 1)
        return;
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
        if (node >= leafBegin)
        {
            int32_t const s = node - leafBegin;
            if (!boxes_overlap(L, U, T.llo[s], T.lhi[s]))
                continue;
            int32_t const f = T.inds[s];
            int4 const t    = M.F[f];
            if (M.B[i] == M.B[t.x])
                continue;
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
            float const d2 = dx * dx + dy * dy + dz * dz;
            best           = fmaxf(best, d2);
            hit            = true;
        }
        else if (boxes_overlap(L, U, T.ilo[node], T.ihi[node]))
        {
            if (top + 2 > kBvhStack)
            {
                atomicOr(S.flags, kBvhErrStackOverflow);
                return;
            }
            stack[top++] = T.child[2 * node];
            stack[top++] = T.child[2 * node + 1];
        }
    }
    if (hit)
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
// callbacks of gpu/impl/contact/VertexTriangleMixedCcdDcd.cuh:109-162): depth-first branch and
// bound from the warm-start radius; triangles within FLT_EPSILON of the best are kept (at most
// kMaxContacts), a strictly better one restarts the list.  finalize = false writes the list to nn,
// finalize = true sets active[v] from the side of the last listed triangle's plane.
template <bool FINALIZE>
__global__ void nearest_kernel(ContactMesh M, ContactState S, BvhView T, float4 const* __restrict__ x)
{
    int const q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *S.nActive || T.n < 1)
        return;
    int const v = S.av[q];
    int const i = M.V[v];
    float3 const p = f3(x[i]);
    int const body = M.B[i];
    float const eps = FLT_EPSILON;
    float dmin      = S.dupper[v];
    int32_t list[kMaxContacts];
    int count = 0;
    int32_t const leafBegin = T.n - 1;
    int32_t stack[kBvhStack];
    int top      = 0;
    stack[top++] = 0;
    while (top > 0)
    {
        int32_t const node = stack[--top];
        float const lo     = dmin - eps;
        float const hi     = dmin + eps;
        if (node < leafBegin)
        {
            if (point_box_sqdist(p, T.ilo[node], T.ihi[node]) <= hi)
            {
                if (top + 2 > kBvhStack)
                {
                    atomicOr(S.flags, kBvhErrStackOverflow);
                    return;
                }
                stack[top++] = T.child[2 * node];
                stack[top++] = T.child[2 * node + 1];
            }
            continue;
        }
        int32_t const s = node - leafBegin;
        if (point_box_sqdist(p, T.llo[s], T.lhi[s]) > hi)
            continue;
        int32_t const f = T.inds[s];
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
            int32_t const f                 = k < count ? list[k] : -1;
            S.nn[v * kMaxContacts + k]      = f;
            S.fc[i * kMaxContacts + k]      = f;
        }
    }
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
    initialize_kernel<<<blocks(M.nSurfV, 128), 128, 0, s>>>(M, S, view_of(S.bvh, M.nF), xt, xnext);
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
    nearest_kernel<false><<<blocks(M.nSurfV, 128), 128, 0, s>>>(M, S, view_of(S.bvh, M.nF), x);
    return cudaGetLastError();
}

cudaError_t contact_finalize(ContactMesh const& M, ContactState const& S, float4 const* x, cudaStream_t s)
{
    if (M.nF <= 0 || M.nSurfV <= 0)
        return cudaSuccess;
    cudaError_t e = refit(M, S, x, s);
    if (e != cudaSuccess)
        return e;
    nearest_kernel<true><<<blocks(M.nSurfV, 128), 128, 0, s>>>(M, S, view_of(S.bvh, M.nF), x);
    return cudaGetLastError();
}

} // namespace pbgb
