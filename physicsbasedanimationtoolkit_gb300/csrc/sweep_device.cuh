// Device-side pieces of the colour sweep and the substep kernels, shared by the per-colour
// launches (vbd_kernels.cu) and the persistent batched step (batched.cu).  COHERENT = true makes
// every access to state that the same kernel writes elsewhere (positions, Chebyshev history,
// inertial targets, velocities) go through L2 (ld.global.cg / st.global.cg), which a kernel that
// reads what its other blocks wrote needs; the per-colour launches use ordinary accesses.  The
// arithmetic is the same either way.
#pragma once

#include <cfloat>

#include "vbd_kernels.cuh"

namespace pbgb {

int constexpr kMaxContactsPerVertex = 8;

namespace {

template <bool COHERENT>
struct Mem
{
    static __device__ __forceinline__ float4 ld(float4 const* q)
    {
        if constexpr (COHERENT)
            return __ldcg(q);
        else
            return *q;
    }
    static __device__ __forceinline__ void st(float4* q, float4 v)
    {
        if constexpr (COHERENT)
            __stcg(q, v);
        else
            *q = v;
    }
};

__device__ __forceinline__ void load3(float4 const v, float* o)
{
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
}

__device__ __forceinline__ uint32_t corner(uint4 const& t, int a)
{
    return a == 0 ? t.x : (a == 1 ? t.y : (a == 2 ? t.z : t.w));
}

// Contact terms of one vertex-triangle pair (gpu/impl/vbd/Kernels.cuh:80-114,203-223): the
// triangle's corners at t and now (from x when their colour is solved before this one, else from
// hprev: bit 31 of the record), then the normal penalty and friction of vertex_triangle_contact
// with the record's penalty.
__device__ __forceinline__ void contact_pair(SweepParams const& p, int4 r, float kCf, float const* xt, float const* xi, float* H, float* g)
{
    uint32_t const v[3] = {uint32_t(r.x), uint32_t(r.y), uint32_t(r.z)};
    float xtf[3][3], xf[3][3];
    for (int k = 0; k < 3; ++k)
    {
        uint32_t const j = v[k] & 0x7FFFFFFFu;
        float4 const a   = p.xt[j];
        float4 const b   = __ldcg(((v[k] >> 31) ? p.x : p.hprev) + j);
        xtf[k][0] = a.x, xtf[k][1] = a.y, xtf[k][2] = a.z;
        xf[k][0] = b.x, xf[k][1] = b.y, xf[k][2] = b.z;
    }
    vertex_triangle_contact(xt, xi, xtf, xf, p.h, kCf, p.muF, p.epsv, FLT_EPSILON, g, H);
}

// Contact energy of vertex i, spread over the vertex's L lanes: lane l takes the record slots
// l, l + L, ... (kMaxContactsPerVertex of them); the lanes' gradients and Hessians are summed with
// xor shuffles inside the group (every lane of the warp takes part in the shuffles).  cH, cg: the
// group's sum, in every lane.
template <int L>
__device__ __forceinline__ void contact_terms(SweepParams const& p, bool valid, int lane, int i, float const* xt, float const* xi, float* cH, float* cg)
{
#pragma unroll
    for (int r = 0; r < 6; ++r)
        cH[r] = 0.f;
    cg[0] = cg[1] = cg[2] = 0.f;
    int const n = valid ? __ldg(p.ccount + i) : 0;
#pragma unroll
    for (int c = 0; c < (kMaxContactsPerVertex + L - 1) / L; ++c)
    {
        int const k = lane + c * L;
        if (k < n)
        {
            int4 const r = p.crec[i * kMaxContactsPerVertex + k];
            if (r.w >= 0)
                contact_pair(p, r, p.cpen[i * kMaxContactsPerVertex + k], xt, xi, cH, cg);
        }
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1)
    {
#pragma unroll
        for (int r = 0; r < 6; ++r)
            cH[r] += __shfl_xor_sync(0xffffffffu, cH[r], off);
#pragma unroll
        for (int r = 0; r < 3; ++r)
            cg[r] += __shfl_xor_sync(0xffffffffu, cg[r], off);
    }
}

// The end of a vertex solve, shared by both sweep kernels: xor-shuffle reduction of the lanes'
// 10 accumulated floats, then lane 0 applies damping, contact, inertia and the 3x3 Newton step and
// writes the iterate(s).
template <int L, bool CHEB, bool REC, bool CONTACT, bool COHERENT = false>
__device__ __forceinline__ void finish_vertex(SweepParams const& p, VertexBlock<float>& b, bool valid, int lane, int i, int s, float* xi)
{
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1)
    {
#pragma unroll
        for (int r = 0; r < 3; ++r)
            b.g[r] += __shfl_xor_sync(0xffffffffu, b.g[r], off);
        b.s += __shfl_xor_sync(0xffffffffu, b.s, off);
#pragma unroll
        for (int r = 0; r < 6; ++r)
            b.C[r] += __shfl_xor_sync(0xffffffffu, b.C[r], off);
    }
    float4 const xt4  = Mem<COHERENT>::ld(p.xt + i);
    float const xt[3] = {xt4.x, xt4.y, xt4.z};
    float cH[6], cg[3];
    bool constexpr contact = CHEB && CONTACT;
    if constexpr (contact)
        contact_terms<L>(p, valid, lane, i, xt, xi, cH, cg);
    if (!valid || lane != 0)
        return;
    float4 const xl4  = Mem<COHERENT>::ld(p.xtilde + i);
    float const xl[3] = {xl4.x, xl4.y, xl4.z};
    float H[6], g[3];
    elastic_system(b, xt, xi, p.h, p.kD, H, g);
    if constexpr (contact)
    {
#pragma unroll
        for (int r = 0; r < 6; ++r)
            H[r] += cH[r];
        g[0] += cg[0];
        g[1] += cg[1];
        g[2] += cg[2];
    }
    float dx[3];
    bool const moved = inertia_solve(H, g, xl, xt4.w, p.h2, p.detHZero, xi, static_cast<float*>(nullptr),
                                     static_cast<float*>(nullptr), dx);
    if (p.step)
        p.step[i] = make_float4(dx[0], dx[1], dx[2], 0.f);
    if (REC)
    {
        // H now includes the inertia term; its inverse by the adjugate, as in inertia_solve.
        float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
        if (moved)
        {
            float const a00 = H[3] * H[5] - H[4] * H[4];
            float const a01 = H[2] * H[4] - H[1] * H[5];
            float const a02 = H[1] * H[4] - H[2] * H[3];
            float const a11 = H[0] * H[5] - H[2] * H[2];
            float const a12 = H[1] * H[2] - H[0] * H[4];
            float const a22 = H[0] * H[3] - H[1] * H[1];
            float const inv = 1.f / (H[0] * a00 + H[1] * a01 + H[2] * a02);
            r0 = make_float4(inv * a00, inv * a01, inv * a02, inv * a11);
            r1 = make_float4(inv * a12, inv * a22, 0.f, 0.f);
        }
        p.tape[2 * s]     = r0;
        p.tape[2 * s + 1] = r1;
    }
    if (CHEB)
    {
        // Raw iterate k (even when the Newton step was skipped: later colours read it).
        Mem<COHERENT>::st(p.x + i, make_float4(xi[0], xi[1], xi[2], 0.f));
        if (p.k > 1)
        {
            float4 const km2 = Mem<COHERENT>::ld(p.hcur + i);
            xi[0]            = p.omega * (xi[0] - km2.x) + km2.x;
            xi[1]            = p.omega * (xi[1] - km2.y) + km2.y;
            xi[2]            = p.omega * (xi[2] - km2.z) + km2.z;
        }
        Mem<COHERENT>::st(p.hcur + i, make_float4(xi[0], xi[1], xi[2], 0.f));
    }
    else if (moved)
        Mem<COHERENT>::st(p.x + i, make_float4(xi[0], xi[1], xi[2], 0.f));
}

// Start of a substep (sim/vbd/Integrator.cpp:31-34,54-71; gpu/impl/vbd/Integrator.cu:190-248):
// xt <- x, xtilde = xt + h v + h^2 aext, x <- initial guess.
template <bool COHERENT = false>
__device__ __forceinline__ void begin_substep_vertex(SubstepParams const& p, int i)
{
    float4 const x4 = Mem<COHERENT>::ld(p.x + i);
    float4 const v4 = Mem<COHERENT>::ld(p.v + i);
    float4 const a4 = __ldg(p.aext + i);
    float const xt[3] = {x4.x, x4.y, x4.z};
    float const vt[3] = {v4.x, v4.y, v4.z};
    float const a[3]  = {a4.x, a4.y, a4.z};
    float vm[3]       = {vt[0], vt[1], vt[2]};
    if (p.gpuSemantics)
    {
        float4 const w = Mem<COHERENT>::ld(p.vprev + i);
        vm[0] = w.x, vm[1] = w.y, vm[2] = w.z;
    }
    Mem<COHERENT>::st(p.xt + i, make_float4(xt[0], xt[1], xt[2], __ldg(p.m + i)));
    Mem<COHERENT>::st(p.xtilde + i, make_float4(
        xt[0] + p.h * vt[0] + p.h2 * a[0],
        xt[1] + p.h * vt[1] + p.h2 * a[1],
        xt[2] + p.h * vt[2] + p.h2 * a[2],
        0.f));
    float x0[3];
    initial_position(xt, vm, vt, a, p.h, p.h2, p.strategy, FLT_MIN, x0);
    float4 const x04 = make_float4(x0[0], x0[1], x0[2], 0.f);
    Mem<COHERENT>::st(p.x + i, x04);
    if (p.h0)
    {
        Mem<COHERENT>::st(p.h0 + i, x04);
        Mem<COHERENT>::st(p.h1 + i, x04);
    }
}

// End of a substep: v = (x - xt)/h (sim/vbd/Kernels.h:121-129); the previous velocity is kept
// for the GPU integrator's AdaptiveVbd (gpu/impl/vbd/Integrator.cu:329-347).  Non-finite state
// raises flags[0].
template <bool COHERENT = false>
__device__ __forceinline__ void end_substep_vertex(SubstepParams const& p, int i)
{
    float4 const x4  = Mem<COHERENT>::ld(p.result + i);
    float4 const xt4 = Mem<COHERENT>::ld(p.xt + i);
    float4 const vo  = Mem<COHERENT>::ld(p.v + i);
    if (p.result != p.x)
        Mem<COHERENT>::st(p.x + i, x4);
    float const inv  = 1.f / p.h;
    float4 const vn  = make_float4((x4.x - xt4.x) * inv, (x4.y - xt4.y) * inv, (x4.z - xt4.z) * inv, 0.f);
    if (p.gpuSemantics)
        Mem<COHERENT>::st(p.vprev + i, vo);
    Mem<COHERENT>::st(p.v + i, vn);
    bool const finite = isfinite(x4.x) && isfinite(x4.y) && isfinite(x4.z) && isfinite(vn.x) &&
                        isfinite(vn.y) && isfinite(vn.z);
    if (!finite)
        atomicOr(p.flags, 1);
}


} // namespace

} // namespace pbgb
