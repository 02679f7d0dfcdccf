// CUDA kernels of the VBD step (sm_103a).  See vbd_kernels.cuh for the data layout.
#include "vbd_kernels.cuh"
#include "energy.cuh"

#include <algorithm>
#include <cfloat>

namespace pbgb {

int constexpr kMaxContactsPerVertex = 8;

namespace {

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
#pragma unroll
    for (int c = 0; c < (kMaxContactsPerVertex + L - 1) / L; ++c)
    {
        int const k = lane + c * L;
        if (valid && k < kMaxContactsPerVertex)
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
template <int L, bool CHEB, bool REC, bool CONTACT>
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
    float4 const xt4  = p.xt[i];
    float const xt[3] = {xt4.x, xt4.y, xt4.z};
    float cH[6], cg[3];
    bool constexpr contact = CHEB && CONTACT;
    if constexpr (contact)
        contact_terms<L>(p, valid, lane, i, xt, xi, cH, cg);
    if (!valid || lane != 0)
        return;
    float4 const xl4  = p.xtilde[i];
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
        p.x[i] = make_float4(xi[0], xi[1], xi[2], 0.f);
        if (p.k > 1)
        {
            float4 const km2 = p.hcur[i];
            xi[0]            = p.omega * (xi[0] - km2.x) + km2.x;
            xi[1]            = p.omega * (xi[1] - km2.y) + km2.y;
            xi[2]            = p.omega * (xi[2] - km2.z) + km2.z;
        }
        p.hcur[i] = make_float4(xi[0], xi[1], xi[2], 0.f);
    }
    else if (moved)
        p.x[i] = make_float4(xi[0], xi[1], xi[2], 0.f);
}

// Per-colour Gauss-Seidel sweep (reference: VbdIteration, gpu/impl/vbd/Kernels.cuh:148-233, and
// Integrator::SolveVertex, sim/vbd/Integrator.cpp:98-136).  L lanes cooperate on one vertex: lane
// l takes incidences l, l+L, ...; the 10 accumulated floats are then reduced with xor shuffles
// and lane 0 applies damping, inertia and the 3x3 Newton step, writing x in place.  Vertices of a
// colour share no tet, so the in-place write races with no reader of this launch.
//
// CHEB: the Chebyshev update of the reference (applied to all vertices after each full sweep,
// sim/vbd/ChebyshevIntegrator.cpp:15-32) is fused in.  Only vertex i's own values enter its
// update, so it is applied right after i's solve, with two position buffers keeping the
// reference's ordering: a neighbour of lower colour rank (already solved in iteration k) is read
// from x (raw iterate k), one of higher rank from hprev (accelerated iterate k-1).  hcur holds
// iterate k-2 on entry and receives the accelerated iterate k.
//
// REC (without CHEB): also writes the inverse Newton matrix of every solved vertex to p.tape for
// the adjoint sweep.
template <int L, bool CHEB, bool REC = false, bool CONTACT = false>
__global__ void __launch_bounds__(256, CONTACT ? 2 : 4) sweep_kernel(SweepParams p)
{
    int const tid    = blockIdx.x * blockDim.x + threadIdx.x;
    int const s      = p.begin + tid / L;
    int const lane   = tid & (L - 1);
    bool const valid = s < p.end;

    VertexBlock<float> b;
    zero(b);
    int i       = 0;
    float xi[3] = {0.f, 0.f, 0.f};
    float Xi[3] = {0.f, 0.f, 0.f};
    int k = 0, k1 = 0;
    uint32_t q0 = 0u, q1 = 0u;
    uint4 t     = make_uint4(0u, 0u, 0u, 0u);
    float4 mat  = make_float4(0.f, 0.f, 0.f, 0.f);
    // Prologue on data no earlier launch writes (mesh tables): with programmatic dependent launch
    // it overlaps the previous colour's tail.
    if (valid)
    {
        i  = __ldg(p.solve + s);
        load3(__ldg(p.X + i), Xi);
        k1 = __ldg(p.incPtr + s + 1);
        k  = __ldg(p.incPtr + s) + lane;
        // Software pipeline: the record of incidence k+L and the incidence word of k+2L are in
        // flight while incidence k's corners are gathered and its block accumulated.
        q0 = k < k1 ? __ldg(p.inc + k) : 0u;
        q1 = k + L < k1 ? __ldg(p.inc + k + L) : 0u;
        if (k < k1)
        {
            t   = __ldg(&p.tets[q0 >> 2].v);
            mat = __ldg(&p.tets[q0 >> 2].mat);
        }
    }
    // Positions are written by the previous launches: wait for them (no-op without PDL), then let
    // the next colour's grid start its own prologue.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (valid)
    {
        load3(CHEB ? p.hprev[i] : p.x[i], xi);
        for (; k < k1; k += L)
        {
            int const il = int(q0 & 3u);
            uint4 tn     = make_uint4(0u, 0u, 0u, 0u);
            float4 matn  = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k + L < k1)
            {
                tn   = __ldg(&p.tets[q1 >> 2].v);
                matn = __ldg(&p.tets[q1 >> 2].mat);
            }
            uint32_t const q2 = k + 2 * L < k1 ? __ldg(p.inc + k + 2 * L) : 0u;
            uint32_t const own = corner(t, il) >> 30;
            float d[3][3], e[3][3];
#pragma unroll
            for (int m = 0; m < 3; ++m)
            {
                uint32_t const ta = corner(t, (il + 1 + m) & 3);
                uint32_t const j  = ta & kIndexMask;
                float4 const* src = p.x;
                if (CHEB && (ta >> 30) > own)
                    src = p.hprev;
                float4 const xa = __ldg(src + j);
                float4 const Xa = __ldg(p.X + j);
                d[m][0] = xa.x - xi[0];
                d[m][1] = xa.y - xi[1];
                d[m][2] = xa.z - xi[2];
                e[m][0] = Xa.x - Xi[0];
                e[m][1] = Xa.y - Xi[1];
                e[m][2] = Xa.z - Xi[2];
            }
            float G[3][3];
            rest_gradients(e, G);
            accumulate_tet(b, d, G, mat.x, mat.y, mat.z);
            q0  = q1;
            q1  = q2;
            t   = tn;
            mat = matn;
        }
    }
    finish_vertex<L, CHEB, REC, CONTACT>(p, b, valid, lane, i, s, xi);
}

// The same sweep with each vertex's neighbours staged in shared memory.  A vertex's ~23 incident
// tets reference only ~14 distinct neighbours, so instead of gathering three corners' current
// and rest positions per incidence, the vertex's lanes load each neighbour once into its slice of
// the block's slab (rest positions before griddepcontrol.wait: no launch writes them; current
// positions after it), and the incidence loop reads them back through the three slot bytes of its
// packed incidence word.  The slab slice of solve entry s starts at nbrPtr[s] - nbrPtr[first
// entry of the block]; a slot of the plain and Chebyshev sweeps is 24 bytes, a float4 (position,
// rest x) in the first array of p.slab float4 and a float2 (rest y, rest z) in the second (a
// 16-byte stride spreads random slots over all shared-memory banks; an incidence reads a 16- and
// an 8-byte word per corner instead of two 16-byte words), and the same lane writes both parts of
// a slot (rest x before the wait, the position after it, disjoint bytes); the contact variant keeps
// two float4 arrays.  The lanes of a vertex share a warp, so __syncwarp orders the staging.
template <int L, bool CHEB, bool REC = false, bool CONTACT = false>
__global__ void __launch_bounds__(256, CONTACT ? 2 : 4) staged_sweep_kernel(SweepParams p)
{
    // Neighbour slot j.  Plain and Chebyshev sweeps: slab[j] = (x, y, z, rest x) and
    // restYZ[j] = (rest y, rest z), 24 bytes a slot.  Contact variant: slab[j] = position and
    // rest[j] = rest position, 32 bytes a slot (measured faster for that variant: 2.22 against
    // 2.35 ms per contact step, where the packed slots took the Chebyshev beam step from 4.87 to
    // 4.77 ms).
    extern __shared__ float4 slab[];
    float2* const restYZ = reinterpret_cast<float2*>(slab + p.slab);
    float4* const rest   = slab + p.slab;
    int const tid    = blockIdx.x * blockDim.x + threadIdx.x;
    int const s      = p.begin + tid / L;
    int const lane   = tid & (L - 1);
    bool const valid = s < p.end;
    // The block's first entry is valid: the grid covers exactly (end - begin) * L threads.
    int const first = p.begin + int(blockIdx.x) * (int(blockDim.x) / L);
    int const nb0   = __ldg(p.nbrPtr + first);

    VertexBlock<float> b;
    zero(b);
    int i       = 0;
    float xi[3] = {0.f, 0.f, 0.f};
    float Xi[3] = {0.f, 0.f, 0.f};
    int k = 0, k1 = 0, n0 = 0, n1 = 0, base = 0;
    uint2 q     = make_uint2(0u, 0u);
    float4 mat  = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid)
    {
        i  = __ldg(p.solve + s);
        load3(__ldg(p.X + i), Xi);
        n0   = __ldg(p.nbrPtr + s);
        n1   = __ldg(p.nbrPtr + s + 1);
        base = n0 - nb0;
        for (int j = n0 + lane; j < n1; j += L)
        {
            float4 const Xa = __ldg(p.X + (__ldg(p.nbr + j) & kIndexMask));
            if constexpr (CONTACT)
                rest[base + j - n0] = Xa;
            else
            {
                restYZ[base + j - n0]                               = make_float2(Xa.y, Xa.z);
                reinterpret_cast<float*>(slab + base + j - n0)[3] = Xa.x;
            }
        }
        k1 = __ldg(p.incPtr + s + 1);
        k  = __ldg(p.incPtr + s) + lane;
        if (k < k1)
        {
            q   = __ldg(p.incPack + k);
            mat = __ldg(p.mats + q.x);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (valid)
    {
        load3(CHEB ? p.hprev[i] : p.x[i], xi);
        for (int j = n0 + lane; j < n1; j += L)
        {
            uint32_t const a  = __ldg(p.nbr + j);
            float4 const* src = p.x;
            if (CHEB && !(a >> 31))
                src = p.hprev;
            float4 const xa = __ldg(src + (a & kIndexMask));
            if constexpr (CONTACT)
                slab[base + j - n0] = xa;
            else
            {
                float* const dst                = reinterpret_cast<float*>(slab + base + j - n0);
                *reinterpret_cast<float2*>(dst) = make_float2(xa.x, xa.y);
                dst[2]                          = xa.z;
            }
        }
    }
    __syncwarp();
    if (valid)
    {
        for (; k < k1; k += L)
        {
            uint2 qn     = make_uint2(0u, 0u);
            float4 matn  = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k + L < k1)
            {
                qn   = __ldg(p.incPack + k + L);
                matn = __ldg(p.mats + qn.x);
            }
            float d[3][3], e[3][3];
#pragma unroll
            for (int m = 0; m < 3; ++m)
            {
                int const slot   = base + int((q.y >> (8 * m)) & 0xFFu);
                float4 const xa = slab[slot];
                float Xa[3];
                if constexpr (CONTACT)
                {
                    float4 const r = rest[slot];
                    Xa[0] = r.x, Xa[1] = r.y, Xa[2] = r.z;
                }
                else
                {
                    float2 const r = restYZ[slot];
                    Xa[0] = xa.w, Xa[1] = r.x, Xa[2] = r.y;
                }
                d[m][0] = xa.x - xi[0];
                d[m][1] = xa.y - xi[1];
                d[m][2] = xa.z - xi[2];
                e[m][0] = Xa[0] - Xi[0];
                e[m][1] = Xa[1] - Xi[1];
                e[m][2] = Xa[2] - Xi[2];
            }
            float G[3][3];
            rest_gradients(e, G);
            accumulate_tet(b, d, G, mat.x, mat.y, mat.z);
            q   = qn;
            mat = matn;
        }
    }
    finish_vertex<L, CHEB, REC, CONTACT>(p, b, valid, lane, i, s, xi);
}

// Start of a substep (sim/vbd/Integrator.cpp:31-34,54-71; gpu/impl/vbd/Integrator.cu:190-248):
// xt <- x, xtilde = xt + h v + h^2 aext, x <- initial guess.
__global__ void begin_substep_kernel(SubstepParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    float4 const x4 = p.x[i];
    float4 const v4 = p.v[i];
    float4 const a4 = p.aext[i];
    float const xt[3] = {x4.x, x4.y, x4.z};
    float const vt[3] = {v4.x, v4.y, v4.z};
    float const a[3]  = {a4.x, a4.y, a4.z};
    float vm[3]       = {vt[0], vt[1], vt[2]};
    if (p.gpuSemantics)
    {
        float4 const w = p.vprev[i];
        vm[0] = w.x, vm[1] = w.y, vm[2] = w.z;
    }
    p.xt[i]     = make_float4(xt[0], xt[1], xt[2], p.m[i]);
    p.xtilde[i] = make_float4(
        xt[0] + p.h * vt[0] + p.h2 * a[0],
        xt[1] + p.h * vt[1] + p.h2 * a[1],
        xt[2] + p.h * vt[2] + p.h2 * a[2],
        0.f);
    float x0[3];
    initial_position(xt, vm, vt, a, p.h, p.h2, p.strategy, FLT_MIN, x0);
    float4 const x04 = make_float4(x0[0], x0[1], x0[2], 0.f);
    p.x[i]           = x04;
    if (p.h0)
    {
        p.h0[i] = x04;
        p.h1[i] = x04;
    }
}

// End of a substep: v = (x - xt)/h (sim/vbd/Kernels.h:121-129); the previous velocity is kept
// for the GPU integrator's AdaptiveVbd (gpu/impl/vbd/Integrator.cu:329-347).  Non-finite state
// raises flags[0].
__global__ void end_substep_kernel(SubstepParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n)
        return;
    float4 const x4  = p.result[i];
    float4 const xt4 = p.xt[i];
    float4 const vo  = p.v[i];
    if (p.result != p.x)
        p.x[i] = x4;
    float const inv  = 1.f / p.h;
    float4 const vn  = make_float4((x4.x - xt4.x) * inv, (x4.y - xt4.y) * inv, (x4.z - xt4.z) * inv, 0.f);
    if (p.gpuSemantics)
        p.vprev[i] = vo;
    p.v[i] = vn;
    bool const finite = isfinite(x4.x) && isfinite(x4.y) && isfinite(x4.z) && isfinite(vn.x) &&
                        isfinite(vn.y) && isfinite(vn.z);
    if (!finite)
        atomicOr(p.flags, 1);
}

// Objective of the backward-Euler step (sim/vbd/Integrator.cpp:138-165): per-entity terms in FP32,
// the global sum in FP64.  Entity j is always summed by the same thread of the same block of a
// fixed grid, warps and blocks are added in index order, so the value is the same on every run.
__global__ void __launch_bounds__(256) objective_kernel(EnergyParams p)
{
    __shared__ double warps[8];
    double acc  = 0.0;
    int const n = p.nV > p.nT ? p.nV : p.nT;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        acc += objective_term(p, j);
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0)
        warps[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double b = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w)
            b += warps[w];
        p.partials[blockIdx.x] = b;
    }
}

// Sum of the objective's block partials in block order, plus the rest-state energy.
__global__ void __launch_bounds__(32) objective_finish_kernel(EnergyParams p, int32_t blocks)
{
    double acc = 0.0;
    for (int b = int(threadIdx.x); b < blocks; b += 32)
        acc += p.partials[b];
    acc = warp_sum(acc);
    if (threadIdx.x == 0)
        p.out[0] = acc + p.dt2 * p.restEnergy;
}

// Gradient of the objective (sim/vbd/Integrator.cpp:167-200): inertial part per vertex, elastic
// part per tet scattered with FP64 atomics.
__global__ void gradient_kernel(EnergyParams p)
{
    int const n = p.nV > p.nT ? p.nV : p.nT;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    {
        if (j < p.nV)
        {
            float4 const x = p.x[j], y = p.xtilde[j];
            double const mj = p.m[j];
            atomicAdd(p.out + 3 * j + 0, mj * (double(x.x) - y.x));
            atomicAdd(p.out + 3 * j + 1, mj * (double(x.y) - y.y));
            atomicAdd(p.out + 3 * j + 2, mj * (double(x.z) - y.z));
        }
        if (j < p.nT)
        {
            float f[3][3], G[4][3];
            int4 t;
            float4 mat;
            tet_F(p, j, f, t, G, mat);
            float k[3][3];
            k[0][0] = f[1][1] * f[2][2] - f[1][2] * f[2][1];
            k[0][1] = f[1][2] * f[2][0] - f[1][0] * f[2][2];
            k[0][2] = f[1][0] * f[2][1] - f[1][1] * f[2][0];
            k[1][0] = f[2][1] * f[0][2] - f[2][2] * f[0][1];
            k[1][1] = f[2][2] * f[0][0] - f[2][0] * f[0][2];
            k[1][2] = f[2][0] * f[0][1] - f[2][1] * f[0][0];
            k[2][0] = f[0][1] * f[1][2] - f[0][2] * f[1][1];
            k[2][1] = f[0][2] * f[1][0] - f[0][0] * f[1][2];
            k[2][2] = f[0][0] * f[1][1] - f[0][1] * f[1][0];
            float const J  = f[0][0] * k[0][0] + f[0][1] * k[0][1] + f[0][2] * k[0][2];
            float const sl = mat.y * (J - mat.z);
            // P = mu' F + lambda' (J - alpha) cof F ; dE/dx_a = P w_a
            float P[3][3];
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r)
                    P[c][r] = mat.x * f[c][r] + sl * k[c][r];
            int const vid[4] = {t.x, t.y, t.z, t.w};
            for (int a = 0; a < 4; ++a)
                for (int r = 0; r < 3; ++r)
                {
                    double const s = double(P[0][r]) * G[a][0] + double(P[1][r]) * G[a][1] +
                                     double(P[2][r]) * G[a][2];
                    atomicAdd(p.out + 3 * vid[a] + r, p.dt2 * s);
                }
        }
    }
}

__global__ void pack3_kernel(float const* __restrict__ in3, float4* __restrict__ out4, int32_t n)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out4[i] = make_float4(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2], 0.f);
}

__global__ void unpack3_kernel(float4 const* __restrict__ in4, float* __restrict__ out3, int32_t n)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        float4 const v = in4[i];
        out3[3 * i]     = v.x;
        out3[3 * i + 1] = v.y;
        out3[3 * i + 2] = v.z;
    }
}

// Contact records of vertex i (SweepParams::crec): the area-scaled penalty of every listed
// triangle (the vertex area over the summed areas of its listed triangles, times muC and the
// triangle's area) and the corners' read rule for the colour sweep.
__global__ void contact_records_kernel(int32_t nV, int32_t const* __restrict__ fc, int4 const* __restrict__ F,
                                       float const* __restrict__ FA, float const* __restrict__ XVA,
                                       int32_t const* __restrict__ vcolor, float muC, int4* __restrict__ crec,
                                       float* __restrict__ cpen)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nV)
        return;
    int32_t f[kMaxContactsPerVertex];
    float sumfa = 0.f;
    for (int c = 0; c < kMaxContactsPerVertex; ++c)
    {
        f[c] = fc[i * kMaxContactsPerVertex + c];
        if (f[c] >= 0)
            sumfa += FA[f[c]];
    }
    float const kC  = sumfa > 0.f ? (XVA[i] * muC) / sumfa : 0.f;
    int32_t const own = vcolor[i];
    for (int c = 0; c < kMaxContactsPerVertex; ++c)
    {
        int4 r   = make_int4(0, 0, 0, -1);
        float pn = 0.f;
        if (f[c] >= 0)
        {
            int4 const t     = F[f[c]];
            int const v[3]   = {t.x, t.y, t.z};
            uint32_t code[3];
            for (int k = 0; k < 3; ++k)
                code[k] = uint32_t(v[k]) | (vcolor[v[k]] < own ? 0x80000000u : 0u);
            r  = make_int4(int(code[0]), int(code[1]), int(code[2]), f[c]);
            pn = kC * FA[f[c]];
        }
        crec[i * kMaxContactsPerVertex + c] = r;
        cpen[i * kMaxContactsPerVertex + c] = pn;
    }
}

inline int blocks_for(int64_t n, int block)
{
    return int((n + block - 1) / block);
}

} // namespace

template <int L, bool CHEB, bool REC = false, bool CONTACT = false>
cudaError_t launch_sweep_l(SweepParams const& p, int g, int block, bool pdl, cudaStream_t s, size_t stagedBytes)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = dim3(unsigned(g));
    cfg.blockDim           = dim3(unsigned(block));
    // stagedBytes sizes the largest slot; this variant's slots may be smaller (staged_sweep_kernel).
    cfg.dynamicSmemBytes   = stagedBytes > 0 ? size_t(p.slab) * kStagedSlotBytes<CONTACT> : 0;
    cfg.stream             = s;
    cudaLaunchAttribute attr[1];
    attr[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs                                          = attr;
    cfg.numAttrs                                       = pdl ? 1 : 0;
    if (stagedBytes > 0)
        return cudaLaunchKernelEx(&cfg, staged_sweep_kernel<L, CHEB, REC, CONTACT>, p);
    return cudaLaunchKernelEx(&cfg, sweep_kernel<L, CHEB, REC, CONTACT>, p);
}

template <bool CHEB, bool REC, bool CONTACT = false>
cudaError_t launch_sweep_t(SweepParams const& p, int lanes, int g, int block, bool pdl, cudaStream_t s, size_t stagedBytes)
{
    switch (lanes)
    {
        case 1: return launch_sweep_l<1, CHEB, REC, CONTACT>(p, g, block, pdl, s, stagedBytes);
        case 2: return launch_sweep_l<2, CHEB, REC, CONTACT>(p, g, block, pdl, s, stagedBytes);
        case 4: return launch_sweep_l<4, CHEB, REC, CONTACT>(p, g, block, pdl, s, stagedBytes);
        case 8: return launch_sweep_l<8, CHEB, REC, CONTACT>(p, g, block, pdl, s, stagedBytes);
        case 16: return launch_sweep_l<16, CHEB, REC, CONTACT>(p, g, block, pdl, s, stagedBytes);
        case 32: return launch_sweep_l<32, CHEB, REC, CONTACT>(p, g, block, pdl, s, stagedBytes);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_sweep(SweepParams const& p, int lanes, int block, bool chebyshev, bool pdl, cudaStream_t s, size_t stagedBytes)
{
    int64_t const n = int64_t(p.end - p.begin) * lanes;
    if (n <= 0)
        return cudaSuccess;
    if (stagedBytes > kStagedMaxBytes || (stagedBytes > 0 && (!p.nbrPtr || !p.nbr || !p.incPack || !p.mats)))
        return cudaErrorInvalidValue;
    // Contact terms exist only in the two-buffer sweep (a contact partner of the same colour is
    // read as it was before the pass): a one-buffer launch with contact lists is a caller error.
    if (p.fc && !chebyshev)
        return cudaErrorInvalidValue;
    int const g   = blocks_for(n, block);
    SweepParams q = p;
    q.slab        = int32_t(stagedBytes / kStagedSlotBytesMax);
    if (chebyshev && q.fc)
        return launch_sweep_t<true, false, true>(q, lanes, g, block, pdl, s, stagedBytes);
    return chebyshev ? launch_sweep_t<true, false>(q, lanes, g, block, pdl, s, stagedBytes)
                     : launch_sweep_t<false, false>(q, lanes, g, block, pdl, s, stagedBytes);
}

cudaError_t launch_sweep_record(SweepParams const& p, int lanes, int block, bool pdl, cudaStream_t s, size_t stagedBytes)
{
    int64_t const n = int64_t(p.end - p.begin) * lanes;
    if (n <= 0)
        return cudaSuccess;
    if (!p.tape || stagedBytes > kStagedMaxBytes || (stagedBytes > 0 && (!p.nbrPtr || !p.nbr || !p.incPack || !p.mats)))
        return cudaErrorInvalidValue;
    SweepParams q = p;
    q.slab        = int32_t(stagedBytes / kStagedSlotBytesMax);
    return launch_sweep_t<false, true>(q, lanes, blocks_for(n, block), block, pdl, s, stagedBytes);
}

size_t staged_sweep_bytes(int32_t const* nbrPtr, int32_t begin, int32_t end, int lanes, int block)
{
    int const per = block / lanes;
    if (per <= 0)
        return 0;
    int64_t most = 0;
    for (int32_t b0 = begin; b0 < end; b0 += per)
    {
        int32_t const b1 = b0 + per < end ? b0 + per : end;
        most             = std::max<int64_t>(most, int64_t(nbrPtr[b1]) - nbrPtr[b0]);
    }
    return size_t(most) * kStagedSlotBytesMax;
}

namespace {

template <bool CHEB, bool REC, bool CONTACT = false>
cudaError_t allow_staged_smem()
{
    cudaError_t e = cudaSuccess;
    auto set      = [&](auto kernel) {
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStagedMaxBytes));
    };
    set(staged_sweep_kernel<1, CHEB, REC, CONTACT>);
    set(staged_sweep_kernel<2, CHEB, REC, CONTACT>);
    set(staged_sweep_kernel<4, CHEB, REC, CONTACT>);
    set(staged_sweep_kernel<8, CHEB, REC, CONTACT>);
    set(staged_sweep_kernel<16, CHEB, REC, CONTACT>);
    set(staged_sweep_kernel<32, CHEB, REC, CONTACT>);
    return e;
}

} // namespace

cudaError_t prepare_staged_sweeps()
{
    cudaError_t e = allow_staged_smem<false, false>();
    if (e == cudaSuccess)
        e = allow_staged_smem<true, false>();
    if (e == cudaSuccess)
        e = allow_staged_smem<false, true>();
    if (e == cudaSuccess)
        e = allow_staged_smem<true, false, true>();
    return e;
}

cudaError_t launch_begin_substep(SubstepParams const& p, cudaStream_t s)
{
    if (p.n <= 0)
        return cudaSuccess;
    begin_substep_kernel<<<blocks_for(p.n, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_end_substep(SubstepParams const& p, cudaStream_t s)
{
    if (p.n <= 0)
        return cudaSuccess;
    end_substep_kernel<<<blocks_for(p.n, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_objective(EnergyParams const& p, cudaStream_t s)
{
    if (!p.partials || !p.out)
        return cudaErrorInvalidValue;
    int const n = p.nV > p.nT ? p.nV : p.nT;
    int g       = blocks_for(n, 256);
    if (g > kObjectiveMaxBlocks)
        g = kObjectiveMaxBlocks;
    if (g < 1)
        g = 1;
    objective_kernel<<<g, 256, 0, s>>>(p);
    cudaError_t const e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    objective_finish_kernel<<<1, 32, 0, s>>>(p, g);
    return cudaGetLastError();
}

cudaError_t launch_gradient(EnergyParams const& p, cudaStream_t s)
{
    int const n = p.nV > p.nT ? p.nV : p.nT;
    int g       = blocks_for(n, 256);
    if (g > 4096)
        g = 4096;
    if (g < 1)
        g = 1;
    gradient_kernel<<<g, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_pack3(float const* in3, float4* out4, int32_t n, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    pack3_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in3, out4, n);
    return cudaGetLastError();
}

cudaError_t launch_contact_records(int32_t nV, int32_t const* fc, int4 const* F, float const* FA, float const* XVA,
                                   int32_t const* vcolor, float muC, int4* crec, float* cpen, cudaStream_t s)
{
    if (nV <= 0)
        return cudaSuccess;
    contact_records_kernel<<<blocks_for(nV, 256), 256, 0, s>>>(nV, fc, F, FA, XVA, vcolor, muC, crec, cpen);
    return cudaGetLastError();
}

cudaError_t launch_unpack3(float4 const* in4, float* out3, int32_t n, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    unpack3_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in4, out3, n);
    return cudaGetLastError();
}

} // namespace pbgb
