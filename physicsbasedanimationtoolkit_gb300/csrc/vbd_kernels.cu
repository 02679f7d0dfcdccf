// CUDA kernels of the VBD step (sm_103a).  See vbd_kernels.cuh for the data layout.
#include "vbd_kernels.cuh"
#include "energy.cuh"
#include "sweep_device.cuh"

#include <algorithm>
#include <cfloat>

namespace pbgb {

namespace {

// Per-colour Gauss-Seidel sweep (reference: VbdIteration, gpu/impl/vbd/Kernels.cuh:148-233, and
// Integrator::SolveVertex, sim/vbd/Integrator.cpp:98-136).  L lanes cooperate on one vertex: lane
// l takes incidences l, l+L, ...; the 10 accumulated floats are then reduced with xor shuffles
// and lane 0 applies damping, inertia and the 3x3 Newton step, writing x in place.  Vertices of a
// colour share no tet, so the in-place write races with no reader of this launch.  Each incidence
// reads its 20 bytes of rest-state stiffness (b0, b1, b2, kappa, sigma; TetStiffness resolved for
// the vertex's corner) and the three other corners' current positions: no rest position is read.
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
    int k = 0, k1 = 0;
    uint32_t q0 = 0u, q1 = 0u;
    uint4 t     = make_uint4(0u, 0u, 0u, 0u);
    float4 st   = make_float4(0.f, 0.f, 0.f, 0.f);
    float sg    = 0.f;
    // Prologue on data no earlier launch writes (mesh tables): with programmatic dependent launch
    // it overlaps the previous colour's tail.
    if (valid)
    {
        i  = __ldg(p.solve + s);
        k1 = __ldg(p.incPtr + s + 1);
        k  = __ldg(p.incPtr + s) + lane;
        // Software pipeline: the records of incidence k+L and the incidence word of k+2L are in
        // flight while incidence k's corners are gathered and its block accumulated.
        q0 = k < k1 ? __ldg(p.inc + k) : 0u;
        q1 = k + L < k1 ? __ldg(p.inc + k + L) : 0u;
        if (k < k1)
        {
            t  = __ldg(&p.tets[q0 >> 2].v);
            st = __ldg(p.stiff + k);
            sg = __uint_as_float(__ldg(&p.incPack[k].y));
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
            float4 stn   = make_float4(0.f, 0.f, 0.f, 0.f);
            float sgn    = 0.f;
            if (k + L < k1)
            {
                tn  = __ldg(&p.tets[q1 >> 2].v);
                stn = __ldg(p.stiff + k + L);
                sgn = __uint_as_float(__ldg(&p.incPack[k + L].y));
            }
            uint32_t const q2 = k + 2 * L < k1 ? __ldg(p.inc + k + 2 * L) : 0u;
            uint32_t const own = corner(t, il) >> 30;
            float d[3][3];
#pragma unroll
            for (int m = 0; m < 3; ++m)
            {
                uint32_t const ta = corner(t, (il + 1 + m) & 3);
                uint32_t const j  = ta & kIndexMask;
                float4 const* src = p.x;
                if (CHEB && (ta >> 30) > own)
                    src = p.hprev;
                float4 const xa = __ldg(src + j);
                d[m][0] = xa.x - xi[0];
                d[m][1] = xa.y - xi[1];
                d[m][2] = xa.z - xi[2];
            }
            accumulate_incidence(b, d, st.x, st.y, st.z, sg, st.w);
            q0 = q1;
            q1 = q2;
            t  = tn;
            st = stn;
            sg = sgn;
        }
    }
    finish_vertex<L, CHEB, REC, CONTACT>(p, b, valid, lane, i, s, xi);
}

// The same sweep with each vertex's neighbours staged in shared memory.  A vertex's ~23 incident
// tets reference only ~14 distinct neighbours, so instead of gathering three corners' positions
// per incidence, the vertex's lanes load each neighbour's current position once into its slice of
// the block's slab (a float4 per neighbour) after griddepcontrol.wait, and the incidence loop reads
// them back through the three slot bytes of its packed incidence word.  The slab slice of solve entry s starts at nbrPtr[s] - nbrPtr[first entry of the block].
// The lanes of a vertex share a warp, so __syncwarp orders the staging.
template <int L, bool CHEB, bool REC = false, bool CONTACT = false>
__global__ void __launch_bounds__(256, CONTACT ? 2 : 4) staged_sweep_kernel(SweepParams p)
{
    extern __shared__ float4 slab[];
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
    int k = 0, k1 = 0, n0 = 0, n1 = 0, base = 0;
    uint2 q0 = make_uint2(0u, 0u), q1 = q0;
    float4 st0 = make_float4(0.f, 0.f, 0.f, 0.f), st1 = st0;
    // The mesh tables are not written by any launch of the step: the vertex's first neighbour
    // indices and first two incidence records are loaded before griddepcontrol.wait, so that
    // only the position loads remain on the path after it.
    int constexpr kPreNbr = 4;
    uint32_t pre[kPreNbr];
#pragma unroll
    for (int m = 0; m < kPreNbr; ++m)
        pre[m] = 0u;
    if (valid)
    {
        i    = __ldg(p.solve + s);
        n0   = __ldg(p.nbrPtr + s);
        n1   = __ldg(p.nbrPtr + s + 1);
        base = n0 - nb0;
        k1   = __ldg(p.incPtr + s + 1);
        k    = __ldg(p.incPtr + s) + lane;
#pragma unroll
        for (int m = 0; m < kPreNbr; ++m)
            if (n0 + lane + m * L < n1)
                pre[m] = __ldg(p.nbr + n0 + lane + m * L);
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
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (valid)
    {
        load3(CHEB ? p.hprev[i] : p.x[i], xi);
#pragma unroll
        for (int m = 0; m < kPreNbr; ++m)
        {
            int const j = n0 + lane + m * L;
            if (j < n1)
            {
                float4 const* src = p.x;
                if (CHEB && !(pre[m] >> 31))
                    src = p.hprev;
                slab[base + j - n0] = __ldg(src + (pre[m] & kIndexMask));
            }
        }
        for (int j = n0 + lane + kPreNbr * L; j < n1; j += L)
        {
            uint32_t const a  = __ldg(p.nbr + j);
            float4 const* src = p.x;
            if (CHEB && !(a >> 31))
                src = p.hprev;
            slab[base + j - n0] = __ldg(src + (a & kIndexMask));
        }
    }
    __syncwarp();
    if (valid)
    {
        // Two incidences' records in flight ahead of the one being accumulated.
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
    finish_vertex<L, CHEB, REC, CONTACT>(p, b, valid, lane, i, s, xi);
}

// Start of a substep, one thread per vertex (begin_substep_vertex).
__global__ void begin_substep_kernel(SubstepParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < p.n)
        begin_substep_vertex(p, i);
}

// End of a substep, one thread per vertex (end_substep_vertex).
__global__ void end_substep_kernel(SubstepParams p)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < p.n)
        end_substep_vertex(p, i);
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

// 3 x n floats -> float4 per vertex, minus the vertex's origin when given (positions of a batch,
// stored relative to their mesh's origin).
__global__ void pack3_kernel(float const* __restrict__ in3, float4* __restrict__ out4, int32_t n, float4 const* __restrict__ origin)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        float4 v = make_float4(in3[3 * i], in3[3 * i + 1], in3[3 * i + 2], 0.f);
        if (origin)
        {
            float4 const o = origin[i];
            v.x -= o.x;
            v.y -= o.y;
            v.z -= o.z;
        }
        out4[i] = v;
    }
}

// float4 per vertex -> 3 x n floats, plus the vertex's origin when given.
__global__ void unpack3_kernel(float4 const* __restrict__ in4, float* __restrict__ out3, int32_t n, float4 const* __restrict__ origin)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        float4 v = in4[i];
        if (origin)
        {
            float4 const o = origin[i];
            v.x += o.x;
            v.y += o.y;
            v.z += o.z;
        }
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
                                       float* __restrict__ cpen, int32_t* __restrict__ ccount)
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
    // Listed triangles first, in list order (the lists hold no gaps, so this keeps every slot).
    int n = 0;
    for (int c = 0; c < kMaxContactsPerVertex; ++c)
    {
        if (f[c] < 0)
            continue;
        int4 const t   = F[f[c]];
        int const v[3] = {t.x, t.y, t.z};
        uint32_t code[3];
        for (int k = 0; k < 3; ++k)
            code[k] = uint32_t(v[k]) | (vcolor[v[k]] < own ? 0x80000000u : 0u);
        crec[i * kMaxContactsPerVertex + n] = make_int4(int(code[0]), int(code[1]), int(code[2]), f[c]);
        cpen[i * kMaxContactsPerVertex + n] = kC * FA[f[c]];
        ++n;
    }
    for (int c = n; c < kMaxContactsPerVertex; ++c)
    {
        crec[i * kMaxContactsPerVertex + c] = make_int4(0, 0, 0, -1);
        cpen[i * kMaxContactsPerVertex + c] = 0.f;
    }
    ccount[i] = n;
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
    cfg.dynamicSmemBytes   = stagedBytes;
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
    if (!p.stiff || !p.incPack || stagedBytes > kStagedMaxBytes || (stagedBytes > 0 && (!p.nbrPtr || !p.nbr)))
        return cudaErrorInvalidValue;
    // Contact terms exist only in the two-buffer sweep (a contact partner of the same colour is
    // read as it was before the pass): a one-buffer launch with contact lists is a caller error.
    if (p.fc && !chebyshev)
        return cudaErrorInvalidValue;
    int const g   = blocks_for(n, block);
    SweepParams q = p;
    if (chebyshev && q.fc)
        return launch_sweep_t<true, false, true>(q, lanes, g, block, pdl, s, stagedBytes);
    return chebyshev ? launch_sweep_t<true, false>(q, lanes, g, block, pdl, s, stagedBytes)
                     : launch_sweep_t<false, false>(q, lanes, g, block, pdl, s, stagedBytes);
}

cudaError_t launch_sweep_record(SweepParams const& p, int lanes, int block, bool chebyshev, bool pdl, cudaStream_t s, size_t stagedBytes)
{
    int64_t const n = int64_t(p.end - p.begin) * lanes;
    if (n <= 0)
        return cudaSuccess;
    if (!p.tape || !p.stiff || !p.incPack || p.fc || stagedBytes > kStagedMaxBytes || (stagedBytes > 0 && (!p.nbrPtr || !p.nbr)))
        return cudaErrorInvalidValue;
    int const g = blocks_for(n, block);
    return chebyshev ? launch_sweep_t<true, true>(p, lanes, g, block, pdl, s, stagedBytes)
                     : launch_sweep_t<false, true>(p, lanes, g, block, pdl, s, stagedBytes);
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
    return size_t(most) * kStagedSlotBytes;
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
        e = allow_staged_smem<true, true>();
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

cudaError_t launch_pack3(float const* in3, float4* out4, int32_t n, cudaStream_t s, float4 const* origin)
{
    if (n <= 0)
        return cudaSuccess;
    pack3_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in3, out4, n, origin);
    return cudaGetLastError();
}

cudaError_t launch_contact_records(int32_t nV, int32_t const* fc, int4 const* F, float const* FA, float const* XVA,
                                   int32_t const* vcolor, float muC, int4* crec, float* cpen, int32_t* ccount,
                                   cudaStream_t s)
{
    if (nV <= 0)
        return cudaSuccess;
    contact_records_kernel<<<blocks_for(nV, 256), 256, 0, s>>>(nV, fc, F, FA, XVA, vcolor, muC, crec, cpen, ccount);
    return cudaGetLastError();
}

cudaError_t launch_unpack3(float4 const* in4, float* out3, int32_t n, cudaStream_t s, float4 const* origin)
{
    if (n <= 0)
        return cudaSuccess;
    unpack3_kernel<<<blocks_for(n, 256), 256, 0, s>>>(in4, out3, n, origin);
    return cudaGetLastError();
}

} // namespace pbgb
