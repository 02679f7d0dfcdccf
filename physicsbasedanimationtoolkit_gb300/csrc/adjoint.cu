// Adjoint sweep kernels (see adjoint.cuh).
#include "adjoint.cuh"

#include <cfloat>

namespace pbgb {

namespace {

__device__ __forceinline__ uint32_t corner_of(uint4 const& t, int a)
{
    return a == 0 ? t.x : (a == 1 ? t.y : (a == 2 ? t.z : t.w));
}

// One incidence of the reversed vertex: its tet, the three other corners' positions as the vertex
// saw them (lower colour rank: X_k, higher: X_{k-1}) relative to o's, and the rest edges.
struct AdjointIncidence
{
    int e;
    float4 mat;
    int j[3];
    float d[3][3];
    float E[3][3];
};

__device__ __forceinline__ void load_incidence(AdjointSweepParams const& p, uint32_t q, float4 const& pre, float4 const& Xo, AdjointIncidence& a)
{
    a.e                = int(q >> 2);
    int const il       = int(q & 3u);
    TetRecord const r  = p.tets[a.e];
    a.mat              = r.mat;
    uint32_t const rnk = corner_of(r.v, il) >> 30;
#pragma unroll
    for (int m = 0; m < 3; ++m)
    {
        uint32_t const ta = corner_of(r.v, (il + 1 + m) & 3);
        a.j[m]            = int(ta & kIndexMask);
        float4 const xa   = (ta >> 30) < rnk ? p.xk[a.j[m]] : p.xkm1[a.j[m]];
        float4 const Xa   = p.X[a.j[m]];
        a.d[m][0] = xa.x - pre.x, a.d[m][1] = xa.y - pre.y, a.d[m][2] = xa.z - pre.z;
        a.E[m][0] = Xa.x - Xo.x, a.E[m][1] = Xa.y - Xo.y, a.E[m][2] = Xa.z - Xo.z;
    }
}

// L lanes per vertex o of the colour, as in the forward sweep: lane l takes incidences l, l+L, ...
// Everything but o's own adjoint comes from the tape and the mesh tables, which no launch of the
// reversed step writes: the vertex's tape entries, its lane's first incidence and that
// incidence's w-independent terms (adjoint_tet_prepare) are formed before griddepcontrol.wait, so
// that with programmatic dependent launch they overlap the previous colour's tail; the adjoint is
// read, and the neighbours' adjoints and the tets' sensitivities written, only after it.
template <int L>
__global__ void __launch_bounds__(256) adjoint_sweep_kernel(AdjointSweepParams p)
{
    int const tid    = blockIdx.x * blockDim.x + threadIdx.x;
    int const s      = p.begin + tid / L;
    int const lane   = tid & (L - 1);
    bool const valid = s < p.end;
    float own[3]     = {0.f, 0.f, 0.f};
    float w[3]       = {0.f, 0.f, 0.f};
    int i = 0, k = 0, k1 = 0;
    float4 pre = make_float4(0.f, 0.f, 0.f, 0.f), pst = pre, Xo = pre, r0 = pre, r1 = pre;
    AdjointIncidence a;
    AdjointTetPre<float> q;
    float delta[3] = {0.f, 0.f, 0.f};
    bool has = false, skipped = true;
    if (valid)
    {
        i   = p.solve[s];
        pre = p.xkm1[i];
        pst = p.xk[i];
        Xo  = p.X[i];
        r0  = p.tape[2 * s];
        r1  = p.tape[2 * s + 1];
        k   = p.incPtr[s] + lane;
        k1  = p.incPtr[s + 1];
        has = k < k1;
        // The step was skipped (singular Newton matrix, tape entry zero): x_o' = x_o, and nothing
        // else of the update depends on its inputs.
        skipped = r0.x == 0.f && r0.w == 0.f && r1.y == 0.f;
        delta[0] = pre.x - pst.x, delta[1] = pre.y - pst.y, delta[2] = pre.z - pst.z;
        if (p.D != 0.f)
        {
            float4 const xs = p.xs[i];
            delta[0]        = (1.f + p.D) * delta[0] - p.D * (pre.x - xs.x);
            delta[1]        = (1.f + p.D) * delta[1] - p.D * (pre.y - xs.y);
            delta[2]        = (1.f + p.D) * delta[2] - p.D * (pre.z - xs.z);
        }
        if (skipped)
            has = false;
        // The first incidence's w-independent terms (positions, rest state, delta: all from the
        // tape and the tables) are formed before the wait as well.
        if (has)
        {
            load_incidence(p, p.inc[k], pre, Xo, a);
            float G[3][3];
            rest_gradients(a.E, G);
            adjoint_tet_prepare(a.d, a.E, G, delta, q);
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (valid)
    {
        float4 const u = p.ubar[i];
        // w = H^-1 u (symmetric: xx xy xz yy yz zz)
        w[0] = r0.x * u.x + r0.y * u.y + r0.z * u.z;
        w[1] = r0.y * u.x + r0.w * u.y + r1.x * u.z;
        w[2] = r0.z * u.x + r1.x * u.y + r1.y * u.z;
        while (has)
        {
            float c[3][3], dmu = 0.f, dla = 0.f;
            adjoint_tet_finish(q, w, delta, a.mat.x, a.mat.y, c, dmu, dla);
#pragma unroll
            for (int m = 0; m < 3; ++m)
            {
                atomicAdd(p.ubar + a.j[m], make_float4(-c[m][0], -c[m][1], -c[m][2], 0.f));
                own[0] += c[m][0];
                own[1] += c[m][1];
                own[2] += c[m][2];
            }
            // One corner of each tet per colour: this lane is the only writer of tet e here.
            p.dlogmu[a.e] -= double(dmu);
            p.dloglambda[a.e] -= double(dla);
            k += L;
            has = k < k1;
            if (has)
            {
                load_incidence(p, p.inc[k], pre, Xo, a);
                float G[3][3];
                rest_gradients(a.E, G);
                adjoint_tet_prepare(a.d, a.E, G, delta, q);
            }
        }
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            own[r] += __shfl_xor_sync(0xffffffffu, own[r], off);
    if (!valid || lane != 0 || skipped)
        return;
    // d(phi)/dx_o = K w + D H_e w - sum_e (own contributions) with K = m/h^2 from the inertia term
    // and H_e w = (u - K w)/(1 + D) from the damping term.
    float const K  = p.m[i] / p.h2;
    float4 const u = p.ubar[i];
    float dHw[3]   = {0.f, 0.f, 0.f};
    if (p.D != 0.f)
    {
        float const s = p.D / (1.f + p.D);
        dHw[0]        = s * (u.x - K * w[0]);
        dHw[1]        = s * (u.y - K * w[1]);
        dHw[2]        = s * (u.z - K * w[2]);
        float4 const q = p.xsbar[i];
        p.xsbar[i]     = make_float4(q.x + dHw[0], q.y + dHw[1], q.z + dHw[2], 0.f);
    }
    p.ubar[i] = make_float4(u.x - K * w[0] - dHw[0] + own[0], u.y - K * w[1] - dHw[1] + own[1],
                            u.z - K * w[2] - dHw[2] + own[2], 0.f);
    float4 const t = p.xtbar[i];
    p.xtbar[i]     = make_float4(t.x + K * w[0], t.y + K * w[1], t.z + K * w[2], 0.f);
}

__global__ void adjoint_begin_kernel(int32_t n, float const* __restrict__ xbar, float const* __restrict__ vbar, float4* __restrict__ ubar,
                                     float4* __restrict__ xtbar, float4* __restrict__ xsbar, float4* __restrict__ yp,
                                     float4* __restrict__ ypp, float invh)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    ubar[i] = make_float4(xbar[3 * i] + invh * vbar[3 * i], xbar[3 * i + 1] + invh * vbar[3 * i + 1],
                          xbar[3 * i + 2] + invh * vbar[3 * i + 2], 0.f);
    float4 const z = make_float4(0.f, 0.f, 0.f, 0.f);
    xtbar[i]       = z;
    xsbar[i]       = z;
    if (yp)
    {
        yp[i]  = z;
        ypp[i] = z;
    }
}

__global__ void adjoint_cheb_mix_kernel(int32_t n, float4* __restrict__ ubar, float4* __restrict__ yp, float4* __restrict__ ypp, float c1, float c2)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 const u = ubar[i], a = yp[i], b = ypp[i];
    float4 const y = make_float4(a.x + u.x, a.y + u.y, a.z + u.z, 0.f);
    ubar[i]        = make_float4(c1 * y.x, c1 * y.y, c1 * y.z, 0.f);
    yp[i]          = b;
    ypp[i]         = make_float4(c2 * y.x, c2 * y.y, c2 * y.z, 0.f);
}

__global__ void adjoint_end_kernel(int32_t n, float* __restrict__ xbar, float* __restrict__ vbar, float* __restrict__ pbar,
                                   float4 const* __restrict__ ubar, float4 const* __restrict__ xtbar,
                                   float4 const* __restrict__ xsbar, float4 const* __restrict__ v0,
                                   float4 const* __restrict__ p0, float4 const* __restrict__ a0, float h,
                                   int32_t strategy, int32_t gpuSemantics)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float const invh  = 1.f / h;
    float const s1    = strategy == 0 ? 0.f : 1.f;
    float4 const u    = ubar[i];
    float4 const t    = xtbar[i];
    float4 const q    = xsbar[i];
    float4 const v4   = v0[i];
    float4 const a4   = a0[i];
    float4 const m4   = gpuSemantics ? p0[i] : v4;
    float const uu[3] = {u.x, u.y, u.z};
    float const tt[3] = {t.x, t.y, t.z};
    float const qq[3] = {q.x, q.y, q.z};
    float const vt[3] = {v4.x, v4.y, v4.z};
    float const vm[3] = {m4.x, m4.y, m4.z};
    float const a[3]  = {a4.x, a4.y, a4.z};
    float dAv[3], dAvm[3];
    initial_position_factor_derivatives(vm, vt, a, h, strategy, FLT_MIN, dAv, dAvm);
    float const au = a[0] * uu[0] + a[1] * uu[1] + a[2] * uu[2];
    for (int r = 0; r < 3; ++r)
    {
        float const vb  = vbar[3 * i + r];
        float const pb  = pbar[3 * i + r];
        xbar[3 * i + r] = -invh * vb + uu[r] + tt[r] + qq[r];
        vbar[3 * i + r] = s1 * h * uu[r] + h * tt[r] + h * h * au * dAv[r] + (gpuSemantics ? pb : 0.f);
        pbar[3 * i + r] = h * h * au * dAvm[r];
    }
}

inline int blocks_of(int64_t n, int b)
{
    return int((n + b - 1) / b);
}

template <int L>
cudaError_t launch_l(AdjointSweepParams const& p, int block, bool pdl, cudaStream_t s)
{
    int64_t const n        = int64_t(p.end - p.begin) * L;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = dim3(unsigned(blocks_of(n, block)));
    cfg.blockDim           = dim3(unsigned(block));
    cfg.stream             = s;
    cudaLaunchAttribute attr[1];
    attr[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs                                          = attr;
    cfg.numAttrs                                       = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, adjoint_sweep_kernel<L>, p);
}

} // namespace

cudaError_t launch_adjoint_sweep(AdjointSweepParams const& p, int lanes, int block, bool pdl, cudaStream_t s)
{
    if (p.end <= p.begin)
        return cudaSuccess;
    if (block <= 0 || block > 256 || block % 32 != 0)
        return cudaErrorInvalidValue;
    switch (lanes)
    {
        case 1: return launch_l<1>(p, block, pdl, s);
        case 2: return launch_l<2>(p, block, pdl, s);
        case 4: return launch_l<4>(p, block, pdl, s);
        case 8: return launch_l<8>(p, block, pdl, s);
        case 16: return launch_l<16>(p, block, pdl, s);
        case 32: return launch_l<32>(p, block, pdl, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_adjoint_begin(int32_t n, float const* xbar, float const* vbar, float4* ubar, float4* xtbar, float4* xsbar,
                                 float4* yp, float4* ypp, float h, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    if ((yp == nullptr) != (ypp == nullptr))
        return cudaErrorInvalidValue;
    adjoint_begin_kernel<<<blocks_of(n, 256), 256, 0, s>>>(n, xbar, vbar, ubar, xtbar, xsbar, yp, ypp, 1.f / h);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_cheb_mix(int32_t n, float4* ubar, float4* yp, float4* ypp, float c1, float c2, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    adjoint_cheb_mix_kernel<<<blocks_of(n, 256), 256, 0, s>>>(n, ubar, yp, ypp, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_end(int32_t n, float* xbar, float* vbar, float* pbar, float4 const* ubar, float4 const* xtbar,
                               float4 const* xsbar, float4 const* v0, float4 const* p0, float4 const* a, float h,
                               int32_t strategy, int32_t gpuSemantics, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    adjoint_end_kernel<<<blocks_of(n, 256), 256, 0, s>>>(n, xbar, vbar, pbar, ubar, xtbar, xsbar, v0, p0, a, h, strategy,
                                                         gpuSemantics);
    return cudaGetLastError();
}

} // namespace pbgb
