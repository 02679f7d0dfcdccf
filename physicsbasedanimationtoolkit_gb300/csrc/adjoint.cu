// Adjoint sweep kernels (see adjoint.cuh).
#include "adjoint.cuh"

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
// reversed step writes: the vertex's tape entries and its lane's first incidence are loaded before
// griddepcontrol.wait, so that with programmatic dependent launch they overlap the previous
// colour's tail; the adjoint is read, and the neighbours' adjoints and the tets' sensitivities
// written, only after it.
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
    bool has = false;
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
        if (has)
            load_incidence(p, p.inc[k], pre, Xo, a);
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
        float const delta[3] = {pre.x - pst.x, pre.y - pst.y, pre.z - pst.z};
        while (has)
        {
            float G[3][3];
            rest_gradients(a.E, G);
            float c[3][3], dmu = 0.f, dla = 0.f;
            adjoint_tet(a.d, a.E, G, w, delta, a.mat.x, a.mat.y, c, dmu, dla);
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
                load_incidence(p, p.inc[k], pre, Xo, a);
        }
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            own[r] += __shfl_xor_sync(0xffffffffu, own[r], off);
    if (!valid || lane != 0)
        return;
    // d(phi)/dx_o = K w - sum_e (own contributions) with K = m/h^2 from the inertia term.
    float const K  = p.m[i] / p.h2;
    float4 const u = p.ubar[i];
    p.ubar[i]      = make_float4(u.x - K * w[0] + own[0], u.y - K * w[1] + own[1], u.z - K * w[2] + own[2], 0.f);
    float4 const t = p.xtbar[i];
    p.xtbar[i]     = make_float4(t.x + K * w[0], t.y + K * w[1], t.z + K * w[2], 0.f);
}

__global__ void adjoint_begin_kernel(int32_t n, float const* __restrict__ xbar, float const* __restrict__ vbar, float4* __restrict__ ubar, float4* __restrict__ xtbar, float invh)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    ubar[i] = make_float4(xbar[3 * i] + invh * vbar[3 * i], xbar[3 * i + 1] + invh * vbar[3 * i + 1],
                          xbar[3 * i + 2] + invh * vbar[3 * i + 2], 0.f);
    xtbar[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void adjoint_end_kernel(int32_t n, float* __restrict__ xbar, float* __restrict__ vbar, float4 const* __restrict__ ubar, float4 const* __restrict__ xtbar, float h, float s1)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float const invh = 1.f / h;
    float4 const u   = ubar[i];
    float4 const t   = xtbar[i];
    float const uu[3] = {u.x, u.y, u.z};
    float const tt[3] = {t.x, t.y, t.z};
    for (int r = 0; r < 3; ++r)
    {
        float const vb   = vbar[3 * i + r];
        xbar[3 * i + r]  = -invh * vb + uu[r] + tt[r];
        vbar[3 * i + r]  = s1 * h * uu[r] + h * tt[r];
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

cudaError_t launch_adjoint_begin(int32_t n, float const* xbar, float const* vbar, float4* ubar, float4* xtbar, float h, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    adjoint_begin_kernel<<<blocks_of(n, 256), 256, 0, s>>>(n, xbar, vbar, ubar, xtbar, 1.f / h);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_end(int32_t n, float* xbar, float* vbar, float4 const* ubar, float4 const* xtbar, float h, float s1, cudaStream_t s)
{
    if (n <= 0)
        return cudaSuccess;
    adjoint_end_kernel<<<blocks_of(n, 256), 256, 0, s>>>(n, xbar, vbar, ubar, xtbar, h, s1);
    return cudaGetLastError();
}

} // namespace pbgb
