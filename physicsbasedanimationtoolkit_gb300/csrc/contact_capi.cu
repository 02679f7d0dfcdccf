// C ABI of the vertex-triangle contact detector on its own (pbgb_ccd_*), the counterpart of the
// reference's gpu::impl::contact::VertexTriangleMixedCcdDcd (gpu/impl/contact/
// VertexTriangleMixedCcdDcd.cu:17-223): initialise / update / finalise the active set for given
// positions and read the results back.
#include "contact.cuh"
#include "pbat_gb300.h"

#include <cuda_runtime.h>

#include <cfloat>
#include <exception>
#include <new>
#include <string>
#include <vector>

namespace {

thread_local std::string gCcdError;

struct CcdCudaError
{
    cudaError_t e;
    char const* what;
};

void cc(cudaError_t e, char const* what)
{
    if (e != cudaSuccess)
        throw CcdCudaError{e, what};
}

template <class T>
T* dnew(size_t n)
{
    T* p = nullptr;
    cc(cudaMalloc(reinterpret_cast<void**>(&p), (n > 0 ? n : 1) * sizeof(T)), "cudaMalloc");
    return p;
}

} // namespace

struct pbgb_ccd
{
    pbgb::ContactMesh M{};
    pbgb::ContactState S{};
    int32_t* V     = nullptr;
    int4* F        = nullptr;
    int32_t* B     = nullptr;
    float4* xt     = nullptr;
    float4* x      = nullptr;
    cudaStream_t stream = nullptr;
    std::string error;

    ~pbgb_ccd()
    {
        if (stream)
            cudaStreamSynchronize(stream);
        pbgb::bvh_release(S.bvh);
        void* ptrs[] = {V, F, B, xt, x, S.tlo, S.thi, S.vlo, S.vhi, S.active, S.dupper, S.av, S.nActive, S.nn, S.fc};
        for (void* p : ptrs)
            if (p)
                cudaFree(p);
        if (stream)
            cudaStreamDestroy(stream);
    }

    void upload(float const* h3, float4* d)
    {
        std::vector<float4> tmp(static_cast<size_t>(M.nV));
        for (int32_t i = 0; i < M.nV; ++i)
            tmp[i] = make_float4(h3[3 * size_t(i)], h3[3 * size_t(i) + 1], h3[3 * size_t(i) + 2], 0.f);
        cc(cudaMemcpyAsync(d, tmp.data(), sizeof(float4) * tmp.size(), cudaMemcpyHostToDevice, stream), "H2D");
        cc(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }
};

namespace {

int ccd_fail(pbgb_ccd* c, int code, std::string const& m)
{
    gCcdError = m;
    if (c)
        c->error = m;
    return code;
}

template <class F>
int ccd_guard(pbgb_ccd* c, F&& f)
{
    try
    {
        return f();
    }
    catch (CcdCudaError const& e)
    {
        return ccd_fail(c, PBGB_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
    }
    catch (std::exception const& e)
    {
        return ccd_fail(c, PBGB_ERR_INTERNAL, e.what());
    }
}

int ccd_flags(pbgb_ccd* c)
{
    int32_t f = 0;
    cc(cudaMemcpyAsync(&f, c->S.flags, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "D2H");
    cc(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (f)
    {
        cc(cudaMemset(c->S.flags, 0, sizeof(int32_t)), "cudaMemset");
        return ccd_fail(c, PBGB_ERR_INTERNAL, "BVH traversal stack overflow or tree deeper than 64 levels");
    }
    return PBGB_OK;
}

} // namespace

extern "C" {

PBGB_API int pbgb_ccd_create(int32_t nV, int32_t nSurfV, const int32_t* V, int32_t nF, const int32_t* F, const int32_t* B, pbgb_ccd** out)
{
    if (!out || nV < 1 || nSurfV < 0 || nF < 0 || (nSurfV > 0 && !V) || (nF > 0 && !F))
        return ccd_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "pbgb_ccd_create: invalid argument");
    *out = nullptr;
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices < 1)
    {
        cudaGetLastError();
        return ccd_fail(nullptr, PBGB_ERR_NO_DEVICE, "no CUDA device available");
    }
    for (int32_t q = 0; q < nSurfV; ++q)
        if (V[q] < 0 || V[q] >= nV)
            return ccd_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "collision vertex out of range");
    for (int64_t k = 0; k < int64_t(nF) * 3; ++k)
        if (F[k] < 0 || F[k] >= nV)
            return ccd_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "collision triangle index out of range");
    pbgb_ccd* c = new (std::nothrow) pbgb_ccd();
    if (!c)
        return ccd_fail(nullptr, PBGB_ERR_INTERNAL, "host allocation failed");
    int const rc = ccd_guard(c, [&] {
        cc(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        std::vector<int4> hF(static_cast<size_t>(nF));
        for (int32_t f = 0; f < nF; ++f)
            hF[f] = make_int4(F[3 * f], F[3 * f + 1], F[3 * f + 2], 0);
        std::vector<int32_t> hB(static_cast<size_t>(nV), 1);
        if (B)
            hB.assign(B, B + nV);
        std::vector<float> hD(static_cast<size_t>(nSurfV > 0 ? nSurfV : 1), FLT_MAX);
        c->V  = dnew<int32_t>(size_t(nSurfV));
        c->F  = dnew<int4>(size_t(nF));
        c->B  = dnew<int32_t>(size_t(nV));
        c->xt = dnew<float4>(size_t(nV));
        c->x  = dnew<float4>(size_t(nV));
        auto& S   = c->S;
        cc(pbgb::bvh_allocate(S.bvh, nF > 0 ? nF : 1), "cudaMalloc");
        S.tlo     = dnew<float4>(size_t(nF));
        S.thi     = dnew<float4>(size_t(nF));
        S.vlo     = dnew<float4>(size_t(nSurfV));
        S.vhi     = dnew<float4>(size_t(nSurfV));
        S.active  = dnew<uint8_t>(size_t(nSurfV));
        S.dupper  = dnew<float>(size_t(nSurfV));
        S.av      = dnew<int32_t>(size_t(nSurfV));
        S.nActive = dnew<int32_t>(1);
        S.nn      = dnew<int32_t>(size_t(nSurfV) * pbgb::kMaxContacts);
        S.fc      = dnew<int32_t>(size_t(nV) * pbgb::kMaxContacts);
        S.flags   = S.bvh.flags;
        if (nSurfV > 0)
            cc(cudaMemcpy(c->V, V, sizeof(int32_t) * size_t(nSurfV), cudaMemcpyHostToDevice), "H2D");
        if (nF > 0)
            cc(cudaMemcpy(c->F, hF.data(), sizeof(int4) * size_t(nF), cudaMemcpyHostToDevice), "H2D");
        cc(cudaMemcpy(c->B, hB.data(), sizeof(int32_t) * size_t(nV), cudaMemcpyHostToDevice), "H2D");
        cc(cudaMemcpy(S.dupper, hD.data(), sizeof(float) * hD.size(), cudaMemcpyHostToDevice), "H2D");
        cc(cudaMemset(S.active, 0, size_t(nSurfV > 0 ? nSurfV : 1)), "cudaMemset");
        cc(cudaMemset(S.nActive, 0, sizeof(int32_t)), "cudaMemset");
        cc(cudaMemset(S.nn, 0xFF, sizeof(int32_t) * size_t(nSurfV > 0 ? nSurfV : 1) * pbgb::kMaxContacts), "cudaMemset");
        cc(cudaMemset(S.fc, 0xFF, sizeof(int32_t) * size_t(nV) * pbgb::kMaxContacts), "cudaMemset");
        c->M = pbgb::ContactMesh{nV, nSurfV, nF, c->V, c->F, c->B};
        return int(PBGB_OK);
    });
    if (rc != PBGB_OK)
    {
        delete c;
        return rc;
    }
    *out = c;
    return PBGB_OK;
}

PBGB_API int pbgb_ccd_destroy(pbgb_ccd* c)
{
    delete c;
    return PBGB_OK;
}

PBGB_API int pbgb_ccd_initialize(pbgb_ccd* c, const float* xt, const float* x, const float* wmin, const float* wmax)
{
    if (!c || !xt || !x || !wmin || !wmax)
        return ccd_fail(c, PBGB_ERR_INVALID_ARGUMENT, "pbgb_ccd_initialize: null argument");
    return ccd_guard(c, [&] {
        c->upload(xt, c->xt);
        c->upload(x, c->x);
        cc(pbgb::contact_initialize(c->M, c->S, c->xt, c->x, make_float3(wmin[0], wmin[1], wmin[2]),
                                    make_float3(wmax[0], wmax[1], wmax[2]), c->stream),
           "contact_initialize");
        return ccd_flags(c);
    });
}

PBGB_API int pbgb_ccd_update(pbgb_ccd* c, const float* x)
{
    if (!c || !x)
        return ccd_fail(c, PBGB_ERR_INVALID_ARGUMENT, "pbgb_ccd_update: null argument");
    return ccd_guard(c, [&] {
        c->upload(x, c->x);
        cc(pbgb::contact_update(c->M, c->S, c->x, c->stream), "contact_update");
        return ccd_flags(c);
    });
}

PBGB_API int pbgb_ccd_finalize(pbgb_ccd* c, const float* x)
{
    if (!c || !x)
        return ccd_fail(c, PBGB_ERR_INVALID_ARGUMENT, "pbgb_ccd_finalize: null argument");
    return ccd_guard(c, [&] {
        c->upload(x, c->x);
        cc(pbgb::contact_finalize(c->M, c->S, c->x, c->stream), "contact_finalize");
        return ccd_flags(c);
    });
}

PBGB_API int pbgb_ccd_get(pbgb_ccd* c, uint8_t* active, int32_t* nn, float* dupper, int32_t* n_active)
{
    if (!c)
        return ccd_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null detector");
    return ccd_guard(c, [&] {
        size_t const nS = size_t(c->M.nSurfV);
        cc(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
        if (active && nS)
            cc(cudaMemcpy(active, c->S.active, nS, cudaMemcpyDeviceToHost), "D2H");
        if (nn && nS)
            cc(cudaMemcpy(nn, c->S.nn, sizeof(int32_t) * nS * pbgb::kMaxContacts, cudaMemcpyDeviceToHost), "D2H");
        if (dupper && nS)
            cc(cudaMemcpy(dupper, c->S.dupper, sizeof(float) * nS, cudaMemcpyDeviceToHost), "D2H");
        if (n_active)
            cc(cudaMemcpy(n_active, c->S.nActive, sizeof(int32_t), cudaMemcpyDeviceToHost), "D2H");
        return int(PBGB_OK);
    });
}

PBGB_API const char* pbgb_ccd_last_error(pbgb_ccd* c)
{
    return c ? c->error.c_str() : gCcdError.c_str();
}

} // extern "C"
