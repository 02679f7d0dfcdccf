// C ABI of the LBVH (include/pbat_gb300.h, pbgb_bvh_*): a BVH object that owns its device arrays
// and a stream, built from host boxes; topology read-back and box-overlap queries for tests and
// for callers of the reference's gpu::geometry::Bvh (gpu/geometry/Bvh.cu).
#include "lbvh.cuh"
#include "pbat_gb300.h"

#include <cuda_runtime.h>

#include <cstdint>

#include <exception>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

thread_local std::string gBvhError;

struct CudaError
{
    cudaError_t e;
    char const* what;
};

void ck(cudaError_t e, char const* what)
{
    if (e != cudaSuccess)
        throw CudaError{e, what};
}

template <class T>
T* dalloc(size_t n)
{
    T* p = nullptr;
    if (n > 0)
        ck(cudaMalloc(reinterpret_cast<void**>(&p), n * sizeof(T)), "cudaMalloc");
    return p;
}

// A device array freed on scope exit (per-call staging of query inputs).
template <class T>
struct Scratch
{
    T* p = nullptr;
    explicit Scratch(size_t n) : p(dalloc<T>(n)) {}
    ~Scratch()
    {
        if (p)
            cudaFree(p);
    }
    Scratch(Scratch const&)            = delete;
    Scratch& operator=(Scratch const&) = delete;
};

// Host 3-vectors -> device float4 (w = 0), on the given stream.
void upload_points(float const* h3, int32_t n, float4* d, cudaStream_t s)
{
    if (n <= 0)
        return;
    std::vector<float4> tmp(static_cast<size_t>(n));
    for (int32_t i = 0; i < n; ++i)
        tmp[size_t(i)] = make_float4(h3[3 * size_t(i)], h3[3 * size_t(i) + 1], h3[3 * size_t(i) + 2], 0.f);
    ck(cudaMemcpyAsync(d, tmp.data(), sizeof(float4) * size_t(n), cudaMemcpyHostToDevice, s), "H2D");
    ck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

} // namespace

struct pbgb_bvh
{
    pbgb::BvhBuffers B{};
    int32_t n        = 0;
    int32_t capacity = 0;
    float4* lo       = nullptr; // unsorted input boxes
    float4* hi       = nullptr;
    float4* qlo      = nullptr; // query staging
    float4* qhi      = nullptr;
    int32_t qcap     = 0;
    int32_t* pairs   = nullptr;
    int64_t pcap     = 0;
    unsigned long long* count = nullptr;
    cudaStream_t stream       = nullptr;
    std::string error;

    ~pbgb_bvh()
    {
        if (stream)
            cudaStreamSynchronize(stream);
        pbgb::bvh_release(B);
        void* ptrs[] = {lo, hi, qlo, qhi, pairs, count};
        for (void* p : ptrs)
            if (p)
                cudaFree(p);
        if (stream)
            cudaStreamDestroy(stream);
    }

    void allocate(int32_t cap)
    {
        capacity = cap;
        size_t n = size_t(cap);
        ck(pbgb::bvh_allocate(B, cap), "cudaMalloc");
        lo       = dalloc<float4>(n);
        hi         = dalloc<float4>(n);
        count      = dalloc<unsigned long long>(1);
        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaMemsetAsync(B.flags, 0, sizeof(int32_t), stream), "cudaMemsetAsync");
    }

    void upload_boxes(int32_t m, float const* l3, float const* u3, float4*& dl, float4*& du)
    {
        std::vector<float4> hl(static_cast<size_t>(m)), hu(static_cast<size_t>(m));
        for (int32_t i = 0; i < m; ++i)
        {
            hl[i] = make_float4(l3[3 * size_t(i)], l3[3 * size_t(i) + 1], l3[3 * size_t(i) + 2], 0.f);
            hu[i] = make_float4(u3[3 * size_t(i)], u3[3 * size_t(i) + 1], u3[3 * size_t(i) + 2], 0.f);
        }
        ck(cudaMemcpyAsync(dl, hl.data(), sizeof(float4) * size_t(m), cudaMemcpyHostToDevice, stream), "H2D");
        ck(cudaMemcpyAsync(du, hu.data(), sizeof(float4) * size_t(m), cudaMemcpyHostToDevice, stream), "H2D");
        ck(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    int check_flags()
    {
        int32_t f = 0;
        ck(cudaMemcpyAsync(&f, B.flags, sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        if (f)
        {
            ck(cudaMemsetAsync(B.flags, 0, sizeof(int32_t), stream), "cudaMemsetAsync");
            error = (f & pbgb::kBvhErrStackOverflow) ? "BVH traversal stack (64) overflowed"
                                                      : "BVH deeper than 64 levels";
            return PBGB_ERR_INTERNAL;
        }
        return PBGB_OK;
    }
};

namespace {

int bvh_fail(pbgb_bvh* b, int code, std::string const& msg)
{
    gBvhError = msg;
    if (b)
        b->error = msg;
    return code;
}

template <class F>
int bvh_guard(pbgb_bvh* b, F&& f)
{
    try
    {
        return f();
    }
    catch (CudaError const& e)
    {
        return bvh_fail(b, PBGB_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
    }
    catch (std::bad_alloc const&)
    {
        return bvh_fail(b, PBGB_ERR_INTERNAL, "host allocation failed");
    }
    catch (std::exception const& e)
    {
        return bvh_fail(b, PBGB_ERR_INTERNAL, e.what());
    }
}

} // namespace

extern "C" {

PBGB_API int pbgb_bvh_create(int32_t capacity, pbgb_bvh** out)
{
    if (!out || capacity < 1 || capacity >= (1 << 30))
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_create: expected 1 <= capacity < 2^30");
    *out = nullptr;
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices < 1)
    {
        cudaGetLastError();
        return bvh_fail(nullptr, PBGB_ERR_NO_DEVICE, "no CUDA device available");
    }
    pbgb_bvh* b = new (std::nothrow) pbgb_bvh();
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INTERNAL, "host allocation failed");
    int const rc = bvh_guard(b, [&] {
        b->allocate(capacity);
        return int(PBGB_OK);
    });
    if (rc != PBGB_OK)
    {
        delete b;
        return rc;
    }
    *out = b;
    return PBGB_OK;
}

PBGB_API int pbgb_bvh_destroy(pbgb_bvh* b)
{
    delete b;
    return PBGB_OK;
}

PBGB_API int pbgb_bvh_build(pbgb_bvh* b, int32_t n, const float* lower, const float* upper, const float* wmin, const float* wmax)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (n < 1 || n > b->capacity || !lower || !upper || !wmin || !wmax)
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_build: expected 1 <= n <= capacity and non-null boxes");
    return bvh_guard(b, [&] {
        b->upload_boxes(n, lower, upper, b->lo, b->hi);
        b->n = n;
        ck(pbgb::bvh_build(b->B, n, b->lo, b->hi, make_float3(wmin[0], wmin[1], wmin[2]),
                           make_float3(wmax[0], wmax[1], wmax[2]), b->stream),
           "bvh_build");
        return b->check_flags();
    });
}

PBGB_API int pbgb_bvh_build_device(pbgb_bvh* b, int32_t n, const float* lower4, const float* upper4, const float* wmin, const float* wmax)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (n < 1 || n > b->capacity || !lower4 || !upper4 || !wmin || !wmax ||
        (reinterpret_cast<uintptr_t>(lower4) & 15u) || (reinterpret_cast<uintptr_t>(upper4) & 15u))
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT,
                        "pbgb_bvh_build_device: expected 1 <= n <= capacity and 16-byte aligned device boxes");
    return bvh_guard(b, [&] {
        b->n = n;
        ck(pbgb::bvh_build(b->B, n, reinterpret_cast<float4 const*>(lower4), reinterpret_cast<float4 const*>(upper4),
                           make_float3(wmin[0], wmin[1], wmin[2]), make_float3(wmax[0], wmax[1], wmax[2]), b->stream),
           "bvh_build");
        return int(PBGB_OK);
    });
}

PBGB_API int pbgb_bvh_stream(pbgb_bvh* b, void** stream)
{
    if (!b || !stream)
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "null argument");
    *stream = b->stream;
    return PBGB_OK;
}

PBGB_API int pbgb_bvh_refit(pbgb_bvh* b, const float* lower, const float* upper)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (b->n < 1 || !lower || !upper)
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_refit: build first; non-null boxes");
    return bvh_guard(b, [&] {
        b->upload_boxes(b->n, lower, upper, b->lo, b->hi);
        ck(pbgb::bvh_refit(b->B, b->n, b->lo, b->hi, b->stream), "bvh_refit");
        return b->check_flags();
    });
}

PBGB_API int pbgb_bvh_topology(
    pbgb_bvh* b,
    uint32_t* codes,
    int32_t* inds,
    int32_t* child,
    int32_t* parent,
    int32_t* rightmost,
    float* internal_lower,
    float* internal_upper)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (b->n < 1)
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_topology: build first");
    return bvh_guard(b, [&] {
        size_t const n = size_t(b->n), ni = n - 1;
        auto get = [&](void* dst, void const* src, size_t bytes) {
            if (dst && bytes)
                ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, b->stream), "D2H");
        };
        get(codes, b->B.codes, sizeof(uint32_t) * n);
        get(inds, b->B.inds, sizeof(int32_t) * n);
        get(child, b->B.child, sizeof(int32_t) * 2 * ni);
        get(parent, b->B.parent, sizeof(int32_t) * (2 * n - 1));
        get(rightmost, b->B.rightmost, sizeof(int32_t) * 2 * ni);
        // Internal node records come first: 2 float4 (lower | link, upper | link) per node.
        std::vector<float4> rec(2 * ni);
        if (ni && (internal_lower || internal_upper))
            get(rec.data(), b->B.nodes, sizeof(float4) * 2 * ni);
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        for (size_t i = 0; i < ni; ++i)
        {
            float4 const lo = rec[2 * i], hi = rec[2 * i + 1];
            if (internal_lower)
            {
                internal_lower[3 * i]     = lo.x;
                internal_lower[3 * i + 1] = lo.y;
                internal_lower[3 * i + 2] = lo.z;
            }
            if (internal_upper)
            {
                internal_upper[3 * i]     = hi.x;
                internal_upper[3 * i + 1] = hi.y;
                internal_upper[3 * i + 2] = hi.z;
            }
        }
        return int(PBGB_OK);
    });
}

PBGB_API int pbgb_bvh_overlaps(
    pbgb_bvh* b,
    int32_t nq,
    const float* qlower,
    const float* qupper,
    int32_t* pairs,
    int64_t capacity,
    int64_t* count)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (b->n < 1 || nq < 0 || (nq > 0 && (!qlower || !qupper)) || !count || capacity < 0 || (capacity > 0 && !pairs))
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_overlaps: invalid argument");
    return bvh_guard(b, [&] {
        if (nq > b->qcap)
        {
            if (b->qlo)
                cudaFree(b->qlo);
            if (b->qhi)
                cudaFree(b->qhi);
            b->qlo  = dalloc<float4>(size_t(nq));
            b->qhi  = dalloc<float4>(size_t(nq));
            b->qcap = nq;
        }
        if (capacity > b->pcap)
        {
            if (b->pairs)
                cudaFree(b->pairs);
            b->pairs = dalloc<int32_t>(2 * size_t(capacity));
            b->pcap  = capacity;
        }
        if (nq > 0)
            b->upload_boxes(nq, qlower, qupper, b->qlo, b->qhi);
        ck(pbgb::bvh_overlaps(pbgb::view_of(b->B, b->n), nq, b->qlo, b->qhi, b->pairs, capacity, b->count,
                              b->B.flags, b->stream),
           "bvh_overlaps");
        unsigned long long c = 0;
        ck(cudaMemcpyAsync(&c, b->count, sizeof(c), cudaMemcpyDeviceToHost, b->stream), "D2H");
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        int64_t const m = int64_t(c) < capacity ? int64_t(c) : capacity;
        if (m > 0)
            ck(cudaMemcpy(pairs, b->pairs, sizeof(int32_t) * 2 * size_t(m), cudaMemcpyDeviceToHost), "D2H");
        *count = int64_t(c);
        return b->check_flags();
    });
}

PBGB_API int pbgb_bvh_self_overlaps(pbgb_bvh* b, const int32_t* set, int32_t* pairs, int64_t capacity, int64_t* count)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (b->n < 1 || !count || capacity < 0 || (capacity > 0 && !pairs))
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_self_overlaps: invalid argument");
    return bvh_guard(b, [&] {
        if (capacity > b->pcap)
        {
            if (b->pairs)
                cudaFree(b->pairs);
            b->pairs = nullptr;
            b->pairs = dalloc<int32_t>(2 * size_t(capacity));
            b->pcap  = capacity;
        }
        Scratch<int32_t> dset{set ? size_t(b->n) : size_t(0)};
        if (set)
            ck(cudaMemcpyAsync(dset.p, set, sizeof(int32_t) * size_t(b->n), cudaMemcpyHostToDevice, b->stream), "H2D");
        ck(pbgb::bvh_self_overlaps(pbgb::view_of(b->B, b->n), set ? dset.p : nullptr, b->pairs, capacity, b->count,
                                   b->B.flags, b->stream),
           "bvh_self_overlaps");
        unsigned long long c = 0;
        ck(cudaMemcpyAsync(&c, b->count, sizeof(c), cudaMemcpyDeviceToHost, b->stream), "D2H");
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        int64_t const m = int64_t(c) < capacity ? int64_t(c) : capacity;
        if (m > 0)
            ck(cudaMemcpy(pairs, b->pairs, sizeof(int32_t) * 2 * size_t(m), cudaMemcpyDeviceToHost), "D2H");
        *count = int64_t(c);
        return b->check_flags();
    });
}

PBGB_API int pbgb_bvh_nearest_simplices(
    pbgb_bvh* b,
    int32_t nq,
    const float* X,
    int32_t nP,
    const float* P,
    int32_t nS,
    const int32_t* S,
    int32_t k,
    int32_t* nn)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (b->n < 1 || nq < 0 || (nq > 0 && (!X || !nn)) || nP < 1 || !P || nS != b->n || !S || (k != 3 && k != 4))
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT,
                        "pbgb_bvh_nearest_simplices: expected the built BVH's simplices (nS = boxes), k = 3 or 4");
    for (int64_t i = 0; i < int64_t(nS) * k; ++i)
        if (S[i] < 0 || S[i] >= nP)
            return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_nearest_simplices: simplex index out of range");
    return bvh_guard(b, [&] {
        Scratch<float4> dX{size_t(nq)}, dP{size_t(nP)};
        Scratch<int32_t> dS{size_t(nS) * size_t(k)}, dnn{size_t(nq)};
        upload_points(X, nq, dX.p, b->stream);
        upload_points(P, nP, dP.p, b->stream);
        ck(cudaMemcpyAsync(dS.p, S, sizeof(int32_t) * size_t(nS) * size_t(k), cudaMemcpyHostToDevice, b->stream), "H2D");
        ck(pbgb::bvh_nearest_simplices(pbgb::view_of(b->B, b->n), nq, dX.p, dP.p, dS.p, k, dnn.p, b->B.flags, b->stream),
           "bvh_nearest_simplices");
        if (nq > 0)
            ck(cudaMemcpyAsync(nn, dnn.p, sizeof(int32_t) * size_t(nq), cudaMemcpyDeviceToHost, b->stream), "D2H");
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        return b->check_flags();
    });
}

PBGB_API int pbgb_bvh_visits(pbgb_bvh* b, int32_t* visits)
{
    if (!b)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "null BVH");
    if (b->n < 1 || !visits)
        return bvh_fail(b, PBGB_ERR_INVALID_ARGUMENT, "pbgb_bvh_visits: invalid argument");
    return bvh_guard(b, [&] {
        if (b->n > 1)
            ck(cudaMemcpyAsync(visits, b->B.visits, sizeof(int32_t) * size_t(b->n - 1), cudaMemcpyDeviceToHost, b->stream),
               "D2H");
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        return int(PBGB_OK);
    });
}

PBGB_API int pbgb_simplex_boxes(int32_t nP, const float* P, int32_t nS, const int32_t* S, int32_t k, float* lower, float* upper)
{
    if (nP < 1 || !P || nS < 0 || (nS > 0 && (!S || !lower || !upper)) || k < 1 || k > 4)
        return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "pbgb_simplex_boxes: invalid argument");
    for (int64_t i = 0; i < int64_t(nS) * k; ++i)
        if (S[i] < 0 || S[i] >= nP)
            return bvh_fail(nullptr, PBGB_ERR_INVALID_ARGUMENT, "pbgb_simplex_boxes: simplex index out of range");
    try
    {
        cudaStream_t s = nullptr;
        ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
        struct StreamGuard
        {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } guard{s};
        Scratch<float4> dP{size_t(nP)}, lo{size_t(nS)}, hi{size_t(nS)};
        Scratch<int32_t> dS{size_t(nS) * size_t(k)};
        upload_points(P, nP, dP.p, s);
        if (nS > 0)
            ck(cudaMemcpyAsync(dS.p, S, sizeof(int32_t) * size_t(nS) * size_t(k), cudaMemcpyHostToDevice, s), "H2D");
        ck(pbgb::simplex_boxes(nS, k, dP.p, dS.p, lo.p, hi.p, s), "simplex_boxes");
        std::vector<float4> hl(static_cast<size_t>(nS)), hu(static_cast<size_t>(nS));
        if (nS > 0)
        {
            ck(cudaMemcpyAsync(hl.data(), lo.p, sizeof(float4) * size_t(nS), cudaMemcpyDeviceToHost, s), "D2H");
            ck(cudaMemcpyAsync(hu.data(), hi.p, sizeof(float4) * size_t(nS), cudaMemcpyDeviceToHost, s), "D2H");
        }
        ck(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        for (int32_t i = 0; i < nS; ++i)
        {
            lower[3 * size_t(i)] = hl[size_t(i)].x, lower[3 * size_t(i) + 1] = hl[size_t(i)].y, lower[3 * size_t(i) + 2] = hl[size_t(i)].z;
            upper[3 * size_t(i)] = hu[size_t(i)].x, upper[3 * size_t(i) + 1] = hu[size_t(i)].y, upper[3 * size_t(i) + 2] = hu[size_t(i)].z;
        }
        return PBGB_OK;
    }
    catch (CudaError const& e)
    {
        return bvh_fail(nullptr, PBGB_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
    }
    catch (std::exception const& e)
    {
        return bvh_fail(nullptr, PBGB_ERR_INTERNAL, e.what());
    }
}

PBGB_API const char* pbgb_bvh_last_error(pbgb_bvh* b)
{
    return b ? b->error.c_str() : gBvhError.c_str();
}

} // extern "C"
