// CPU restatement of the reference's GPU LBVH (TEST INFRASTRUCTURE ONLY; see vbd_oracle.cpp).
//
//   Morton codes      gpu/impl/geometry/Morton.cu:23-44, geometry/Morton.h:35-80
//   stable sort       gpu/impl/geometry/Bvh.cu:139-157 (thrust::stable_sort_by_key)
//   hierarchy         gpu/impl/geometry/Bvh.cu:24-114 (Karras 2012), restated top-down: the node
//                     covering sorted range [f, l] splits after the last key sharing more than
//                     delta(f, l) leading bits with key f; its index is the range end that the
//                     parallel construction assigns (root 0, left child = split, right child =
//                     split + 1, a one-element range is a leaf)
//   internal boxes    gpu/impl/geometry/Bvh.cu:175-229 (unions, exact)
//   overlap pairs     brute force over all (query, box) pairs (the set the BVH query must find)
//
// FP32 with the reference's operation order; this file is compiled with -ffp-contract=off.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

namespace {

uint32_t spread10(uint32_t v)
{
    // Bit k of v moves to bit 3k (plain loop; independent of the device's shift-or form).
    uint32_t r = 0;
    for (int k = 0; k < 10; ++k)
        r |= ((v >> k) & 1u) << (3 * k);
    return r;
}

uint32_t quantise(float c)
{
    float q = c * 1024.f;
    q       = std::min(std::max(q, 0.f), 1023.f);
    return static_cast<uint32_t>(q);
}

int clz64(uint64_t x)
{
    if (x == 0)
        return 64;
    int n = 0;
    while (!(x & (uint64_t(1) << 63)))
    {
        x <<= 1;
        ++n;
    }
    return n;
}

struct Builder
{
    std::vector<uint64_t> key; // (code << 32) | original index: the order of the stable sort
    int32_t n;
    int32_t* child;
    int32_t* parent;
    int32_t* rightmost;

    int delta(int32_t i, int32_t j) const { return clz64(key[i] ^ key[j]); }
};

// Top-down construction with explicit side tracking (recursion depth <= 64 for 64-bit keys).
int32_t build_range(Builder& B, int32_t f, int32_t l, int side)
{
    int32_t const leafBegin = B.n - 1;
    if (f == l)
        return leafBegin + f;
    int const dnode = B.delta(f, l);
    int32_t lo = f, hi = l;
    while (hi - lo > 1)
    {
        int32_t const mid = lo + (hi - lo) / 2;
        if (B.delta(f, mid) > dnode)
            lo = mid;
        else
            hi = mid;
    }
    int32_t const gamma = lo;
    int32_t const lc    = build_range(B, f, gamma, 0);
    int32_t const rc    = build_range(B, gamma + 1, l, 1);
    int32_t node        = (side < 0) ? 0 : (side == 0 ? l : f);
    B.child[2 * node]         = lc;
    B.child[2 * node + 1]     = rc;
    B.parent[lc]              = node;
    B.parent[rc]              = node;
    B.rightmost[2 * node]     = leafBegin + gamma;
    B.rightmost[2 * node + 1] = leafBegin + l;
    return node;
}

} // namespace

extern "C" {

// Morton codes of box centres normalised by [wmin, wmax].  lo, hi: n x 3.
void orc_morton(int32_t n, float const* lo, float const* hi, float const* wmin, float const* wmax, uint32_t* codes)
{
    float ext[3];
    for (int d = 0; d < 3; ++d)
        ext[d] = wmax[d] - wmin[d];
    for (int32_t i = 0; i < n; ++i)
    {
        uint32_t q[3];
        for (int d = 0; d < 3; ++d)
        {
            float const c = (0.5f * (lo[3 * size_t(i) + d] + hi[3 * size_t(i) + d]) - wmin[d]) / ext[d];
            q[d]          = quantise(c);
        }
        codes[i] = spread10(q[0]) * 4u + spread10(q[1]) * 2u + spread10(q[2]);
    }
}

// Full build.  Outputs: codes[n] and inds[n] in sorted order, child[2(n-1)], parent[2n-1],
// rightmost[2(n-1)], internal boxes ilo/ihi (n-1) x 3.
void orc_bvh_build(
    int32_t n,
    float const* lo,
    float const* hi,
    float const* wmin,
    float const* wmax,
    uint32_t* codes,
    int32_t* inds,
    int32_t* child,
    int32_t* parent,
    int32_t* rightmost,
    float* ilo,
    float* ihi)
{
    if (n <= 0)
        return;
    std::vector<uint32_t> raw(static_cast<size_t>(n));
    orc_morton(n, lo, hi, wmin, wmax, raw.data());
    std::vector<int32_t> order(static_cast<size_t>(n));
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return raw[a] < raw[b]; });
    for (int32_t s = 0; s < n; ++s)
    {
        codes[s] = raw[order[s]];
        inds[s]  = order[s];
    }
    std::fill(parent, parent + (2 * n - 1), -1);
    if (n < 2)
        return;
    Builder B;
    B.n         = n;
    B.child     = child;
    B.parent    = parent;
    B.rightmost = rightmost;
    B.key.resize(static_cast<size_t>(n));
    for (int32_t s = 0; s < n; ++s)
        B.key[s] = (uint64_t(codes[s]) << 32) | uint64_t(uint32_t(s));
    build_range(B, 0, n - 1, -1);
    // Internal boxes by a post-order pass (children before parents).
    int32_t const leafBegin = n - 1;
    std::vector<int32_t> stack{0};
    std::vector<char> done(static_cast<size_t>(n - 1), 0);
    while (!stack.empty())
    {
        int32_t const p = stack.back();
        int32_t const c[2] = {child[2 * p], child[2 * p + 1]};
        bool ready = true;
        for (int32_t q : c)
            if (q < leafBegin && !done[q])
            {
                stack.push_back(q);
                ready = false;
            }
        if (!ready)
            continue;
        stack.pop_back();
        for (int d = 0; d < 3; ++d)
        {
            float mn[2], mx[2];
            for (int k = 0; k < 2; ++k)
            {
                int32_t const q = c[k];
                if (q >= leafBegin)
                {
                    int32_t const box = inds[q - leafBegin];
                    mn[k]             = lo[3 * size_t(box) + d];
                    mx[k]             = hi[3 * size_t(box) + d];
                }
                else
                {
                    mn[k] = ilo[3 * size_t(q) + d];
                    mx[k] = ihi[3 * size_t(q) + d];
                }
            }
            ilo[3 * size_t(p) + d] = std::min(mn[0], mn[1]);
            ihi[3 * size_t(p) + d] = std::max(mx[0], mx[1]);
        }
        done[p] = 1;
    }
}

// Internal boxes for a given topology (child, inds) and leaf boxes lo/hi (n x 3, original order).
void orc_bvh_boxes(int32_t n, int32_t const* child, int32_t const* inds, float const* lo, float const* hi, float* ilo, float* ihi)
{
    if (n < 2)
        return;
    int32_t const leafBegin = n - 1;
    std::vector<int32_t> stack{0};
    std::vector<char> done(static_cast<size_t>(n - 1), 0);
    while (!stack.empty())
    {
        int32_t const p    = stack.back();
        int32_t const c[2] = {child[2 * p], child[2 * p + 1]};
        bool ready         = true;
        for (int32_t q : c)
            if (q < leafBegin && !done[q])
            {
                stack.push_back(q);
                ready = false;
            }
        if (!ready)
            continue;
        stack.pop_back();
        for (int d = 0; d < 3; ++d)
        {
            float mn[2], mx[2];
            for (int k = 0; k < 2; ++k)
            {
                int32_t const q = c[k];
                bool const leaf = q >= leafBegin;
                int32_t const r = leaf ? inds[q - leafBegin] : q;
                mn[k]           = leaf ? lo[3 * size_t(r) + d] : ilo[3 * size_t(r) + d];
                mx[k]           = leaf ? hi[3 * size_t(r) + d] : ihi[3 * size_t(r) + d];
            }
            ilo[3 * size_t(p) + d] = std::min(mn[0], mn[1]);
            ihi[3 * size_t(p) + d] = std::max(mx[0], mx[1]);
        }
        done[p] = 1;
    }
}

// All (query, box) pairs with overlapping closed boxes.  Returns the count; writes at most
// `capacity` pairs, ordered by query then box.  Every pair is decided by the full closed-box test;
// the boxes are only pre-sorted by their lower x so that each query tests the boxes whose lower x
// lies in [q.lo.x - w, q.hi.x] (w: the widest box in x, in FP64), which contains every box that
// can overlap it.  Queries run in parallel (OpenMP); each query's pairs are written at its prefix
// offset, so the output does not depend on threading.
int64_t orc_overlaps(int32_t n, float const* lo, float const* hi, int32_t nq, float const* qlo, float const* qhi, int32_t* pairs, int64_t capacity)
{
    auto overlap = [&](int32_t q, int32_t i) {
        bool ov = true;
        for (int d = 0; d < 3; ++d)
            ov = ov && qlo[3 * size_t(q) + d] <= hi[3 * size_t(i) + d] && lo[3 * size_t(i) + d] <= qhi[3 * size_t(q) + d];
        return ov;
    };
    std::vector<int32_t> order(size_t(std::max(n, 0)));
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return lo[3 * size_t(a)] < lo[3 * size_t(b)]; });
    std::vector<float> keys(order.size());
    double width = 0.0;
    for (size_t k = 0; k < order.size(); ++k)
    {
        keys[k] = lo[3 * size_t(order[k])];
        width   = std::max(width, double(hi[3 * size_t(order[k])]) - double(keys[k]));
    }
    auto candidates = [&](int32_t q, std::vector<int32_t>& hits) {
        hits.clear();
        double const from = double(qlo[3 * size_t(q)]) - width;
        auto b = std::lower_bound(keys.begin(), keys.end(), from, [](float k, double v) { return double(k) < v; });
        auto e = std::upper_bound(keys.begin(), keys.end(), qhi[3 * size_t(q)]);
        for (auto it = b; it < e; ++it)
        {
            int32_t const i = order[size_t(it - keys.begin())];
            if (overlap(q, i))
                hits.push_back(i);
        }
        std::sort(hits.begin(), hits.end());
    };
    std::vector<int64_t> start(size_t(nq) + 1, 0);
#pragma omp parallel
    {
        std::vector<int32_t> hits;
#pragma omp for schedule(dynamic, 64)
        for (int32_t q = 0; q < nq; ++q)
        {
            candidates(q, hits);
            start[size_t(q) + 1] = int64_t(hits.size());
        }
    }
    for (int32_t q = 0; q < nq; ++q)
        start[size_t(q) + 1] += start[size_t(q)];
#pragma omp parallel
    {
        std::vector<int32_t> hits;
#pragma omp for schedule(dynamic, 64)
        for (int32_t q = 0; q < nq; ++q)
        {
            int64_t k = start[size_t(q)];
            if (k >= capacity || start[size_t(q) + 1] == k)
                continue;
            candidates(q, hits);
            for (size_t j = 0; j < hits.size() && k < capacity; ++j, ++k)
            {
                pairs[2 * k]     = q;
                pairs[2 * k + 1] = hits[j];
            }
        }
    }
    return start[size_t(nq)];
}

// The same pairs by testing every (query, box) pair (used to check orc_overlaps).
int64_t orc_overlaps_all_pairs(int32_t n, float const* lo, float const* hi, int32_t nq, float const* qlo, float const* qhi, int32_t* pairs, int64_t capacity)
{
    int64_t count = 0;
    for (int32_t q = 0; q < nq; ++q)
        for (int32_t i = 0; i < n; ++i)
        {
            bool ov = true;
            for (int d = 0; d < 3; ++d)
                ov = ov && qlo[3 * size_t(q) + d] <= hi[3 * size_t(i) + d] && lo[3 * size_t(i) + d] <= qhi[3 * size_t(q) + d];
            if (ov)
            {
                if (count < capacity)
                {
                    pairs[2 * count]     = q;
                    pairs[2 * count + 1] = i;
                }
                ++count;
            }
        }
    return count;
}

} // extern "C"
