// The VBD integrator object behind the C ABI (include/pbat_gb300.h): device layout, step
// orchestration captured in CUDA graphs, host/device copies, and the extern "C" entry points.
//
// Reference counterpart: pbat::gpu::impl::vbd::Integrator (gpu/impl/vbd/Integrator.cu:22-347)
// and the public pimpl pbat::gpu::vbd::Integrator (gpu/vbd/Integrator.cu).  Differences by design:
// one stream per handle (the reference creates one and never uses it), the whole step replayed
// from a CUDA graph, tets packed into 64-byte records, the in-place colour sweep (no xb copy-back
// pass), and several meshes concatenated into one system for the batched form.
#include "adjoint.cuh"
#include "batched.cuh"
#include "anderson.cuh"
#include "nesterov.cuh"
#include "trust_region.cuh"
#include "contact.cuh"
#include "pbat_gb300.h"
#include "vbd_construct.h"
#include "vbd_kernels.cuh"

#include <cfloat>

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <exception>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

namespace pbgb {

namespace {

thread_local std::string gLastError;

struct CudaFailure
{
    cudaError_t err;
    char const* what;
};

inline void check(cudaError_t e, char const* what)
{
    if (e != cudaSuccess)
        throw CudaFailure{e, what};
}

template <class T>
class DeviceArray
{
  public:
    DeviceArray() = default;
    DeviceArray(DeviceArray const&) = delete;
    DeviceArray& operator=(DeviceArray const&) = delete;
    ~DeviceArray() { release(); }
    void allocate(size_t n)
    {
        release();
        n_ = n;
        if (n > 0)
            check(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)), "cudaMalloc");
    }
    void upload(T const* h, size_t n, cudaStream_t s)
    {
        if (n > 0)
            check(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync H2D");
    }
    void release()
    {
        if (p_)
            cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    T* get() const { return p_; }
    size_t size() const { return n_; }

  private:
    T* p_     = nullptr;
    size_t n_ = 0;
};

} // namespace

// Host checks of a batch of descriptors, before any device work (the reference validates in
// Data::Construct, sim/vbd/Data.cpp:259-305): present and in-range fields, finite and positive
// physical inputs, and a valid colouring -- every free vertex in exactly one partition, and no two
// free vertices of one colour in the same tet (the sweep updates a colour's vertices in place and
// relies on it).
inline void validate_descs(pbgb_vbd_desc const* descs, int32_t nMeshes)
{
    auto bad = [](std::string const& what) { throw std::invalid_argument("pbgb_vbd_desc: " + what); };
    auto finite = [](double const* a, int64_t n) {
        for (int64_t k = 0; k < n; ++k)
            if (!std::isfinite(a[k]))
                return false;
        return true;
    };
    int64_t totV = 0, totT = 0;
    for (int32_t b = 0; b < nMeshes; ++b)
    {
        auto const& d = descs[b];
        if (d.n_vertices < 0 || d.n_tets < 0 || !d.x || (d.n_tets > 0 && !d.T) || !d.m ||
            (d.n_tets > 0 && (!d.wg || !d.mu || !d.lambda)) || d.n_partitions < 0 ||
            d.n_partitions > kMaxColors || !d.Pptr || (d.Pptr[d.n_partitions] > 0 && !d.Padj))
            bad("missing or invalid field");
        int64_t const n3 = 3 * int64_t(d.n_vertices);
        if (!finite(d.x, n3) || (d.X && !finite(d.X, n3)) || (d.v && !finite(d.v, n3)) ||
            (d.aext && !finite(d.aext, n3)))
            bad("non-finite positions, velocities or accelerations");
        for (int32_t i = 0; i < d.n_vertices; ++i)
            if (!(d.m[i] >= 0.0) || !std::isfinite(d.m[i]))
                bad("masses must be finite and non-negative");
        for (int32_t e = 0; e < d.n_tets; ++e)
            if (!(d.wg[e] > 0.0) || !(d.mu[e] > 0.0) || !(d.lambda[e] > 0.0) || !std::isfinite(d.wg[e]) ||
                !std::isfinite(d.mu[e]) || !std::isfinite(d.lambda[e]))
                bad("quadrature weights and Lame coefficients must be finite and positive");
        if (!std::isfinite(d.kD) || d.kD < 0.0 || !std::isfinite(d.detHZero) || d.detHZero < 0.0)
            bad("damping and the Hessian determinant threshold must be finite and non-negative");
        for (int64_t k = 0; k < int64_t(d.n_tets) * 4; ++k)
            if (d.T[k] < 0 || d.T[k] >= d.n_vertices)
                bad("tetrahedron index out of range");
        if (d.Pptr[0] != 0)
            bad("partition pointers must start at 0");
        for (int32_t c = 0; c < d.n_partitions; ++c)
            if (d.Pptr[c + 1] < d.Pptr[c])
                bad("partition pointers must not decrease");
        std::vector<int32_t> colour(static_cast<size_t>(d.n_vertices), -1);
        for (int32_t c = 0; c < d.n_partitions; ++c)
            for (int32_t k = d.Pptr[c]; k < d.Pptr[c + 1]; ++k)
            {
                int32_t const v = d.Padj[k];
                if (v < 0 || v >= d.n_vertices)
                    bad("partition vertex out of range");
                if (colour[v] >= 0)
                    bad("a vertex appears in more than one partition");
                colour[v] = c;
            }
        for (int32_t e = 0; e < d.n_tets; ++e)
        {
            int32_t const* t = d.T + 4 * size_t(e);
            for (int a = 0; a < 4; ++a)
                for (int q = a + 1; q < 4; ++q)
                {
                    if (t[a] == t[q])
                        bad("a tetrahedron repeats a vertex");
                    if (colour[t[a]] >= 0 && colour[t[a]] == colour[t[q]])
                        bad("invalid colouring: two vertices of one colour share a tetrahedron");
                }
        }
        if (d.acceleration == PBGB_ACCEL_CHEBYSHEV && !(d.rho > 0.0 && d.rho < 1.0))
            throw std::invalid_argument("Expected 0 < rho < 1");
        if (d.acceleration != PBGB_ACCEL_NONE && d.acceleration != PBGB_ACCEL_CHEBYSHEV &&
            d.acceleration != PBGB_ACCEL_ANDERSON && d.acceleration != PBGB_ACCEL_NESTEROV &&
            d.acceleration != PBGB_ACCEL_BROYDEN && d.acceleration != PBGB_ACCEL_TRUST_REGION)
            bad("unsupported acceleration strategy");
        if (d.acceleration == PBGB_ACCEL_TRUST_REGION)
        {
            if (!(d.tr_eta >= 0.0) || !std::isfinite(d.tr_eta) || !(d.tr_tau > 1.0) || !std::isfinite(d.tr_tau))
                bad("trust-region acceleration expects eta >= 0 and tau > 1");
            if (nMeshes != 1)
                bad("trust-region acceleration needs a single mesh");
        }
        if (d.acceleration == PBGB_ACCEL_NESTEROV &&
            (!(d.nesterov_lipschitz > 0.0) || !std::isfinite(d.nesterov_lipschitz) || d.nesterov_start < 0))
            bad("Nesterov acceleration expects L > 0 and start >= 0");
        if (d.acceleration == PBGB_ACCEL_NESTEROV && (nMeshes != 1 || d.n_collision_triangles > 0))
            bad("Nesterov acceleration needs a single mesh without contact");
        if (d.acceleration == PBGB_ACCEL_ANDERSON || d.acceleration == PBGB_ACCEL_BROYDEN)
        {
            char const* name = d.acceleration == PBGB_ACCEL_ANDERSON ? "Anderson" : "Broyden";
            if (d.window_size < 1 || d.window_size > kAndersonMaxWindow)
                bad(std::string(name) + " window must be in [1, 16]");
            // The reference's GPU integrator runs Anderson with contact; Broyden is a CPU-integrator
            // strategy, whose integrator has no contact.
            if (nMeshes != 1 || (d.acceleration == PBGB_ACCEL_BROYDEN && d.n_collision_triangles > 0))
                bad(std::string(name) + (d.acceleration == PBGB_ACCEL_BROYDEN ? " acceleration needs a single mesh without contact"
                                                                              : " acceleration needs a single mesh"));
        }
        if (d.init_strategy < 0 || d.init_strategy > 4)
            bad("invalid initialization strategy");
        if (d.n_collision_triangles > 0)
        {
            if (d.n_collision_vertices <= 0 || !d.V || !d.F || !d.XVA || !d.FA)
                bad("contact needs V, F, XVA and FA");
            for (int32_t k = 0; k < d.n_collision_vertices; ++k)
                if (d.V[k] < 0 || d.V[k] >= d.n_vertices)
                    bad("collision vertex out of range");
            for (int64_t k = 0; k < 3 * int64_t(d.n_collision_triangles); ++k)
                if (d.F[k] < 0 || d.F[k] >= d.n_vertices)
                    bad("collision triangle index out of range");
            for (int32_t i = 0; i < d.n_vertices; ++i)
                if (!(d.XVA[i] >= 0.0) || !std::isfinite(d.XVA[i]))
                    bad("vertex areas must be finite and non-negative");
            for (int32_t f = 0; f < d.n_collision_triangles; ++f)
                if (!(d.FA[f] >= 0.0) || !std::isfinite(d.FA[f]))
                    bad("triangle areas must be finite and non-negative");
            if (!(d.muC >= 0.0) || !(d.muF >= 0.0) || !(d.epsv > 0.0))
                bad("contact parameters must satisfy muC >= 0, muF >= 0, epsv > 0");
            if (d.active_set_update_frequency < 1)
                bad("active set update frequency must be >= 1");
            if (nMeshes != 1)
                bad("contact is supported on a single (non-batched) mesh");
        }
        totV += d.n_vertices;
        totT += d.n_tets;
    }
    if (totV > INT32_MAX || totT >= (int64_t(1) << 30) || totT * 4 > INT32_MAX)
        bad("system too large for 32-bit indexing");
}

class VbdSystem
{
  public:
    // Host metadata
    int32_t nV = 0, nT = 0, nFree = 0, nColors = 0;
    std::vector<int32_t> colorPtr; // solve-list ranges per colour
    double meanDegree = 0.0;
    int32_t strategy  = PBGB_INIT_ADAPTIVE_PBAT;
    float kD = 0.f, detHZero = 1e-7f;
    int32_t acceleration = PBGB_ACCEL_NONE, chebFormula = PBGB_CHEBYSHEV_REFERENCE, semantics = 0;
    int32_t window = 0; // Anderson / Broyden window
    double nesterovL = 1.0;
    int32_t nesterovStart = 3;
    double trEta = 0.2, trTau = 2.0;
    bool trCurved = true;
    double rho  = 1.0;
    int32_t lanes = 0, block = 256;
    bool pdl   = true;
    int device = 0;
    float sceneMin[3] = {0, 0, 0}, sceneMax[3] = {0, 0, 0};
    std::string lastError;

    // Device state
    cudaStream_t stream = nullptr;
    DeviceArray<float4> x, xt, xtilde, v, aext, vprev, h0, h1, X;
    // Anderson acceleration: the sweep's increments (zero for pinned vertices), last un-accelerated
    // iterate and residual, the window columns, FP64 block partials, Gram matrix and coefficients.
    DeviceArray<float4> anStep, anGkm1, anFkm1, anDF, anDG;
    DeviceArray<double> anPartials, anGram, anRhs, anAlpha;
    // Nesterov acceleration: the solve's start iterate and the extrapolated point.
    DeviceArray<float4> neX0, neY;
    // Trust-region acceleration (linear path): x_{k-1}, the device-resident scalars and the
    // reduction partials.
    DeviceArray<float4> trXkm1;
    DeviceArray<TrustState> trState;
    DeviceArray<double> trPartials, trLog;
    int32_t trLogEntries = 0; // entries the last enqueued step writes
    DeviceArray<float> m, staging;
    DeviceArray<TetRecord> tets;
    DeviceArray<int32_t> solve, incPtr, flags;
    DeviceArray<uint32_t> inc;
    // Staged sweep: per free vertex its distinct neighbours, per incidence (tet, neighbour slots),
    // per tet its material words.  stagedOk is false when some vertex has more than 256
    // neighbours (slots are bytes); `staged` is the user's choice.
    bool stagedOk = false, staged = true;
    std::vector<int32_t> hostNbrPtr;
    DeviceArray<int32_t> nbrPtr;
    DeviceArray<uint32_t> nbr;
    DeviceArray<uint2> incPack;
    // Per-incidence stiffness of the sweeps (TetStiffness resolved for the incidence's own corner):
    // incStiff[k] = (b0, b1, b2, kappa_o) and incPack[k].y = sigma.  Host copies of the incidence
    // words and neighbour slots let pbgb_vbd_set_material rebuild them.
    DeviceArray<float4> incStiff;
    std::vector<uint32_t> hostInc, hostSlots;
    DeviceArray<double> red, gradBuf, objPartials;

    // Sweep timing: with `profiling` on, the captured step records an event pair around the colour
    // sweeps of every iteration (event-record nodes in the graph).
    bool profiling = false;
    std::vector<cudaEvent_t> evBegin, evEnd;

    // Vertex-triangle contact (single mesh with a collision surface).
    bool contact = false;
    float muC = 1e6f, muF = 0.3f, epsv = 1e-3f;
    int32_t activeSetFreq = 1;
    ContactMesh cmesh{};
    ContactState cstate{};
    DeviceArray<int32_t> cV, cB, vcolorD, cAv, cNActive, cNn, cFc, cFlags;
    DeviceArray<int4> cF, cRec;
    DeviceArray<float> cPen;
    DeviceArray<int32_t> cCount; // listed triangles per vertex (its records come first)
    DeviceArray<float> cXVA, cFA, cDupper;
    DeviceArray<float4> cTlo, cThi, cVlo, cVhi, xpred;
    DeviceArray<uint8_t> cActive;

    // Host copies of the tet records and quadrature weights (pbgb_vbd_set_material rewrites the
    // material words).
    std::vector<TetRecord> hostRecords;
    std::vector<double> hostWg;
    // Host copies for the descent-path traces: lumped masses, Lame coefficients and the
    // shape-function gradients (row-major 4x3 per tet; from the descriptor's GP when given, else
    // from the rest positions).
    std::vector<double> hostM, hostMu, hostLambda, hostGP;

    // The next step is traced in the CPU integrator's format (pbgb_vbd_trace_next_step).
    bool traceNext = false;
    std::string tracePath;
    int32_t traceStep = -1;

    // Adjoint tape (pbgb_vbd_adjoint_reserve): one slot per recorded substep, holding the iterates
    // X_0..X_K (nV float4 each) and K x nFree inverse Newton matrices (2 float4 each).
    int32_t tapeSlots = 0, tapeIters = 0;
    std::vector<float> slotH;
    std::vector<int32_t> slotStrategy;
    DeviceArray<float4> tapeX, tapeH, ubar, xtbar;
    // Per slot: the substep's start positions, velocities and previous velocities (3 nV float4),
    // and with Chebyshev the raw sweep result of every iteration (K nV float4).  Reversal buffers:
    // the damping term's adjoint of the start positions and the Chebyshev carries.
    DeviceArray<float4> tapeS, tapeRaw, xsbar, ycarry, ycarry2;
    std::vector<float> slotKD;
    // Reversed steps run on these (the caller's arrays are copied in and out), so that their graphs
    // do not depend on the caller's pointers.
    DeviceArray<float> adjX, adjV, adjP, adjZero;
    DeviceArray<double> adjMu, adjLa;

    // Batch layout: mesh b's vertices are [meshV0[b], meshV0[b+1]); its free vertices of colour c
    // are solve entries [meshSolve[b][2c], meshSolve[b][2c+1]) (inside colour c of the system,
    // meshes in order).
    int32_t nMeshes = 1;
    std::vector<int32_t> meshV0;
    // Positions are stored relative to their mesh's origin (the centre of its rest box, rounded to
    // FP32), so that FP32 differences of nearby positions keep their precision however far from the
    // world origin a mesh lies; the position entry points add and subtract it.  A mesh with contact
    // uses the world frame (its boxes, Morton codes and scene box are world quantities): origin is
    // empty then.
    std::vector<float4> meshOrigin;
    DeviceArray<float4> origin;
    std::vector<std::vector<int32_t>> meshSolve;
    // Persistent batched step (batched.cuh): on for batches by default.  The work items are
    // rebuilt when the step shape or the launch changes.
    bool persistent = true;
    struct PersistentPlan
    {
        int32_t iters = -1, sub = -1, lanes = 0, block = 0, tile = 0;
        float dt      = 0.f;
        int32_t nItems = 0, grid = 0;
        size_t smem = 0;
    } plan;
    int32_t batchTile = 1; // sub-tiles of blockDim / lanes vertices per sweep item
    long long batchWaitNs = kBatchWaitNs;
    int32_t batchPoison   = -1;
    DeviceArray<BatchItemWords> batchItems;
    DeviceArray<int32_t> batchCounters; // [0] ticket, [1] abort, then one completion counter per mesh
    DeviceArray<float> batchOmega;

    // Graph cache for Step(dt, iterations, substeps)
    cudaGraphExec_t graph = nullptr;
    float gDt = -1.f;
    int32_t gIters = -1, gSub = -1;
    bool graphValid = false;
    int64_t graphKernels = -1; // kernel nodes of the step graph last captured

    ~VbdSystem()
    {
        if (stream)
            cudaStreamSynchronize(stream);
        bvh_release(cstate.bvh);
        releaseEvents();
        dropSlotGraphs();
        if (graph)
            cudaGraphExecDestroy(graph);
        if (stream)
            cudaStreamDestroy(stream);
    }

    void invalidate()
    {
        graphValid = false;
        dropSlotGraphs();
    }

    // Graphs of recorded and reversed steps, one per first slot (captured on first use).
    struct SlotGraph
    {
        cudaGraphExec_t exec = nullptr;
        float dt             = 0.f;
        int32_t iters = -1, sub = -1;
        std::vector<float> h; // reversed steps: the step size of every covered slot
        std::vector<int32_t> strategy;
        std::vector<float> kd;
    };
    std::vector<SlotGraph> recGraphs, adjGraphs;

    void dropSlotGraphs()
    {
        for (auto* v : {&recGraphs, &adjGraphs})
        {
            for (auto& g : *v)
                if (g.exec)
                    cudaGraphExecDestroy(g.exec);
            v->clear();
        }
    }

    // Captures what `enqueue` puts on the stream into an executable graph.
    template <class F>
    cudaGraphExec_t capture(F&& enqueue)
    {
        cudaGraph_t g = nullptr;
        check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        try
        {
            enqueue();
        }
        catch (...)
        {
            cudaStreamEndCapture(stream, &g);
            if (g)
                cudaGraphDestroy(g);
            throw;
        }
        check(cudaStreamEndCapture(stream, &g), "cudaStreamEndCapture");
        cudaGraphExec_t exec = nullptr;
        cudaError_t const e  = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        check(e, "cudaGraphInstantiate");
        return exec;
    }

    void releaseEvents()
    {
        for (auto e : evBegin)
            cudaEventDestroy(e);
        for (auto e : evEnd)
            cudaEventDestroy(e);
        evBegin.clear();
        evEnd.clear();
    }

    void ensureEvents(size_t n)
    {
        while (evBegin.size() < n)
        {
            cudaEvent_t a = nullptr, b = nullptr;
            check(cudaEventCreate(&a), "cudaEventCreate");
            evBegin.push_back(a);
            check(cudaEventCreate(&b), "cudaEventCreate");
            evEnd.push_back(b);
        }
    }

    // Sum of the sweep intervals of the last replayed step (stream must be idle).
    double sweepMilliseconds(int32_t iterations, int32_t substeps)
    {
        double total = 0.0;
        size_t const n = size_t(iterations) * size_t(substeps);
        for (size_t k = 0; k < n && k < evBegin.size(); ++k)
        {
            float ms = 0.f;
            check(cudaEventElapsedTime(&ms, evBegin[k], evEnd[k]), "cudaEventElapsedTime");
            total += ms;
        }
        return total;
    }

    // Staged-sweep fields of a SweepParams, and the shared memory of colour c's launch (0: gather).
    void stagedFields(SweepParams& w) const
    {
        w.nbrPtr  = nbrPtr.get();
        w.nbr     = nbr.get();
        w.incPack = incPack.get();
    }
    size_t stagedBytes(int32_t c, int L) const
    {
        if (!stagedOk || !staged)
            return 0;
        size_t const bytes = staged_sweep_bytes(hostNbrPtr.data(), colorPtr[c], colorPtr[c + 1], L, block);
        return bytes <= kStagedMaxBytes ? bytes : 0;
    }

    int lanesToUse() const
    {
        if (lanes > 0)
            return lanes;
        // Default: enough lanes that a colour fills the GPU, few enough that the incidence loop
        // keeps each lane busy.
        int const perColor = nColors > 0 ? nFree / nColors : nFree;
        if (perColor < 4096)
            return 32;
        return 4;
    }

    void build(pbgb_vbd_desc const* descs, int32_t nMeshes)
    {
        validate_descs(descs, nMeshes);
        int64_t totV = 0, totT = 0, totFree = 0;
        int32_t maxC = 0;
        for (int32_t b = 0; b < nMeshes; ++b)
        {
            auto const& d = descs[b];
            totV += d.n_vertices;
            totT += d.n_tets;
            totFree += d.Pptr[d.n_partitions];
            maxC = std::max(maxC, d.n_partitions);
        }
        if (totV > INT32_MAX || totT >= (int64_t(1) << 30) || totT * 4 > INT32_MAX)
            throw std::invalid_argument("pbgb_vbd_desc: system too large for 32-bit indexing");
        nV      = int32_t(totV);
        nT      = int32_t(totT);
        nFree   = int32_t(totFree);
        nColors = maxC;
        // Settings come from the first mesh (one step size and solver for the whole batch).
        auto const& d0 = descs[0];
        strategy       = d0.init_strategy;
        kD             = float(d0.kD);
        detHZero       = float(d0.detHZero);
        acceleration   = d0.acceleration;
        rho            = d0.rho;
        chebFormula    = d0.chebyshev_formula;
        semantics      = d0.semantics;
        window         = windowed() ? d0.window_size : 0;
        nesterovL      = d0.nesterov_lipschitz;
        nesterovStart  = d0.nesterov_start;
        trEta          = d0.tr_eta;
        trTau          = d0.tr_tau;
        trCurved       = d0.tr_curved != 0;

        // Host staging of the concatenated layout.
        std::vector<float4> hx(nV), hv(nV), ha(nV), hX(nV);
        std::vector<float> hm(nV);
        std::vector<TetRecord> hrec(nT);
        hostWg.assign(size_t(nT), 0.0);
        hostM.assign(size_t(nV), 0.0);
        hostMu.assign(size_t(nT), 0.0);
        hostLambda.assign(size_t(nT), 0.0);
        hostGP.assign(size_t(nT) * 12, 0.0);
        std::vector<int32_t> deg(nV, 0);
        // Colour of every vertex (free vertices from the partitions; pinned ones are never solved
        // and hold the same value in every position buffer, so any colour works: -1).
        std::vector<int32_t> color(nV, -1);
        {
            int32_t vb = 0;
            for (int32_t b = 0; b < nMeshes; ++b)
            {
                auto const& d = descs[b];
                for (int32_t c = 0; c < d.n_partitions; ++c)
                    for (int32_t k = d.Pptr[c]; k < d.Pptr[c + 1]; ++k)
                        color[d.Padj[k] + vb] = c;
                vb += d.n_vertices;
            }
        }
        // Mesh origins, per axis: zero unless the mesh's box (over its rest and initial positions)
        // lies farther from the world origin than its own extent; then the box centre rounded to a
        // multiple of the FP32 spacing at the box's largest coordinate.  Such an origin makes
        // x - origin exact for every FP32 coordinate in the box (a multiple of that coordinate's
        // spacing, no larger than the coordinate), so positions set and read back round-trip bit
        // for bit, and meshes near the world origin keep the world frame.
        meshOrigin.assign(size_t(nMeshes), make_float4(0.f, 0.f, 0.f, 0.f));
        bool const useOrigins = !(nMeshes == 1 && d0.n_collision_triangles > 0);
        if (useOrigins)
            for (int32_t b = 0; b < nMeshes; ++b)
            {
                auto const& d = descs[b];
                double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
                for (double const* R : {d.x, d.X})
                    if (R)
                        for (int32_t i = 0; i < d.n_vertices; ++i)
                            for (int k = 0; k < 3; ++k)
                            {
                                double const c = double(float(R[3 * size_t(i) + k]));
                                lo[k] = std::min(lo[k], c);
                                hi[k] = std::max(hi[k], c);
                            }
                float o[3] = {0.f, 0.f, 0.f};
                for (int k = 0; k < 3 && d.n_vertices > 0; ++k)
                {
                    double const ext = hi[k] - lo[k];
                    bool const far   = (lo[k] > 0.0 && lo[k] > ext) || (hi[k] < 0.0 && -hi[k] > ext);
                    if (!far)
                        continue;
                    int exponent = 0;
                    std::frexp(std::max(std::fabs(lo[k]), std::fabs(hi[k])), &exponent);
                    double const spacing = std::ldexp(1.0, exponent - 24); // FP32 spacing at that magnitude
                    o[k] = float(std::round(0.5 * (lo[k] + hi[k]) / spacing) * spacing);
                }
                meshOrigin[b] = make_float4(o[0], o[1], o[2], 0.f);
            }
        int32_t v0 = 0, t0 = 0;
        for (int32_t b = 0; b < nMeshes; ++b)
        {
            auto const& d = descs[b];
            float const o[3] = {meshOrigin[b].x, meshOrigin[b].y, meshOrigin[b].z};
            for (int32_t i = 0; i < d.n_vertices; ++i)
            {
                double const* p = d.x + 3 * size_t(i);
                hx[v0 + i]      = make_float4(float(p[0]) - o[0], float(p[1]) - o[1], float(p[2]) - o[2], 0.f);
                if (d.v)
                {
                    double const* q = d.v + 3 * size_t(i);
                    hv[v0 + i]      = make_float4(float(q[0]), float(q[1]), float(q[2]), 0.f);
                }
                else
                    hv[v0 + i] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (d.aext)
                {
                    double const* q = d.aext + 3 * size_t(i);
                    ha[v0 + i]      = make_float4(float(q[0]), float(q[1]), float(q[2]), 0.f);
                }
                else
                    ha[v0 + i] = make_float4(0.f, 0.f, -9.81f, 0.f);
                hm[v0 + i]    = float(d.m[i]);
                hostM[v0 + i] = d.m[i];
                double const* R = (d.X ? d.X : d.x) + 3 * size_t(i);
                hX[v0 + i]      = make_float4(float(R[0]) - o[0], float(R[1]) - o[1], float(R[2]) - o[2], 0.f);
            }
            for (int32_t e = 0; e < d.n_tets; ++e)
            {
                int32_t const* t = d.T + 4 * size_t(e);
                uint32_t gv[4];
                for (int q = 0; q < 4; ++q)
                {
                    gv[q] = uint32_t(t[q] + v0);
                    deg[gv[q]]++;
                }
                // Rank of each vertex by colour inside the tet (ties broken by position).
                uint32_t packed[4];
                for (int q = 0; q < 4; ++q)
                {
                    uint32_t rank = 0;
                    for (int o = 0; o < 4; ++o)
                        if (color[gv[o]] < color[gv[q]] || (color[gv[o]] == color[gv[q]] && o < q))
                            ++rank;
                    packed[q] = gv[q] | (rank << 30);
                }
                double const w = d.wg[e], mu = d.mu[e], la = d.lambda[e];
                hostWg[t0 + e]     = w;
                hostMu[t0 + e]     = mu;
                hostLambda[t0 + e] = la;
                if (d.GP)
                    std::copy(d.GP + 12 * size_t(e), d.GP + 12 * size_t(e + 1), hostGP.begin() + 12 * size_t(t0 + e));
                else
                {
                    // Gradients of the linear shape functions from the rest positions (FP64).
                    double const* R  = d.X ? d.X : d.x;
                    int32_t const* q = d.T + 4 * size_t(e);
                    double ed[3][3], Gd[3][3];
                    for (int mm = 0; mm < 3; ++mm)
                        for (int r = 0; r < 3; ++r)
                            ed[mm][r] = R[3 * size_t(q[mm + 1]) + r] - R[3 * size_t(q[0]) + r];
                    rest_gradients(ed, Gd);
                    double* out = hostGP.data() + 12 * size_t(t0 + e);
                    for (int c = 0; c < 3; ++c)
                    {
                        out[c] = -(Gd[0][c] + Gd[1][c] + Gd[2][c]);
                        for (int mm = 0; mm < 3; ++mm)
                            out[3 * (mm + 1) + c] = Gd[mm][c];
                    }
                }
                TetRecord& r   = hrec[t0 + e];
                r.v            = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                r.mat          = make_float4(float(w * mu), float(w * la), float(1.0 + mu / la), 0.f);
            }
            v0 += d.n_vertices;
            t0 += d.n_tets;
        }
        // Incidences per vertex, tets ascending (counting sort over the global tet index).
        std::vector<int32_t> vPtr(size_t(nV) + 1, 0);
        for (int32_t i = 0; i < nV; ++i)
            vPtr[i + 1] = vPtr[i] + deg[i];
        std::vector<uint32_t> vInc(static_cast<size_t>(vPtr[nV]));
        {
            std::vector<int32_t> cur(vPtr.begin(), vPtr.end() - 1);
            for (int32_t e = 0; e < nT; ++e)
            {
                uint4 const t       = hrec[e].v;
                uint32_t const a[4] = {t.x & kIndexMask, t.y & kIndexMask, t.z & kIndexMask, t.w & kIndexMask};
                for (int q = 0; q < 4; ++q)
                    vInc[cur[a[q]]++] = (uint32_t(e) << 2) | uint32_t(q);
            }
        }
        // Colour-major solve list: colour c = union of every mesh's partition c; inside a colour,
        // stable order by decreasing degree so that lanes of a warp see similar trip counts.
        // Inside a colour the meshes follow one another, each mesh's entries in stable order of
        // decreasing degree, so that a (mesh, colour) pair is one range of the list.
        std::vector<int32_t> hsolve;
        hsolve.reserve(nFree);
        colorPtr.assign(size_t(nColors) + 1, 0);
        this->nMeshes = nMeshes;
        meshV0.assign(size_t(nMeshes) + 1, 0);
        for (int32_t b = 0; b < nMeshes; ++b)
            meshV0[b + 1] = meshV0[b] + descs[b].n_vertices;
        meshSolve.assign(size_t(nMeshes), std::vector<int32_t>(2 * size_t(nColors), 0));
        for (int32_t c = 0; c < nColors; ++c)
        {
            for (int32_t b = 0; b < nMeshes; ++b)
            {
                auto const& d      = descs[b];
                size_t const start = hsolve.size();
                meshSolve[b][2 * c] = int32_t(start);
                if (c < d.n_partitions)
                    for (int32_t k = d.Pptr[c]; k < d.Pptr[c + 1]; ++k)
                        hsolve.push_back(d.Padj[k] + meshV0[b]);
                std::stable_sort(hsolve.begin() + start, hsolve.end(), [&](int32_t a, int32_t q) {
                    return deg[a] > deg[q];
                });
                meshSolve[b][2 * c + 1] = int32_t(hsolve.size());
            }
            colorPtr[c + 1] = int32_t(hsolve.size());
        }
        std::vector<int32_t> hIncPtr(size_t(nFree) + 1, 0);
        std::vector<uint32_t> hInc;
        hInc.reserve(vInc.size());
        int64_t degSum = 0;
        for (int32_t s = 0; s < nFree; ++s)
        {
            int32_t const i = hsolve[s];
            hInc.insert(hInc.end(), vInc.begin() + vPtr[i], vInc.begin() + vPtr[i + 1]);
            hIncPtr[s + 1] = int32_t(hInc.size());
            degSum += deg[i];
        }
        meanDegree = nFree > 0 ? double(degSum) / nFree : 0.0;

        // Neighbour lists of the staged sweep, in first-use order over the vertex's incidences and
        // corners ((local + 1 + m) & 3, the order the sweep visits them).
        std::vector<uint32_t> hNbr;
        hostSlots.assign(hInc.size(), 0u);
        hostNbrPtr.assign(size_t(nFree) + 1, 0);
        stagedOk = true;
        {
            std::vector<uint32_t> list;
            for (int32_t s = 0; s < nFree; ++s)
            {
                list.clear();
                for (int32_t k = hIncPtr[s]; k < hIncPtr[s + 1]; ++k)
                {
                    uint32_t const q  = hInc[k];
                    uint4 const t     = hrec[q >> 2].v;
                    int const il      = int(q & 3u);
                    uint32_t const c4[4] = {t.x, t.y, t.z, t.w};
                    uint32_t const own = c4[il] >> 30;
                    uint32_t slots     = 0;
                    for (int m = 0; m < 3; ++m)
                    {
                        uint32_t const ca = c4[(il + 1 + m) & 3];
                        uint32_t const a  = (ca & kIndexMask) | ((ca >> 30) < own ? 0x80000000u : 0u);
                        size_t idx        = 0;
                        while (idx < list.size() && list[idx] != a)
                            ++idx;
                        if (idx == list.size())
                            list.push_back(a);
                        slots |= uint32_t(idx) << (8 * m);
                    }
                    hostSlots[k] = slots; // meaningful only while the list has at most 256 entries
                }
                if (list.size() > 256)
                    stagedOk = false;
                if (stagedOk)
                {
                    hNbr.insert(hNbr.end(), list.begin(), list.end());
                    hostNbrPtr[s + 1] = int32_t(hNbr.size());
                }
            }
        }
        hostInc = hInc;
        std::vector<float4> hStiff;
        std::vector<uint2> hPack;
        incidenceRecords(hStiff, hPack);

        // Device allocation and upload.
        check(cudaGetDevice(&device), "cudaGetDevice");
        check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        x.allocate(nV);
        xt.allocate(nV);
        xtilde.allocate(nV);
        v.allocate(nV);
        aext.allocate(nV);
        vprev.allocate(nV);
        m.allocate(nV);
        staging.allocate(size_t(nV) * 3);
        tets.allocate(nT);
        X.allocate(nV);
        solve.allocate(nFree);
        incPtr.allocate(size_t(nFree) + 1);
        inc.allocate(hInc.size());
        flags.allocate(4);
        red.allocate(1);
        objPartials.allocate(size_t(kObjectiveMaxBlocks));
        if (acceleration == PBGB_ACCEL_CHEBYSHEV)
        {
            h0.allocate(nV);
            h1.allocate(nV);
        }
        if (acceleration == PBGB_ACCEL_NESTEROV)
        {
            neX0.allocate(nV);
            neY.allocate(nV);
        }
        if (trustLinear())
        {
            trXkm1.allocate(nV);
            trState.allocate(1);
            trPartials.allocate(size_t(kTrustMaxBlocks));
            check(cudaMemsetAsync(trState.get(), 0, sizeof(TrustState), stream), "memset");
        }
        if (windowed())
        {
            anStep.allocate(nV);
            anGkm1.allocate(nV);
            anFkm1.allocate(nV);
            anDF.allocate(size_t(window) * size_t(nV));
            anDG.allocate(size_t(window) * size_t(nV));
            anPartials.allocate(size_t(anderson_window_blocks(nV)) * 2 * size_t(window));
            anGram.allocate(size_t(window) * size_t(window));
            anAlpha.allocate(size_t(window));
            anRhs.allocate(size_t(window));
            // Pinned vertices are never solved: their increment stays zero.
            check(cudaMemsetAsync(anStep.get(), 0, sizeof(float4) * size_t(nV), stream), "memset");
            check(cudaMemsetAsync(anGram.get(), 0, sizeof(double) * size_t(window) * size_t(window), stream), "memset");
        }
        x.upload(hx.data(), nV, stream);
        v.upload(hv.data(), nV, stream);
        aext.upload(ha.data(), nV, stream);
        m.upload(hm.data(), nV, stream);
        tets.upload(hrec.data(), nT, stream);
        X.upload(hX.data(), nV, stream);
        std::vector<float4> hOrigin;
        if (useOrigins)
        {
            hOrigin.resize(size_t(nV));
            for (int32_t b = 0; b < nMeshes; ++b)
                std::fill(hOrigin.begin() + meshV0[b], hOrigin.begin() + meshV0[b + 1], meshOrigin[b]);
            origin.allocate(size_t(nV));
            origin.upload(hOrigin.data(), size_t(nV), stream);
        }
        solve.upload(hsolve.data(), nFree, stream);
        incStiff.allocate(hStiff.size());
        incStiff.upload(hStiff.data(), hStiff.size(), stream);
        incPack.allocate(hPack.size());
        incPack.upload(hPack.data(), hPack.size(), stream);
        incPtr.upload(hIncPtr.data(), hIncPtr.size(), stream);
        inc.upload(hInc.data(), hInc.size(), stream);
        if (stagedOk)
        {
            nbrPtr.allocate(hostNbrPtr.size());
            nbr.allocate(hNbr.size());
            nbrPtr.upload(hostNbrPtr.data(), hostNbrPtr.size(), stream);
            nbr.upload(hNbr.data(), hNbr.size(), stream);
            check(prepare_staged_sweeps(), "cudaFuncSetAttribute");
            if (nMeshes > 1)
                check(prepare_batched_step(), "cudaFuncSetAttribute");
        }
        else
            hostNbrPtr.clear();
        if (nV > 0)
        {
            check(cudaMemcpyAsync(xt.get(), x.get(), sizeof(float4) * nV, cudaMemcpyDeviceToDevice, stream), "copy");
            check(cudaMemsetAsync(vprev.get(), 0, sizeof(float4) * nV, stream), "memset");
            check(cudaMemsetAsync(xtilde.get(), 0, sizeof(float4) * nV, stream), "memset");
        }
        check(cudaMemsetAsync(flags.get(), 0, sizeof(int32_t) * 4, stream), "memset");
        vcolorD.allocate(nV);
        vcolorD.upload(color.data(), nV, stream);
        std::vector<int32_t> hV, hB;
        std::vector<int4> hF;
        std::vector<float> hXVA, hFA;
        std::vector<float> hDupper;
        if (d0.n_collision_triangles > 0)
        {
            if (nMeshes != 1)
                throw std::invalid_argument("contact is supported on a single (non-batched) mesh");
            if (!d0.V || !d0.F || !d0.XVA || !d0.FA || d0.n_collision_vertices <= 0)
                throw std::invalid_argument("pbgb_vbd_desc: contact needs V, F, XVA and FA");
            if (d0.active_set_update_frequency < 1)
                throw std::invalid_argument("pbgb_vbd_desc: active set update frequency must be >= 1");
            contact       = true;
            muC           = float(d0.muC);
            muF           = float(d0.muF);
            epsv          = float(d0.epsv);
            activeSetFreq = d0.active_set_update_frequency;
            int32_t const nS = d0.n_collision_vertices, nF = d0.n_collision_triangles;
            hV.assign(d0.V, d0.V + nS);
            for (int32_t q : hV)
                if (q < 0 || q >= nV)
                    throw std::invalid_argument("pbgb_vbd_desc: collision vertex out of range");
            hF.resize(size_t(nF));
            for (int32_t f = 0; f < nF; ++f)
            {
                int32_t const* t = d0.F + 3 * size_t(f);
                for (int k = 0; k < 3; ++k)
                    if (t[k] < 0 || t[k] >= nV)
                        throw std::invalid_argument("pbgb_vbd_desc: collision triangle index out of range");
                hF[f] = make_int4(t[0], t[1], t[2], 0);
            }
            hB.resize(size_t(nV));
            for (int32_t i = 0; i < nV; ++i)
                hB[i] = d0.B ? d0.B[i] : 1;
            hXVA.resize(size_t(nV));
            for (int32_t i = 0; i < nV; ++i)
                hXVA[i] = float(d0.XVA[i]);
            hFA.resize(size_t(nF));
            for (int32_t f = 0; f < nF; ++f)
                hFA[f] = float(d0.FA[f]);
            hDupper.assign(size_t(nS), FLT_MAX);
            cV.allocate(nS);
            cF.allocate(nF);
            cB.allocate(nV);
            cXVA.allocate(nV);
            cFA.allocate(nF);
            cDupper.allocate(nS);
            cTlo.allocate(nF);
            cThi.allocate(nF);
            cVlo.allocate(nS);
            cVhi.allocate(nS);
            xpred.allocate(nV);
            cActive.allocate(nS);
            cAv.allocate(nS);
            cNActive.allocate(1);
            cNn.allocate(size_t(nS) * kMaxContacts);
            cFc.allocate(size_t(nV) * kMaxContacts);
            cRec.allocate(size_t(nV) * kMaxContacts);
            cPen.allocate(size_t(nV) * kMaxContacts);
            cCount.allocate(size_t(nV));
            check(cudaMemset(cCount.get(), 0, sizeof(int32_t) * size_t(nV)), "cudaMemset");
            check(bvh_allocate(cstate.bvh, nF), "cudaMalloc");
            cV.upload(hV.data(), nS, stream);
            cF.upload(hF.data(), nF, stream);
            cB.upload(hB.data(), nV, stream);
            cXVA.upload(hXVA.data(), nV, stream);
            cFA.upload(hFA.data(), nF, stream);
            cDupper.upload(hDupper.data(), nS, stream);
            check(cudaMemsetAsync(cActive.get(), 0, size_t(nS), stream), "memset");
            check(cudaMemsetAsync(cNActive.get(), 0, sizeof(int32_t), stream), "memset");
            check(cudaMemsetAsync(cNn.get(), 0xFF, sizeof(int32_t) * size_t(nS) * kMaxContacts, stream), "memset");
            check(cudaMemsetAsync(cFc.get(), 0xFF, sizeof(int32_t) * size_t(nV) * kMaxContacts, stream), "memset");
            cmesh  = ContactMesh{nV, nS, nF, cV.get(), cF.get(), cB.get()};
            cstate.tlo     = cTlo.get();
            cstate.thi     = cThi.get();
            cstate.vlo     = cVlo.get();
            cstate.vhi     = cVhi.get();
            cstate.active  = cActive.get();
            cstate.dupper  = cDupper.get();
            cstate.av      = cAv.get();
            cstate.nActive = cNActive.get();
            cstate.nn      = cNn.get();
            cstate.fc      = cFc.get();
            cstate.flags   = cstate.bvh.flags;
            // Default scene box: the rest positions' box (pbgb_vbd_set_scene_bounding_box overrides).
            for (int k = 0; k < 3; ++k)
            {
                sceneMin[k] = FLT_MAX;
                sceneMax[k] = -FLT_MAX;
            }
            for (int32_t i = 0; i < nV; ++i)
            {
                float const p[3] = {hX[i].x, hX[i].y, hX[i].z};
                for (int k = 0; k < 3; ++k)
                {
                    sceneMin[k] = std::min(sceneMin[k], p[k]);
                    sceneMax[k] = std::max(sceneMax[k], p[k]);
                }
            }
            if (!h0.get())
            {
                h0.allocate(nV);
                h1.allocate(nV);
            }
        }
        // The host staging vectors die at the end of this scope: wait for the uploads.
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        hostRecords = std::move(hrec);
    }

    // Per-incidence stiffness of all solved incidences (solve order) from the host copies of the
    // shape-function gradients, quadrature weights and Lame coefficients: stiff[k] = (b0, b1, b2,
    // kappa_o) of incidence k's own corner o, pack[k] = (neighbour slots, sigma as bits).
    void incidenceRecords(std::vector<float4>& stiffOut, std::vector<uint2>& packOut) const
    {
        std::vector<double> words(8 * size_t(nT));
        for (int32_t e = 0; e < nT; ++e)
        {
            double w[8];
            tet_stiffness_words(hostGP.data() + 12 * size_t(e), hostWg[e], hostMu[e], hostLambda[e], w);
            std::copy(w, w + 8, words.begin() + 8 * size_t(e));
        }
        stiffOut.resize(hostInc.size());
        packOut.resize(hostInc.size());
        for (size_t k = 0; k < hostInc.size(); ++k)
        {
            uint32_t const q   = hostInc[k];
            double const* w    = words.data() + 8 * size_t(q >> 2);
            double const bw[6] = {w[0], w[1], w[2], w[3], w[4], w[5]};
            double b0, b1, b2, kappa;
            corner_stiffness(bw, w[7], int(q & 3u), b0, b1, b2, kappa);
            stiffOut[k]        = make_float4(float(b0), float(b1), float(b2), float(kappa));
            float const sigma  = float(w[6]);
            uint32_t sbits     = 0;
            std::memcpy(&sbits, &sigma, sizeof(sbits));
            packOut[k] = make_uint2(hostSlots[k], sbits);
        }
    }

    // Per-tet Lame coefficients (system order); the records keep (wg mu, wg lambda, 1 + mu/lambda).
    void setMaterial(double const* mu, double const* lambda)
    {
        restEnergyValid = false;
        for (int32_t e = 0; e < nT; ++e)
            if (!(mu[e] > 0.0) || !(lambda[e] > 0.0) || !std::isfinite(mu[e]) || !std::isfinite(lambda[e]))
                throw std::invalid_argument("pbgb_vbd_set_material: expected finite mu > 0 and lambda > 0");
        for (int32_t e = 0; e < nT; ++e)
        {
            double const w     = hostWg[e];
            hostRecords[e].mat = make_float4(float(w * mu[e]), float(w * lambda[e]), float(1.0 + mu[e] / lambda[e]), 0.f);
            hostMu[e]          = mu[e];
            hostLambda[e]      = lambda[e];
        }
        tets.upload(hostRecords.data(), size_t(nT), stream);
        std::vector<float4> hStiff;
        std::vector<uint2> hPack;
        incidenceRecords(hStiff, hPack);
        incStiff.upload(hStiff.data(), hStiff.size(), stream);
        incPack.upload(hPack.data(), hPack.size(), stream);
        // The uploads read the host arrays asynchronously.
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    void adjointReserve(int32_t slots, int32_t iterations)
    {
        if (slots < 0 || iterations < 0)
            throw std::invalid_argument("pbgb_vbd_adjoint_reserve: expected slots >= 0, iterations >= 0");
        checkDifferentiable();
        if (slots == tapeSlots && iterations == tapeIters && ubar.size() == size_t(nV))
            return;
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        dropSlotGraphs();
        adjX.allocate(size_t(nV) * 3);
        adjV.allocate(size_t(nV) * 3);
        adjP.allocate(size_t(nV) * 3);
        adjZero.allocate(size_t(nV) * 3);
        adjMu.allocate(size_t(nT));
        adjLa.allocate(size_t(nT));
        tapeX.allocate(size_t(slots) * size_t(iterations + 1) * size_t(nV));
        tapeH.allocate(size_t(slots) * size_t(iterations) * size_t(nFree) * 2);
        tapeS.allocate(size_t(slots) * 3 * size_t(nV));
        if (acceleration == PBGB_ACCEL_CHEBYSHEV)
        {
            tapeRaw.allocate(size_t(slots) * size_t(iterations) * size_t(nV));
            ycarry.allocate(size_t(nV));
            ycarry2.allocate(size_t(nV));
        }
        ubar.allocate(size_t(nV));
        xtbar.allocate(size_t(nV));
        xsbar.allocate(size_t(nV));
        if (nV > 0)
            check(cudaMemsetAsync(adjZero.get(), 0, sizeof(float) * 3 * size_t(nV), stream), "memset");
        tapeSlots = slots;
        tapeIters = iterations;
        slotH.assign(size_t(slots), 0.f);
        slotKD.assign(size_t(slots), 0.f);
        slotStrategy.assign(size_t(slots), -1);
    }

    void checkDifferentiable() const
    {
        if (contact)
            throw std::invalid_argument("the adjoint does not support contact");
        if (acceleration != PBGB_ACCEL_NONE && acceleration != PBGB_ACCEL_CHEBYSHEV)
            throw std::invalid_argument("the adjoint supports plain VBD and Chebyshev acceleration only");
    }

    float4* slotX(int32_t slot, int32_t k) const
    {
        return tapeX.get() + (size_t(slot) * size_t(tapeIters + 1) + size_t(k)) * size_t(nV);
    }
    float4* slotTape(int32_t slot, int32_t k) const
    {
        return tapeH.get() + (size_t(slot) * size_t(tapeIters) + size_t(k)) * size_t(nFree) * 2;
    }
    // q = 0: start positions, 1: start velocities, 2: start previous velocities.
    float4* slotStart(int32_t slot, int32_t q) const
    {
        return tapeS.get() + (size_t(slot) * 3 + size_t(q)) * size_t(nV);
    }
    // Raw sweep result of iteration k (Chebyshev); without acceleration it is the iterate itself.
    float4* slotRaw(int32_t slot, int32_t k) const
    {
        if (acceleration != PBGB_ACCEL_CHEBYSHEV)
            return slotX(slot, k + 1);
        return tapeRaw.get() + (size_t(slot) * size_t(tapeIters) + size_t(k)) * size_t(nV);
    }

    // One step like step(), with every substep recorded into slots slot0, slot0 + 1, ...  Launched
    // directly (not from the graph) with the same kernels' recording variant, so the positions
    // match an unrecorded step.
    void recordStep(float dt, int32_t iterations, int32_t substeps, int32_t slot0)
    {
        checkDifferentiable();
        if (iterations != tapeIters || slot0 < 0 || int64_t(slot0) + substeps > tapeSlots)
            throw std::invalid_argument("pbgb_vbd_step_record: slots or iteration count differ from pbgb_vbd_adjoint_reserve");
        if (recGraphs.size() < size_t(tapeSlots))
            recGraphs.resize(size_t(tapeSlots));
        SlotGraph& g = recGraphs[slot0];
        if (!g.exec || g.dt != dt || g.iters != iterations || g.sub != substeps || g.kd != std::vector<float>{kD} ||
            g.strategy != std::vector<int32_t>{strategy})
        {
            if (g.exec)
                cudaGraphExecDestroy(g.exec);
            g.exec     = nullptr;
            g.exec     = capture([&] { enqueueRecord(dt, iterations, substeps, slot0); });
            g.dt       = dt;
            g.iters    = iterations;
            g.sub      = substeps;
            g.kd       = {kD};
            g.strategy = {strategy};
        }
        check(cudaGraphLaunch(g.exec, stream), "cudaGraphLaunch");
        float const h = dt / float(substeps);
        for (int32_t s = 0; s < substeps; ++s)
        {
            slotH[slot0 + s]        = h;
            slotKD[slot0 + s]       = kD;
            slotStrategy[slot0 + s] = strategy;
        }
    }

    void enqueueRecord(float dt, int32_t iterations, int32_t substeps, int32_t slot0)
    {
        float const h    = dt / float(substeps);
        bool const cheb  = acceleration == PBGB_ACCEL_CHEBYSHEV;
        SubstepParams sp = substepParams(h);
        if (!cheb)
            sp.h0 = sp.h1 = nullptr;
        else if (iterations > 0)
            sp.result = ((iterations - 1) % 2 == 0) ? h0.get() : h1.get();
        SweepParams w{};
        w.x        = x.get();
        w.xt       = xt.get();
        w.xtilde   = xtilde.get();
        w.tets     = tets.get();
        w.stiff    = incStiff.get();
        w.incPack  = incPack.get();
        w.solve    = solve.get();
        w.incPtr   = incPtr.get();
        w.inc      = inc.get();
        stagedFields(w);
        w.h        = h;
        w.h2       = h * h;
        w.kD       = kD;
        w.detHZero = detHZero;
        w.omega    = 1.f;
        int const L = lanesToUse();
        size_t const bytes = sizeof(float4) * size_t(nV);
        float4* H[2] = {h0.get(), h1.get()};
        auto copy = [&](float4* dst, float4 const* src) {
            if (nV > 0)
                check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, stream), "tape copy");
        };
        for (int32_t s = 0; s < substeps; ++s)
        {
            int32_t const slot = slot0 + s;
            copy(slotStart(slot, 0), x.get());
            copy(slotStart(slot, 1), v.get());
            copy(slotStart(slot, 2), vprev.get());
            check(launch_begin_substep(sp, stream), "begin_substep");
            copy(slotX(slot, 0), x.get());
            double omega      = 0.0;
            double const rho2 = rho * rho;
            for (int32_t k = 0; k < iterations; ++k)
            {
                w.tape = slotTape(slot, k);
                if (cheb)
                {
                    omega   = chebyshev_omega<double>(k, rho2, omega, chebFormula);
                    w.omega = float(omega);
                    w.k     = k;
                    w.hprev = H[(k + 1) % 2];
                    w.hcur  = H[k % 2];
                }
                for (int32_t c = 0; c < nColors; ++c)
                {
                    w.begin = colorPtr[c];
                    w.end   = colorPtr[c + 1];
                    w.color = c;
                    // The first colour follows a copy into the tape (not a kernel): no programmatic
                    // launch there, so that it cannot overwrite what the copy reads.
                    check(launch_sweep_record(w, L, block, cheb, pdl && c > 0, stream, stagedBytes(c, L)), "sweep_record");
                }
                if (cheb)
                {
                    copy(slotRaw(slot, k), x.get());
                    copy(slotX(slot, k + 1), H[k % 2]);
                }
                else
                    copy(slotX(slot, k + 1), x.get());
            }
            check(launch_end_substep(sp, stream), "end_substep");
        }
    }

    // Reverses the substeps recorded in slots slot0 + substeps - 1, ..., slot0.  xbar, vbar, pbar
    // (device, nV x 3): adjoints of the positions, velocities and previous velocities after the
    // last substep on entry, before the first on return.  dlogmu, dloglambda (device, nT, FP64):
    // accumulated.
    void adjointStep(int32_t slot0, int32_t substeps, float* xbar, float* vbar, float* pbar, double* dlogmu, double* dloglambda)
    {
        checkDifferentiable();
        if (slot0 < 0 || substeps < 1 || int64_t(slot0) + substeps > tapeSlots)
            throw std::invalid_argument("pbgb_vbd_step_adjoint: slot range outside the reserved tape");
        std::vector<float> hs(slotH.begin() + slot0, slotH.begin() + slot0 + substeps);
        std::vector<float> kds(slotKD.begin() + slot0, slotKD.begin() + slot0 + substeps);
        std::vector<int32_t> st(slotStrategy.begin() + slot0, slotStrategy.begin() + slot0 + substeps);
        for (int32_t v : st)
            if (v < 0)
                throw std::invalid_argument("pbgb_vbd_step_adjoint: slot was not recorded");
        if (adjGraphs.size() < size_t(tapeSlots))
            adjGraphs.resize(size_t(tapeSlots));
        SlotGraph& g = adjGraphs[slot0];
        if (!g.exec || g.sub != substeps || g.h != hs || g.strategy != st || g.kd != kds)
        {
            if (g.exec)
                cudaGraphExecDestroy(g.exec);
            g.exec     = nullptr;
            g.exec     = capture([&] { enqueueAdjoint(slot0, substeps, adjX.get(), adjV.get(), adjP.get(), adjMu.get(), adjLa.get()); });
            g.sub      = substeps;
            g.h        = hs;
            g.strategy = st;
            g.kd       = kds;
        }
        size_t const b3 = sizeof(float) * 3 * size_t(nV), bt = sizeof(double) * size_t(nT);
        auto copy = [&](void* dst, void const* src, size_t n) {
            if (n > 0)
                check(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, stream), "adjoint copy");
        };
        copy(adjX.get(), xbar, b3);
        copy(adjV.get(), vbar, b3);
        copy(adjP.get(), pbar, b3);
        copy(adjMu.get(), dlogmu, bt);
        copy(adjLa.get(), dloglambda, bt);
        check(cudaGraphLaunch(g.exec, stream), "cudaGraphLaunch");
        copy(xbar, adjX.get(), b3);
        copy(vbar, adjV.get(), b3);
        copy(pbar, adjP.get(), b3);
        copy(dlogmu, adjMu.get(), bt);
        copy(dloglambda, adjLa.get(), bt);
    }

    void enqueueAdjoint(int32_t slot0, int32_t substeps, float* xbar, float* vbar, float* pbar, double* dlogmu, double* dloglambda)
    {
        int const L     = lanesToUse();
        bool const cheb = acceleration == PBGB_ACCEL_CHEBYSHEV;
        // Chebyshev weights of the iterations, as the forward formed them.
        std::vector<float> om(size_t(std::max(tapeIters, 1)), 1.f);
        {
            double omega = 0.0;
            for (int32_t k = 0; k < tapeIters; ++k)
            {
                omega         = chebyshev_omega<double>(k, rho * rho, omega, chebFormula);
                om[size_t(k)] = float(omega);
            }
        }
        for (int32_t s = substeps - 1; s >= 0; --s)
        {
            int32_t const slot = slot0 + s;
            float const h      = slotH[slot];
            check(launch_adjoint_begin(nV, xbar, vbar, ubar.get(), xtbar.get(), xsbar.get(), cheb ? ycarry.get() : nullptr,
                                       cheb ? ycarry2.get() : nullptr, h, stream),
                  "adjoint_begin");
            AdjointSweepParams a{};
            a.X          = X.get();
            a.tets       = tets.get();
            a.solve      = solve.get();
            a.incPtr     = incPtr.get();
            a.inc        = inc.get();
            a.m          = m.get();
            a.ubar       = ubar.get();
            a.xtbar      = xtbar.get();
            a.dlogmu     = dlogmu;
            a.dloglambda = dloglambda;
            a.h2         = h * h;
            a.D          = slotKD[slot] / h;
            a.xs         = slotStart(slot, 0);
            a.xsbar      = xsbar.get();
            for (int32_t k = tapeIters - 1; k >= 0; --k)
            {
                if (cheb)
                    check(launch_adjoint_cheb_mix(nV, ubar.get(), ycarry.get(), ycarry2.get(), k > 1 ? om[size_t(k)] : 1.f,
                                                  k > 1 ? 1.f - om[size_t(k)] : 0.f, stream),
                          "adjoint_cheb_mix");
                a.xk   = slotRaw(slot, k);
                a.xkm1 = slotX(slot, k);
                a.tape = slotTape(slot, k);
                for (int32_t c = nColors - 1; c >= 0; --c)
                {
                    a.begin = colorPtr[c];
                    a.end   = colorPtr[c + 1];
                    // A mix kernel precedes the last colour of an iteration: no programmatic launch
                    // across it.
                    check(launch_adjoint_sweep(a, L, std::min(block, 256), pdl && !(cheb && c == nColors - 1), stream),
                          "adjoint_sweep");
                }
            }
            check(launch_adjoint_end(nV, xbar, vbar, pbar, ubar.get(), xtbar.get(), xsbar.get(), slotStart(slot, 1),
                                     slotStart(slot, 2), aext.get(), h, slotStrategy[slot],
                                     semantics == PBGB_SEMANTICS_GPU ? 1 : 0, stream),
                  "adjoint_end");
        }
    }

    SubstepParams substepParams(float h) const
    {
        SubstepParams p{};
        p.x            = x.get();
        p.xt           = xt.get();
        p.xtilde       = xtilde.get();
        p.v            = v.get();
        p.aext         = aext.get();
        p.vprev        = vprev.get();
        p.h0           = h0.get();
        p.h1           = h1.get();
        p.result       = x.get();
        p.m            = m.get();
        p.flags        = flags.get();
        p.n            = nV;
        p.h            = h;
        p.h2           = h * h;
        p.strategy     = strategy;
        p.gpuSemantics = semantics == PBGB_SEMANTICS_GPU ? 1 : 0;
        return p;
    }

    // Whether step() runs the persistent batched kernel (batched.cuh): batches without contact,
    // plain or Chebyshev, every colour staged, and no per-launch sweep timing.
    bool persistentActive() const
    {
        return nMeshes > 1 && persistent && !contact &&
               (acceleration == PBGB_ACCEL_NONE || acceleration == PBGB_ACCEL_CHEBYSHEV) && stagedOk && staged &&
               !profiling;
    }

    // Work items of the persistent step for (iterations, substeps) and the current launch shape,
    // in stage order (substep, then begin / iteration and colour / end), meshes in order inside a
    // stage, tiles in order inside a mesh; each item records how many of its mesh's items must be
    // complete first.  Stage order keeps a whole stage of items (every mesh's colour) between two
    // stages of one mesh, well over the items the resident blocks hold at once, so a block rarely
    // takes an item whose mesh is still on the previous colour.  (Alternating the mesh order
    // between stages, to bring half of the meshes' next colour closer for L2, put the last meshes'
    // items of a stage, still in flight, right before their next ones: 15.3 ms per 256-mesh step
    // against 11.1.)  Built and uploaded outside any stream capture.  Returns false when the batch
    // cannot run persistently with this launch (the colour-launch path is used then).
    bool preparePersistent(int32_t iterations, int32_t substeps)
    {
        int const L = lanesToUse();
        int const B = std::min(block, 256);
        if (plan.iters == iterations && plan.sub == substeps && plan.lanes == L && plan.block == B &&
            plan.tile == batchTile)
            return plan.grid > 0;
        plan       = PersistentPlan{};
        plan.iters = iterations;
        plan.sub   = substeps;
        plan.lanes = L;
        plan.block = B;
        plan.tile  = batchTile;
        int const per = B / L;
        if (per < 1 || B % 32 != 0)
            return false;
        int const tileE = per * batchTile, tileV = 4 * B;
        // Shared memory of the largest sweep tile.
        size_t smem = 0;
        for (int32_t b = 0; b < nMeshes; ++b)
            for (int32_t c = 0; c < nColors; ++c)
                for (int32_t f = meshSolve[b][2 * c]; f < meshSolve[b][2 * c + 1]; f += tileE)
                {
                    int32_t const e = std::min(f + tileE, meshSolve[b][2 * c + 1]);
                    for (int32_t g = f; g < e; g += per)
                        smem = std::max(smem, size_t(hostNbrPtr[std::min(g + per, e)] - hostNbrPtr[g]) * kStagedSlotBytes);
                }
        if (smem > kStagedMaxBytes)
            return false;
        bool const cheb = acceleration == PBGB_ACCEL_CHEBYSHEV;
        int const perSM = batched_step_blocks_per_sm(L, B, smem, cheb);
        if (perSM < 1)
            return false;
        int sms = 0;
        check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
        std::vector<BatchItemWords> items;
        std::vector<int32_t> count(size_t(nMeshes), 0);
        auto emit = [&](int32_t b, int kind, int32_t k, int32_t lo, int32_t hi, int32_t step) {
            int32_t const need = count[b];
            for (int32_t f = lo; f < hi; f += step)
            {
                int32_t const e = std::min(f + step, hi);
                items.push_back(BatchItemWords{make_int4(b, kind | (k << 2), f, e), make_int4(need, 0, 0, 0)});
                ++count[b];
            }
        };
        for (int32_t s = 0; s < substeps; ++s)
        {
            for (int32_t b = 0; b < nMeshes; ++b)
                emit(b, kBatchBegin, 0, meshV0[b], meshV0[b + 1], tileV);
            for (int32_t k = 0; k < iterations; ++k)
                for (int32_t c = 0; c < nColors; ++c)
                    for (int32_t b = 0; b < nMeshes; ++b)
                        emit(b, kBatchSweep, k, meshSolve[b][2 * c], meshSolve[b][2 * c + 1], tileE);
            for (int32_t b = 0; b < nMeshes; ++b)
                emit(b, kBatchEnd, 0, meshV0[b], meshV0[b + 1], tileV);
        }
        if (items.size() > size_t(INT32_MAX))
            return false;
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        batchItems.allocate(std::max<size_t>(items.size(), 1));
        if (!items.empty())
            check(cudaMemcpy(batchItems.get(), items.data(), sizeof(BatchItemWords) * items.size(), cudaMemcpyHostToDevice),
                  "H2D");
        batchCounters.allocate(2 + size_t(nMeshes));
        std::vector<float> om(size_t(std::max(iterations, 1)), 1.f);
        double omega = 0.0;
        for (int32_t k = 0; k < iterations; ++k)
        {
            omega          = chebyshev_omega<double>(k, rho * rho, omega, chebFormula);
            om[size_t(k)] = float(omega);
        }
        batchOmega.allocate(om.size());
        check(cudaMemcpy(batchOmega.get(), om.data(), sizeof(float) * om.size(), cudaMemcpyHostToDevice), "H2D");
        plan.nItems = int32_t(items.size());
        plan.smem   = smem;
        plan.grid   = int32_t(std::min<int64_t>(int64_t(perSM) * sms, std::max<int64_t>(plan.nItems, 1)));
        return true;
    }

    // One persistent launch for the whole step (after the counters are cleared).
    void enqueuePersistentStep(float dt, int32_t iterations, int32_t substeps)
    {
        float const h    = dt / float(substeps);
        bool const cheb  = acceleration == PBGB_ACCEL_CHEBYSHEV;
        SubstepParams sp = substepParams(h);
        if (!cheb)
            sp.h0 = sp.h1 = nullptr;
        else if (iterations > 0)
            sp.result = ((iterations - 1) % 2 == 0) ? h0.get() : h1.get();
        BatchedStepParams bp{};
        SweepParams& w = bp.sweep;
        w.x        = x.get();
        w.xt       = xt.get();
        w.xtilde   = xtilde.get();
        w.stiff    = incStiff.get();
        w.incPack  = incPack.get();
        w.tets     = tets.get();
        w.solve    = solve.get();
        w.incPtr   = incPtr.get();
        w.inc      = inc.get();
        stagedFields(w);
        w.h        = h;
        w.h2       = h * h;
        w.kD       = kD;
        w.detHZero = detHZero;
        w.omega    = 1.f;
        bp.sub     = sp;
        bp.H0      = cheb ? h0.get() : nullptr;
        bp.H1      = cheb ? h1.get() : nullptr;
        bp.omega   = batchOmega.get();
        bp.items   = batchItems.get();
        bp.nItems  = plan.nItems;
        bp.control = batchCounters.get();
        bp.done    = batchCounters.get() + 2;
        bp.flags   = flags.get();
        bp.waitNs  = batchWaitNs;
        bp.poison  = batchPoison;
        check(cudaMemsetAsync(batchCounters.get(), 0, sizeof(int32_t) * (2 + size_t(nMeshes)), stream), "memset");
        check(launch_batched_step(bp, plan.lanes, plan.block, plan.grid, plan.smem, cheb, stream), "batched_step");
    }

    // Enqueue one full step on `stream` (captured into a graph by step()).  Order of the
    // reference GPU integrator (gpu/impl/vbd/Integrator.cu:82-103): contact active set initialised
    // on the full-step prediction, per substep inertial target + initial guess, contact list update,
    // colour sweeps, velocity update; contact active set finalised at the end.
    // Host callbacks of a step run outside a graph (the descent-path traces): after the substep's
    // inertial target and initial guess, at every iterate (k = 0 .. iterations; `current` holds it)
    // and after the velocity update.  plain: plain VBD iterations whatever the acceleration, as the
    // reference's GPU TracedSolve runs them.
    struct StepHooks
    {
        bool plain = false;
        std::function<void(int32_t s)> substepBegin;
        std::function<void(int32_t s, int32_t k, float4 const* current)> iterate;
        std::function<void(int32_t s)> substepEnd;
    };

    void enqueueStep(float dt, int32_t iterations, int32_t substeps, StepHooks const* hooks = nullptr)
    {
        if (!hooks && persistentActive() && plan.iters == iterations && plan.sub == substeps && plan.grid > 0 &&
            plan.lanes == lanesToUse() && plan.block == std::min(block, 256) && plan.tile == batchTile)
        {
            enqueuePersistentStep(dt, iterations, substeps);
            return;
        }
        float const h    = dt / float(substeps);
        float const h2   = h * h;
        bool const plainOnly = hooks && hooks->plain;
        bool const cheb  = !plainOnly && acceleration == PBGB_ACCEL_CHEBYSHEV;
        // Contact reads same-colour partners too, so it always uses the two-buffer sweep (with
        // omega = 1 when there is no acceleration).
        bool const twoBuffer = cheb || contact;
        SubstepParams sp     = substepParams(h);
        if (!twoBuffer)
            sp.h0 = sp.h1 = nullptr;
        else if (iterations > 0)
            sp.result = ((iterations - 1) % 2 == 0) ? h0.get() : h1.get();
        SweepParams w{};
        w.x        = x.get();
        w.xt       = xt.get();
        w.xtilde   = xtilde.get();
        w.tets     = tets.get();
        w.stiff    = incStiff.get();
        w.incPack  = incPack.get();
        w.solve    = solve.get();
        w.incPtr   = incPtr.get();
        w.inc      = inc.get();
        stagedFields(w);
        w.h        = h;
        w.h2       = h2;
        w.kD       = kD;
        w.detHZero = detHZero;
        w.omega    = 1.f;
        w.k        = 0;
        if (contact)
        {
            w.fc     = cFc.get();
            w.F      = cF.get();
            w.XVA    = cXVA.get();
            w.FA     = cFA.get();
            w.vcolor = vcolorD.get();
            w.crec   = cRec.get();
            w.cpen   = cPen.get();
            w.ccount = cCount.get();
            w.muC    = muC;
            w.muF    = muF;
            w.epsv   = epsv;
        }
        int const L = lanesToUse();
        if (profiling)
            ensureEvents(size_t(iterations) * size_t(substeps));
        float4* H[2] = {h0.get(), h1.get()};
        float3 const wmin = make_float3(sceneMin[0], sceneMin[1], sceneMin[2]);
        float3 const wmax = make_float3(sceneMax[0], sceneMax[1], sceneMax[2]);
        if (contact)
        {
            check(contact_predict(nV, x.get(), v.get(), aext.get(), dt, xpred.get(), stream), "contact_predict");
            check(contact_initialize(cmesh, cstate, x.get(), xpred.get(), wmin, wmax, stream), "contact_initialize");
        }
        for (int32_t s = 0; s < substeps; ++s)
        {
            check(launch_begin_substep(sp, stream), "begin_substep");
            if (contact && s % activeSetFreq == 0)
            {
                check(contact_update(cmesh, cstate, x.get(), stream), "contact_update");
                check(launch_contact_records(nV, cFc.get(), cF.get(), cFA.get(), cXVA.get(), vcolorD.get(), muC,
                                             cRec.get(), cPen.get(), cCount.get(), stream),
                      "contact_records");
            }
            if (hooks && hooks->substepBegin)
                hooks->substepBegin(s);
            double omega      = 0.0;
            double const rho2 = rho * rho;
            bool const anderson = !plainOnly && windowed();
            bool const nesterov = !plainOnly && acceleration == PBGB_ACCEL_NESTEROV;
            bool const trust    = !plainOnly && trustLinear();
            TrustParams tp{};
            if (trust)
            {
                if (trLog.size() < size_t(kTrustLogFields) * size_t(iterations) * size_t(substeps))
                    throw std::logic_error("trust-region log not reserved for this step");
                tp.log       = trLog.get();
                trLogEntries = iterations * substeps;
                tp.x        = x.get();
                tp.xkm1     = trXkm1.get();
                tp.energy   = energyParams(h, nullptr);
                tp.state    = trState.get();
                tp.partials = trPartials.get();
                tp.nV       = nV;
                tp.eta      = trEta;
                tp.tau      = trTau;
                if (contact)
                {
                    tp.nActive = cstate.nActive;
                    tp.av      = cstate.av;
                    tp.cV      = cmesh.V;
                    tp.fc      = cFc.get();
                    tp.cF      = cF.get();
                    tp.FA      = cFA.get();
                    tp.XVA     = cXVA.get();
                    tp.xt      = xt.get();
                    tp.muC     = muC;
                    tp.muF     = muF;
                    tp.epsv    = epsv;
                    tp.h       = h;
                }
                // TrustRegionIntegrator::SolveWithLinearAcceleratedPath (:48-170): f at the initial guess.
                check(launch_trust_objective(tp, kTrustInitial, 0, 0, stream), "trust_objective");
            }
            // NesterovIntegrator::Solve (sim/vbd/NesterovIntegrator.cpp:16-43).
            double const neAlpha = 1.0 / nesterovL;
            double neLambda = 0.0, neBeta = 0.0;
            if (nesterov && iterations > 0 && nV > 0)
                check(cudaMemcpyAsync(neX0.get(), x.get(), sizeof(float4) * size_t(nV), cudaMemcpyDeviceToDevice, stream),
                      "nesterov copy");
            AndersonParams ap{};
            if (anderson)
            {
                ap.x        = x.get();
                ap.step     = anStep.get();
                ap.Gkm1     = anGkm1.get();
                ap.Fkm1     = anFkm1.get();
                ap.DF       = anDF.get();
                ap.DG       = anDG.get();
                ap.partials = anPartials.get();
                ap.gram     = anGram.get();
                ap.alpha    = anAlpha.get();
                ap.rhs      = anRhs.get();
                ap.n        = nV;
                ap.m        = window;
                ap.broyden  = acceleration == PBGB_ACCEL_BROYDEN;
                w.step = anStep.get();
            }
            for (int32_t k = 0; k < iterations; ++k)
            {
                if (hooks && hooks->iterate)
                    hooks->iterate(s, k, twoBuffer ? H[(k + 1) % 2] : x.get());
                if (twoBuffer)
                {
                    if (cheb)
                    {
                        omega   = chebyshev_omega<double>(k, rho2, omega, chebFormula);
                        w.omega = float(omega);
                        w.k     = k;
                    }
                    w.hprev = H[(k + 1) % 2];
                    w.hcur  = H[k % 2];
                }
                // With contact the two-buffer sweep keeps the iterate in x and in H[k % 2]; the
                // accelerations update both.
                ap.xh = twoBuffer ? H[k % 2] : nullptr;
                tp.xh = twoBuffer ? H[k % 2] : nullptr;
                if (trust)
                    check(launch_trust_begin(tp, k, stream), "trust_begin");
                bool const neActive = nesterov && nesterovStart < k;
                if (neActive)
                    check(launch_nesterov_extrapolate(nV, x.get(), neX0.get(), neY.get(), float(neBeta), stream),
                          "nesterov_extrapolate");
                size_t const slot = size_t(s) * size_t(iterations) + size_t(k);
                if (profiling)
                    check(cudaEventRecordWithFlags(evBegin[slot], stream, cudaEventRecordExternal), "cudaEventRecord");
                for (int32_t c = 0; c < nColors; ++c)
                {
                    w.begin = colorPtr[c];
                    w.end   = colorPtr[c + 1];
                    w.color = c;
                    check(launch_sweep(w, L, block, twoBuffer, pdl, stream, stagedBytes(c, L)), "sweep");
                }
                if (profiling)
                    check(cudaEventRecordWithFlags(evEnd[slot], stream, cudaEventRecordExternal), "cudaEventRecord");
                int32_t const entry = s * iterations + k;
                if (trust && k < 2)
                    check(launch_trust_objective(tp, kTrustPlain, k, entry, stream), "trust_objective");
                else if (trust)
                {
                    check(launch_trust_step_size(tp, entry, stream), "trust_step_size");
                    check(launch_trust_apply(tp, false, stream), "trust_apply");
                    check(launch_trust_objective(tp, kTrustTrial, k, entry, stream), "trust_objective");
                    check(launch_trust_apply(tp, true, stream), "trust_apply");
                    check(launch_trust_objective(tp, kTrustFinal, k, entry, stream), "trust_objective");
                }
                if (neActive)
                {
                    check(launch_nesterov_update(nV, x.get(), neX0.get(), neY.get(), float(neAlpha), stream),
                          "nesterov_update");
                    double const lk = neLambda;
                    neLambda        = (1.0 + std::sqrt(1.0 + 4.0 * neLambda * neLambda)) / 2.0;
                    neBeta          = (lk - 1.0) / neLambda;
                }
                if (anderson)
                {
                    // AndersonIntegrator::Solve (sim/vbd/AndersonIntegrator.cpp:31-56),
                    // BroydenIntegrator::Solve (sim/vbd/BroydenIntegrator.cpp:41-80).
                    if (k == 0)
                        check(launch_anderson_start(ap, stream), "anderson_start");
                    else
                    {
                        ap.dkl      = (k - 1) % window;
                        ap.mk       = std::min(window, k);
                        ap.maxIters = std::max(1, window - k);
                        ap.next     = k + 1 < iterations ? k % window : -1;
                        check(launch_anderson_window(ap, stream), "anderson_window");
                        check(launch_anderson_solve(ap, stream), "anderson_solve");
                        check(launch_anderson_update(ap, stream), "anderson_update");
                    }
                }
            }
            if (hooks && hooks->iterate)
                hooks->iterate(s, iterations, twoBuffer && iterations > 0 ? sp.result : x.get());
            check(launch_end_substep(sp, stream), "end_substep");
            if (hooks && hooks->substepEnd)
                hooks->substepEnd(s);
        }
        if (contact)
            check(contact_finalize(cmesh, cstate, x.get(), stream), "contact_finalize");
    }

    // Dense Matrix Market ("array" format, column-major) of a rows x cols matrix; value(r, c).
    template <class F>
    static void writeMarket(std::string const& path, int64_t rows, int64_t cols, bool integer, F&& value)
    {
        std::FILE* f = std::fopen(path.c_str(), "w");
        if (!f)
            throw std::invalid_argument("cannot write " + path);
        std::fprintf(f, "%%%%MatrixMarket matrix array %s general\n%lld %lld\n", integer ? "integer" : "real",
                     static_cast<long long>(rows), static_cast<long long>(cols));
        for (int64_t c = 0; c < cols; ++c)
            for (int64_t r = 0; r < rows; ++r)
            {
                if (integer)
                    std::fprintf(f, "%lld\n", static_cast<long long>(value(r, c)));
                else
                    std::fprintf(f, "%.17g\n", static_cast<double>(value(r, c)));
            }
        bool const ok = std::fclose(f) == 0;
        if (!ok)
            throw std::invalid_argument("cannot write " + path);
    }

    // Checkpoint blob: header, x, v, vprev, aext (nV float4 each), then with contact the active
    // flags (nSurfV bytes, padded to 4), search radii (nSurfV float) and contact lists (8 nV int32).
    struct StateHeader
    {
        uint32_t magic;
        uint32_t version;
        int32_t nV;
        int32_t nSurfV;
        int32_t contact;
        int32_t reserved;
    };
    static uint32_t constexpr kStateMagic = 0x53474250u; // "PBGS"

    size_t stateBytes() const
    {
        size_t b = sizeof(StateHeader) + 4 * sizeof(float4) * size_t(nV);
        if (contact)
            b += ((size_t(cmesh.nSurfV) + 3) & ~size_t(3)) + sizeof(float) * size_t(cmesh.nSurfV) +
                 sizeof(int32_t) * 8 * size_t(nV);
        return b;
    }

    template <class F>
    void stateParts(F&& part)
    {
        size_t const v4 = sizeof(float4) * size_t(nV);
        part(static_cast<void*>(x.get()), v4);
        part(static_cast<void*>(v.get()), v4);
        part(static_cast<void*>(vprev.get()), v4);
        part(static_cast<void*>(aext.get()), v4);
        if (contact)
        {
            part(static_cast<void*>(cActive.get()), size_t(cmesh.nSurfV));
            part(nullptr, ((size_t(cmesh.nSurfV) + 3) & ~size_t(3)) - size_t(cmesh.nSurfV)); // padding
            part(static_cast<void*>(cDupper.get()), sizeof(float) * size_t(cmesh.nSurfV));
            part(static_cast<void*>(cFc.get()), sizeof(int32_t) * 8 * size_t(nV));
        }
    }

    void saveState(void* blob, size_t bytes)
    {
        if (bytes < stateBytes())
            throw std::invalid_argument("pbgb_vbd_save_state: buffer smaller than pbgb_vbd_state_size");
        StateHeader hd{kStateMagic, 1u, nV, contact ? cmesh.nSurfV : 0, contact ? 1 : 0, 0};
        auto* out = static_cast<unsigned char*>(blob);
        std::memcpy(out, &hd, sizeof(hd));
        size_t off = sizeof(hd);
        stateParts([&](void* dev, size_t n) {
            if (n == 0)
                return;
            if (dev)
                check(cudaMemcpyAsync(out + off, dev, n, cudaMemcpyDeviceToHost, stream), "D2H");
            else
                std::memset(out + off, 0, n);
            off += n;
        });
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    void loadState(void const* blob, size_t bytes)
    {
        StateHeader hd{};
        if (bytes < sizeof(hd))
            throw std::invalid_argument("pbgb_vbd_load_state: blob too small");
        std::memcpy(&hd, blob, sizeof(hd));
        if (hd.magic != kStateMagic || hd.version != 1u || hd.nV != nV || hd.contact != (contact ? 1 : 0) ||
            hd.nSurfV != (contact ? cmesh.nSurfV : 0) || bytes < stateBytes())
            throw std::invalid_argument("pbgb_vbd_load_state: the blob belongs to another system");
        auto const* in = static_cast<unsigned char const*>(blob);
        size_t off     = sizeof(hd);
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        stateParts([&](void* dev, size_t n) {
            if (dev && n)
                check(cudaMemcpyAsync(dev, in + off, n, cudaMemcpyHostToDevice, stream), "H2D");
            off += n;
        });
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    // deviceToHost of a position array, in world coordinates (mesh origins added).
    std::vector<float4> positionsToHost(float4 const* src)
    {
        std::vector<float4> out = deviceToHost(src);
        if (origin.get())
            for (int32_t b = 0; b < nMeshes; ++b)
                for (int32_t i = meshV0[b]; i < meshV0[b + 1]; ++i)
                {
                    out[size_t(i)].x += meshOrigin[b].x;
                    out[size_t(i)].y += meshOrigin[b].y;
                    out[size_t(i)].z += meshOrigin[b].z;
                }
        return out;
    }

    std::vector<float4> deviceToHost(float4 const* src)
    {
        std::vector<float4> out(static_cast<size_t>(nV));
        if (nV > 0)
            check(cudaMemcpyAsync(out.data(), src, sizeof(float4) * size_t(nV), cudaMemcpyDeviceToHost, stream), "D2H");
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        return out;
    }

    // Integrator::TracedStep of the reference GPU integrator (gpu/impl/vbd/Integrator.cu:105-148,
    // 284-301): on frame 0 the mesh and material (T, M, wg, GP, lame), then per substep the
    // inertial target xtilde.t.{t}.s.{s}.mtx and every iterate x.t.{t}.s.{s}.k.{k}.mtx of plain VBD
    // iterations (k = 0 .. iterations).
    void tracedStep(float dt, int32_t iterations, int32_t substeps, int32_t t, std::string const& dir)
    {
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        auto at = [&](std::string const& name) { return dir + "/" + name; };
        if (t == 0)
        {
            writeMarket(at("T.mtx"), nT, 4, true, [&](int64_t e, int64_t q) {
                uint4 const v = hostRecords[size_t(e)].v;
                uint32_t const c4[4] = {v.x, v.y, v.z, v.w};
                return int64_t(c4[q] & kIndexMask);
            });
            writeMarket(at("M.mtx"), nV, 1, false, [&](int64_t i, int64_t) { return hostM[size_t(i)]; });
            writeMarket(at("wg.mtx"), nT, 1, false, [&](int64_t e, int64_t) { return hostWg[size_t(e)]; });
            // GP: 4 x 3 nT, column 3e + d holding d/dX_d of the 4 shape functions of tet e.
            writeMarket(at("GP.mtx"), 4, 3 * int64_t(nT), false, [&](int64_t a, int64_t c) {
                return hostGP[12 * size_t(c / 3) + 3 * size_t(a) + size_t(c % 3)];
            });
            writeMarket(at("lame.mtx"), nT, 2, false, [&](int64_t e, int64_t q) {
                return q == 0 ? hostMu[size_t(e)] : hostLambda[size_t(e)];
            });
        }
        StepHooks hooks;
        hooks.plain        = true;
        hooks.substepBegin = [&](int32_t s) {
            std::vector<float4> const xt4 = positionsToHost(xtilde.get());
            writeMarket(at("xtilde.t." + std::to_string(t) + ".s." + std::to_string(s) + ".mtx"), nV, 3, false,
                        [&](int64_t i, int64_t c) { return (&xt4[size_t(i)].x)[c]; });
        };
        hooks.iterate = [&](int32_t s, int32_t k, float4 const* current) {
            std::vector<float4> const x4 = positionsToHost(current);
            writeMarket(at("x.t." + std::to_string(t) + ".s." + std::to_string(s) + ".k." + std::to_string(k) + ".mtx"),
                        nV, 3, false, [&](int64_t i, int64_t c) { return (&x4[size_t(i)].x)[c]; });
        };
        enqueueStep(dt, iterations, substeps, &hooks);
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    // The reference CPU integrator's trace of one step (sim/vbd/Integrator.cpp:22-45,202-235): per
    // substep, the FP64 objective, its gradient and the positions at every iterate k = 0 ..
    // iterations (before each VBD iteration, then the result), written as {t}.{s}.f.mtx
    // (iterations+1 x 1), {t}.{s}.grad.mtx and {t}.{s}.x.mtx (3 nV x iterations+1).
    void tracedStepCpuFormat(float dt, int32_t iterations, int32_t substeps)
    {
        reserveTrustLog(iterations, substeps);
        double const h = double(dt) / double(substeps);
        if (gradBuf.size() < size_t(nV) * 3)
            gradBuf.allocate(size_t(nV) * 3);
        std::vector<double> fs, gs, xs;
        StepHooks hooks;
        hooks.iterate = [&](int32_t, int32_t, float4 const* current) {
            check(launch_objective(energyParams(h, red.get(), current), stream), "objective");
            check(cudaMemsetAsync(gradBuf.get(), 0, sizeof(double) * 3 * size_t(nV), stream), "memset");
            check(launch_gradient(energyParams(h, gradBuf.get(), current), stream), "gradient");
            double f = 0.0;
            std::vector<double> g(3 * size_t(nV));
            check(cudaMemcpyAsync(&f, red.get(), sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H");
            if (nV > 0)
                check(cudaMemcpyAsync(g.data(), gradBuf.get(), sizeof(double) * g.size(), cudaMemcpyDeviceToHost, stream), "D2H");
            std::vector<float4> const x4 = positionsToHost(current);
            fs.push_back(f);
            gs.insert(gs.end(), g.begin(), g.end());
            for (auto const& q : x4)
            {
                xs.push_back(q.x);
                xs.push_back(q.y);
                xs.push_back(q.z);
            }
        };
        hooks.substepEnd = [&](int32_t s) {
            std::string const base = tracePath + "/" + std::to_string(traceStep) + "." + std::to_string(s);
            int64_t const n = int64_t(fs.size()), rows = 3 * int64_t(nV);
            writeMarket(base + ".f.mtx", n, 1, false, [&](int64_t r, int64_t) { return fs[size_t(r)]; });
            writeMarket(base + ".grad.mtx", rows, n, false, [&](int64_t r, int64_t c) { return gs[size_t(c * rows + r)]; });
            writeMarket(base + ".x.mtx", rows, n, false, [&](int64_t r, int64_t c) { return xs[size_t(c * rows + r)]; });
            fs.clear();
            gs.clear();
            xs.clear();
        };
        enqueueStep(dt, iterations, substeps, &hooks);
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    // The curved trust-region path moves x exactly as plain VBD does (its constraint solve
    // returns 0, so no accelerated step is ever tried): only the linear path has device work.
    bool trustLinear() const { return acceleration == PBGB_ACCEL_TRUST_REGION && !trCurved; }
    // Anderson and Broyden share the window buffers and kernels.
    bool windowed() const { return acceleration == PBGB_ACCEL_ANDERSON || acceleration == PBGB_ACCEL_BROYDEN; }

    int64_t launchesPerStep(int32_t iterations, int32_t substeps) const
    {
        if (persistentActive() && plan.iters == iterations && plan.sub == substeps && plan.grid > 0)
            return plan.nItems > 0 ? 1 : 0;
        int64_t perIter = 0;
        for (int32_t c = 0; c < nColors; ++c)
            perIter += colorPtr[c + 1] > colorPtr[c] ? 1 : 0;
        int64_t n = int64_t(substeps) * (2 * (nV > 0 ? 1 : 0) + int64_t(iterations) * perIter);
        if (windowed() && iterations > 0)
            n += int64_t(substeps) * (1 + 3 * int64_t(iterations - 1));
        if (acceleration == PBGB_ACCEL_NESTEROV)
            n += int64_t(substeps) * 2 * std::max<int64_t>(0, int64_t(iterations) - 1 - nesterovStart);
        if (trustLinear())
            n += int64_t(substeps) * (1 + 2 * std::min<int64_t>(iterations, 2) +
                                      6 * std::max<int64_t>(0, int64_t(iterations) - 2));
        if (contact)
        {
            // Kernels only (memsets are not counted): the prediction; unless the contact mesh is
            // empty, the vertex and triangle boxes, the LBVH build, the active-set initialization
            // and its compaction; per update the refit (triangle boxes, internal boxes), the
            // nearest query and the contact records; at finalize the refit and the nearest query.
            int64_t const updates = (substeps + activeSetFreq - 1) / activeSetFreq;
            n += 1;
            if (cmesh.nF > 0 && cmesh.nSurfV > 0)
            {
                int64_t const refitK = 1 + bvh_refit_kernels(cmesh.nF);
                n += 2 + bvh_build_kernels(cmesh.nF) + 2 + updates * (refitK + 2) + refitK + 1;
            }
        }
        return n;
    }

    // The trust-region decision log holds one entry per (substep, iteration) of a step; it is
    // grown here, outside any stream capture.
    void reserveTrustLog(int32_t iterations, int32_t substeps)
    {
        size_t const need = size_t(kTrustLogFields) * size_t(std::max(iterations, 1)) * size_t(std::max(substeps, 1));
        if (!trustLinear() || trLog.size() >= need)
            return;
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        graphValid = false;
        dropSlotGraphs();
        trLog.allocate(need);
        check(cudaMemsetAsync(trLog.get(), 0, sizeof(double) * need, stream), "memset");
    }

    void step(float dt, int32_t iterations, int32_t substeps)
    {
        reserveTrustLog(iterations, substeps);
        if (persistentActive())
        {
            int32_t const before = plan.nItems, beforeGrid = plan.grid;
            bool const same = plan.iters == iterations && plan.sub == substeps && plan.lanes == lanesToUse() &&
                              plan.block == std::min(block, 256) && plan.tile == batchTile;
            preparePersistent(iterations, substeps);
            if (!same || before != plan.nItems || beforeGrid != plan.grid)
                graphValid = false;
        }
        if (traceNext)
        {
            traceNext = false;
            tracedStepCpuFormat(dt, iterations, substeps);
            return;
        }
        if (!graphValid || dt != gDt || iterations != gIters || substeps != gSub)
        {
            if (graph)
            {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
            try
            {
                enqueueStep(dt, iterations, substeps);
            }
            catch (...)
            {
                cudaStreamEndCapture(stream, &g);
                if (g)
                    cudaGraphDestroy(g);
                throw;
            }
            check(cudaStreamEndCapture(stream, &g), "cudaStreamEndCapture");
            graphKernels        = countKernelNodes(g);
            cudaError_t const e = cudaGraphInstantiate(&graph, g, 0);
            cudaGraphDestroy(g);
            check(e, "cudaGraphInstantiate");
            gDt        = dt;
            gIters     = iterations;
            gSub       = substeps;
            graphValid = true;
        }
        check(cudaGraphLaunch(graph, stream), "cudaGraphLaunch");
        trLogEntries = trustLinear() ? iterations * substeps : 0;
    }

    // Kernel nodes of a captured graph (the step's graphs hold no child or conditional graphs).
    static int64_t countKernelNodes(cudaGraph_t g)
    {
        size_t count = 0;
        if (cudaGraphGetNodes(g, nullptr, &count) != cudaSuccess)
            return -1;
        std::vector<cudaGraphNode_t> nodes(count);
        if (count > 0 && cudaGraphGetNodes(g, nodes.data(), &count) != cudaSuccess)
            return -1;
        int64_t kernels = 0;
        for (size_t i = 0; i < count; ++i)
        {
            cudaGraphNodeType type;
            if (cudaGraphNodeGetType(nodes[i], &type) != cudaSuccess)
                return -1;
            kernels += type == cudaGraphNodeTypeKernel ? 1 : 0;
        }
        return kernels;
    }

    // Project-written autotuner: times one replayed step per candidate (lanes per vertex x block
    // size) with CUDA events on the handle's stream, restoring the state after each candidate, and
    // keeps the fastest.  Results are cached per (vertices, tets, colours) bucket.
    struct TuneKey
    {
        int64_t nV, nT, nC, iters, sub;
        int32_t accel;
        bool contact;
        bool persistent;
        bool operator==(TuneKey const& o) const
        {
            return nV == o.nV && nT == o.nT && nC == o.nC && iters == o.iters && sub == o.sub && accel == o.accel &&
                   contact == o.contact && persistent == o.persistent;
        }
    };
    struct TuneEntry
    {
        TuneKey key;
        int32_t lanes, block;
        float ms;
    };
    static std::vector<TuneEntry>& tuneCache()
    {
        static std::vector<TuneEntry> cache;
        return cache;
    }

    void autotune(float dt, int32_t iterations, int32_t substeps, int32_t* bestLanes, int32_t* bestBlock, float* bestMs)
    {
        static std::mutex cacheMutex;
        // Size buckets: powers of two of the vertex and tet counts.
        auto bucket = [](int64_t n) {
            int64_t b = 1;
            while (b < n)
                b <<= 1;
            return b;
        };
        TuneKey const key{bucket(nV), bucket(nT), nColors, iterations, substeps, acceleration, contact, persistentActive()};
        {
            std::lock_guard<std::mutex> lock(cacheMutex);
            for (auto const& e : tuneCache())
                if (e.key == key)
                {
                    lanes = e.lanes;
                    block = e.block;
                    invalidate();
                    *bestLanes = e.lanes;
                    *bestBlock = e.block;
                    *bestMs    = e.ms;
                    return;
                }
        }
        // Snapshot the state the steps modify (the checkpoint's parts: positions, velocities,
        // external accelerations and, with contact, the active set and contact lists).
        DeviceArray<unsigned char> snap;
        snap.allocate(stateBytes());
        {
            size_t off = 0;
            stateParts([&](void* dev, size_t n) {
                if (dev && n > 0)
                    check(cudaMemcpyAsync(snap.get() + off, dev, n, cudaMemcpyDeviceToDevice, stream), "snapshot");
                off += n;
            });
        }
        auto restore = [&] {
            size_t off = 0;
            stateParts([&](void* dev, size_t n) {
                if (dev && n > 0)
                    check(cudaMemcpyAsync(dev, snap.get() + off, n, cudaMemcpyDeviceToDevice, stream), "restore");
                off += n;
            });
        };
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        check(cudaEventCreate(&e0), "cudaEventCreate");
        check(cudaEventCreate(&e1), "cudaEventCreate");
        int32_t const savedLanes = lanes, savedBlock = block;
        bool const savedProfiling = profiling;
        profiling = false;
        float best = -1.f;
        int32_t bl = lanesToUse(), bb = block;
        try
        {
            int32_t const laneSet[]  = {1, 2, 4, 8, 16, 32};
            // Odd warp multiples as well: a colour's blocks then spread more evenly over the SMs
            // (the beam's 33.6k-vertex colours: 601 blocks of 224 against 525 of 256 on 152 SMs).
            int32_t const blockSet[] = {64, 96, 128, 160, 192, 224, 256};
            for (int32_t L : laneSet)
                for (int32_t B : blockSet)
                {
                    lanes = L;
                    block = B;
                    invalidate();
                    step(dt, iterations, substeps); // capture + warm-up
                    restore();
                    // The faster of two timed steps from the same state (one step alone picked a
                    // 17 % slower launch for the contact scene now and then).
                    float ms = -1.f;
                    for (int rep = 0; rep < 2; ++rep)
                    {
                        check(cudaEventRecord(e0, stream), "cudaEventRecord");
                        step(dt, iterations, substeps);
                        check(cudaEventRecord(e1, stream), "cudaEventRecord");
                        restore();
                        check(cudaEventSynchronize(e1), "cudaEventSynchronize");
                        float t = 0.f;
                        check(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime");
                        ms = ms < 0.f || t < ms ? t : ms;
                    }
                    if (best < 0.f || ms < best)
                    {
                        best = ms;
                        bl   = L;
                        bb   = B;
                    }
                }
        }
        catch (...)
        {
            lanes     = savedLanes;
            block     = savedBlock;
            profiling = savedProfiling;
            invalidate();
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaStreamSynchronize(stream);
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        check(cudaMemsetAsync(flags.get(), 0, sizeof(int32_t), stream), "cudaMemsetAsync");
        lanes     = bl;
        block     = bb;
        profiling = savedProfiling;
        invalidate();
        {
            std::lock_guard<std::mutex> lock(cacheMutex);
            tuneCache().push_back(TuneEntry{key, bl, bb, best});
        }
        *bestLanes = bl;
        *bestBlock = bb;
        *bestMs    = best;
    }

    int synchronize()
    {
        check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        int32_t f[2] = {0, 0};
        check(cudaMemcpy(f, flags.get(), sizeof(f), cudaMemcpyDeviceToHost), "cudaMemcpy");
        if (f[1] != 0)
        {
            check(cudaMemset(flags.get(), 0, sizeof(f)), "cudaMemset");
            lastError = "a bounded device wait of the persistent batched step gave up; the step's positions are not valid";
            return kTimeout;
        }
        if (f[0] != 0)
        {
            check(cudaMemset(flags.get(), 0, sizeof(int32_t)), "cudaMemset");
            lastError = "non-finite positions or velocities detected on the device";
            return kNonFinite;
        }
        return kOk;
    }

    // Host transfers of a per-vertex vector; positions = true adds / subtracts the mesh origins.
    void getVec(DeviceArray<float4> const& src, float* host, bool positions = false)
    {
        check(launch_unpack3(src.get(), staging.get(), nV, stream, positions ? origin.get() : nullptr), "unpack");
        check(cudaMemcpyAsync(host, staging.get(), sizeof(float) * 3 * size_t(nV), cudaMemcpyDeviceToHost, stream), "D2H");
    }
    void setVec(DeviceArray<float4>& dst, float const* host, bool positions = false)
    {
        check(cudaMemcpyAsync(staging.get(), host, sizeof(float) * 3 * size_t(nV), cudaMemcpyHostToDevice, stream), "H2D");
        check(launch_pack3(staging.get(), dst.get(), nV, stream, positions ? origin.get() : nullptr), "pack");
    }

    EnergyParams energyParams(double dt, double* out, float4 const* at = nullptr) const
    {
        EnergyParams p{};
        p.x      = at ? at : x.get();
        p.xtilde = xtilde.get();
        p.m      = m.get();
        p.tets   = tets.get();
        p.X      = X.get();
        p.nV     = nV;
        p.nT     = nT;
        p.dt2    = dt * dt;
        p.out    = out;
        p.partials = objPartials.get();
        p.restEnergy = restEnergy();
        return p;
    }

    // sum_e wg_e mu_e^2 / (2 lambda_e), the elastic energy of the rest state (cached until the
    // material changes).
    double restEnergy() const
    {
        if (!restEnergyValid)
        {
            double e = 0.0;
            for (size_t t = 0; t < hostWg.size(); ++t)
                e += hostWg[t] * hostMu[t] * hostMu[t] / (2.0 * hostLambda[t]);
            restEnergyCache = e;
            restEnergyValid = true;
        }
        return restEnergyCache;
    }
    mutable double restEnergyCache = 0.0;
    mutable bool restEnergyValid   = false;
};

} // namespace pbgb

struct pbgb_vbd
{
    pbgb::VbdSystem sys;
    // Device address of the fixed accumulation array of pbgb_vbd_gradient_noalloc on the handle's
    // device, looked up when the handle is created.
    double* noallocScratch = nullptr;
};

namespace {

using pbgb::kCuda;
using pbgb::kInternal;
using pbgb::kInvalid;
using pbgb::kOk;
using pbgb::check;

int fail(pbgb_vbd* h, int code, std::string const& msg)
{
    pbgb::gLastError = msg;
    if (h)
        h->sys.lastError = msg;
    return code;
}

// Runs `f` with C++ exceptions mapped to status codes.
template <class F>
int guarded(pbgb_vbd* h, F&& f)
{
    try
    {
        return f();
    }
    catch (pbgb::CudaFailure const& e)
    {
        return fail(h, kCuda, std::string(e.what) + ": " + cudaGetErrorString(e.err));
    }
    catch (std::invalid_argument const& e)
    {
        return fail(h, kInvalid, e.what());
    }
    catch (std::bad_alloc const&)
    {
        return fail(h, kInternal, "host allocation failed");
    }
    catch (std::exception const& e)
    {
        return fail(h, kInternal, e.what());
    }
    catch (...)
    {
        return fail(h, kInternal, "unknown error");
    }
}

// Fixed device array of pbgb_vbd_gradient_noalloc: one FP64 accumulator per vertex coordinate.
// Every device on which this library's module is loaded holds it until the process exits.
__device__ __align__(256) double gNoAllocGradient[3 * PBGB_NOALLOC_MAX_VERTICES];

// Looks up the array's address on the current device.  In host code gNoAllocGradient is only a
// stand-in for the symbol, not an address the GPU can use; cudaGetSymbolAddress also loads the
// module on the device (the array is reserved there then), so that the entry point's own calls
// neither allocate nor load anything.
double* noalloc_scratch_address()
{
    void* p = nullptr;
    check(cudaGetSymbolAddress(&p, gNoAllocGradient), "cudaGetSymbolAddress");
    return static_cast<double*>(p);
}

int create_impl(pbgb_vbd_desc const* descs, int32_t n, pbgb_vbd** out)
{
    if (!descs || n < 1 || !out)
        return fail(nullptr, kInvalid, "pbgb_vbd_create: null argument or empty batch");
    *out = nullptr;
    // Descriptor errors are reported whether or not a device is present.
    int const rc0 = guarded(nullptr, [&] {
        pbgb::validate_descs(descs, n);
        return int(kOk);
    });
    if (rc0 != kOk)
        return rc0;
    int devices = 0;
    if (cudaGetDeviceCount(&devices) != cudaSuccess || devices < 1)
    {
        cudaGetLastError();
        return fail(nullptr, pbgb::kNoDevice, "no CUDA device available");
    }
    auto h = std::make_unique<pbgb_vbd>();
    int const rc = guarded(h.get(), [&] {
        h->sys.build(descs, n);
        // build() made no device current other than the one the handle lives on.
        h->noallocScratch = noalloc_scratch_address();
        return int(kOk);
    });
    if (rc != kOk)
    {
        pbgb::gLastError = h->sys.lastError;
        return rc;
    }
    *out = h.release();
    return kOk;
}

} // namespace

extern "C" {

PBGB_API int pbgb_vbd_data_construct(
    int32_t nV,
    int32_t nT,
    const double* X,
    const int32_t* T,
    const double* rhoe,
    const int32_t* dbc,
    int32_t nDbc,
    int32_t ordering,
    int32_t selection,
    double* m,
    double* GP,
    double* wg,
    int32_t* GVGp,
    int32_t* GVGe,
    int32_t* GVGilocal,
    int32_t* colors,
    int32_t* Pptr,
    int32_t* nPartitions,
    int32_t* Padj,
    int32_t* nPadj)
{
    if (!m || !GP || !wg || !GVGp || !GVGe || !GVGilocal || !colors || !Pptr || !nPartitions || !Padj ||
        !nPadj || (nDbc > 0 && !dbc))
        return fail(nullptr, kInvalid, "pbgb_vbd_data_construct: null output");
    return guarded(nullptr, [&] {
        pbgb::ConstructIn in{nV, nT, X, T, rhoe, dbc, nDbc, ordering, selection};
        pbgb::ConstructOut out{m, GP, wg, GVGp, GVGe, GVGilocal, colors, Pptr, Padj, 0, 0};
        int const rc = pbgb::construct(in, out);
        if (rc == pbgb::kDegenerate)
            return fail(nullptr, rc, "tetrahedron with non-positive volume");
        if (rc == pbgb::kPalette)
            return fail(nullptr, rc, "greedy colouring needs more than 128 colours");
        if (rc != kOk)
            return fail(nullptr, rc, "invalid mesh description");
        *nPartitions = out.nPartitions;
        *nPadj       = out.nPadj;
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_create(const pbgb_vbd_desc* desc, pbgb_vbd** out)
{
    return create_impl(desc, 1, out);
}

PBGB_API int pbgb_vbd_create_batched(const pbgb_vbd_desc* descs, int32_t n_meshes, pbgb_vbd** out)
{
    return create_impl(descs, n_meshes, out);
}

PBGB_API int pbgb_vbd_destroy(pbgb_vbd* h)
{
    if (!h)
        return kOk;
    if (h->sys.stream)
        cudaStreamSynchronize(h->sys.stream);
    delete h;
    return kOk;
}

PBGB_API int pbgb_vbd_step(pbgb_vbd* h, float dt, int32_t iterations, int32_t substeps)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!(dt > 0.f) || !std::isfinite(dt) || iterations < 0 || substeps < 1)
        return fail(h, kInvalid, "pbgb_vbd_step: expected dt > 0, iterations >= 0, substeps >= 1");
    return guarded(h, [&] {
        h->sys.step(dt, iterations, substeps);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_traced_step(pbgb_vbd* h, float dt, int32_t iterations, int32_t substeps, int32_t t, const char* dir)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!dir || !(dt > 0.f) || !std::isfinite(dt) || iterations < 0 || substeps < 1)
        return fail(h, kInvalid, "pbgb_vbd_traced_step: expected a directory, dt > 0, iterations >= 0, substeps >= 1");
    return guarded(h, [&] {
        h->sys.tracedStep(dt, iterations, substeps, t, std::string(dir));
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_trace_next_step(pbgb_vbd* h, const char* path, int32_t t)
{
    if (!h || !path)
        return fail(h, kInvalid, "null argument");
    h->sys.traceNext = true;
    h->sys.tracePath = path;
    h->sys.traceStep = t;
    return kOk;
}

PBGB_API int pbgb_vbd_synchronize(pbgb_vbd* h)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    return guarded(h, [&] {
        int const rc = h->sys.synchronize();
        if (rc != kOk)
            pbgb::gLastError = h->sys.lastError;
        return rc;
    });
}

#define PBGB_CHECK_HANDLE_PTR(h, p)                                                                \
    if (!(h))                                                                                      \
        return fail(nullptr, kInvalid, "null handle");                                             \
    if (!(p) && (h)->sys.nV > 0)                                                                   \
        return fail((h), kInvalid, "null buffer");

PBGB_API int pbgb_vbd_get_positions(pbgb_vbd* h, float* x)
{
    PBGB_CHECK_HANDLE_PTR(h, x)
    return guarded(h, [&] {
        h->sys.getVec(h->sys.x, x, true);
        return h->sys.synchronize();
    });
}

PBGB_API int pbgb_vbd_set_positions(pbgb_vbd* h, const float* x)
{
    PBGB_CHECK_HANDLE_PTR(h, x)
    return guarded(h, [&] {
        h->sys.setVec(h->sys.x, x, true);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_get_velocities(pbgb_vbd* h, float* v)
{
    PBGB_CHECK_HANDLE_PTR(h, v)
    return guarded(h, [&] {
        h->sys.getVec(h->sys.v, v);
        return h->sys.synchronize();
    });
}

PBGB_API int pbgb_vbd_set_velocities(pbgb_vbd* h, const float* v)
{
    PBGB_CHECK_HANDLE_PTR(h, v)
    return guarded(h, [&] {
        h->sys.setVec(h->sys.v, v);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_external_acceleration(pbgb_vbd* h, const float* a)
{
    PBGB_CHECK_HANDLE_PTR(h, a)
    return guarded(h, [&] {
        h->sys.setVec(h->sys.aext, a);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_get_positions_device(pbgb_vbd* h, float* x_dev)
{
    PBGB_CHECK_HANDLE_PTR(h, x_dev)
    return guarded(h, [&] {
        pbgb::check(pbgb::launch_unpack3(h->sys.x.get(), x_dev, h->sys.nV, h->sys.stream, h->sys.origin.get()), "unpack");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_positions_device(pbgb_vbd* h, const float* x_dev)
{
    PBGB_CHECK_HANDLE_PTR(h, x_dev)
    return guarded(h, [&] {
        pbgb::check(pbgb::launch_pack3(x_dev, h->sys.x.get(), h->sys.nV, h->sys.stream, h->sys.origin.get()), "pack");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_get_velocities_device(pbgb_vbd* h, float* v_dev)
{
    PBGB_CHECK_HANDLE_PTR(h, v_dev)
    return guarded(h, [&] {
        pbgb::check(pbgb::launch_unpack3(h->sys.v.get(), v_dev, h->sys.nV, h->sys.stream), "unpack");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_velocities_device(pbgb_vbd* h, const float* v_dev)
{
    PBGB_CHECK_HANDLE_PTR(h, v_dev)
    return guarded(h, [&] {
        pbgb::check(pbgb::launch_pack3(v_dev, h->sys.v.get(), h->sys.nV, h->sys.stream), "pack");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_state_size(pbgb_vbd* h, size_t* bytes)
{
    if (!h || !bytes)
        return fail(h, kInvalid, "null argument");
    *bytes = h->sys.stateBytes();
    return kOk;
}

PBGB_API int pbgb_vbd_save_state(pbgb_vbd* h, void* blob, size_t bytes)
{
    if (!h || !blob)
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        h->sys.saveState(blob, bytes);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_load_state(pbgb_vbd* h, const void* blob, size_t bytes)
{
    if (!h || !blob)
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        h->sys.loadState(blob, bytes);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_material(pbgb_vbd* h, const double* mu, const double* lambda)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (h->sys.nT > 0 && (!mu || !lambda))
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        h->sys.setMaterial(mu, lambda);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_adjoint_reserve(pbgb_vbd* h, int32_t slots, int32_t iterations)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    return guarded(h, [&] {
        h->sys.adjointReserve(slots, iterations);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_step_record(pbgb_vbd* h, float dt, int32_t iterations, int32_t substeps, int32_t slot)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!(dt > 0.f) || !std::isfinite(dt) || iterations < 0 || substeps < 1)
        return fail(h, kInvalid, "pbgb_vbd_step_record: expected dt > 0, iterations >= 0, substeps >= 1");
    return guarded(h, [&] {
        h->sys.recordStep(dt, iterations, substeps, slot);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_step_adjoint(
    pbgb_vbd* h,
    int32_t slot,
    int32_t substeps,
    float* xbar_dev,
    float* vbar_dev,
    double* dlogmu_dev,
    double* dloglambda_dev)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!xbar_dev || !vbar_dev || (h->sys.nT > 0 && (!dlogmu_dev || !dloglambda_dev)))
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        auto& s = h->sys;
        if (s.strategy == PBGB_INIT_ADAPTIVE_VBD && s.semantics == PBGB_SEMANTICS_GPU)
            throw std::invalid_argument(
                "pbgb_vbd_step_adjoint: AdaptiveVbd with the GPU integrator's semantics reads the previous velocity; "
                "use pbgb_vbd_step_adjoint_state, which carries its adjoint");
        if (s.nV > 0)
            check(cudaMemsetAsync(s.adjZero.get(), 0, sizeof(float) * 3 * size_t(s.nV), s.stream), "memset");
        s.adjointStep(slot, substeps, xbar_dev, vbar_dev, s.adjZero.get(), dlogmu_dev, dloglambda_dev);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_step_adjoint_state(
    pbgb_vbd* h,
    int32_t slot,
    int32_t substeps,
    float* xbar_dev,
    float* vbar_dev,
    float* vprevbar_dev,
    double* dlogmu_dev,
    double* dloglambda_dev)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!xbar_dev || !vbar_dev || !vprevbar_dev || (h->sys.nT > 0 && (!dlogmu_dev || !dloglambda_dev)))
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        h->sys.adjointStep(slot, substeps, xbar_dev, vbar_dev, vprevbar_dev, dlogmu_dev, dloglambda_dev);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_get_previous_velocities_device(pbgb_vbd* h, float* p_dev)
{
    if (!h || !p_dev)
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        pbgb::check(pbgb::launch_unpack3(h->sys.vprev.get(), p_dev, h->sys.nV, h->sys.stream), "unpack");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_previous_velocities_device(pbgb_vbd* h, const float* p_dev)
{
    if (!h || !p_dev)
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        pbgb::check(pbgb::launch_pack3(p_dev, h->sys.vprev.get(), h->sys.nV, h->sys.stream), "pack");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_detH_zero(pbgb_vbd* h, float zero)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    h->sys.detHZero = zero;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_set_damping(pbgb_vbd* h, float kD)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    h->sys.kD = kD;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_set_strategy(pbgb_vbd* h, int32_t strategy)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (strategy < 0 || strategy > 4)
        return fail(h, kInvalid, "invalid initialization strategy");
    h->sys.strategy = strategy;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_set_block_size(pbgb_vbd* h, int32_t block_size)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    // Clamp like the reference (gpu/impl/vbd/Integrator.cu:158-161), rounded to a warp multiple.
    int32_t b = std::clamp(block_size, int32_t(32), int32_t(256));
    h->sys.block = (b + 31) / 32 * 32;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_set_lanes_per_vertex(pbgb_vbd* h, int32_t lanes)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
        return fail(h, kInvalid, "lanes per vertex must be 0, 1, 2, 4, 8, 16 or 32");
    h->sys.lanes = lanes;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_autotune(
    pbgb_vbd* h,
    float dt,
    int32_t iterations,
    int32_t substeps,
    int32_t* lanes,
    int32_t* block_size,
    float* ms_per_step)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!(dt > 0.f) || iterations < 0 || substeps < 1)
        return fail(h, kInvalid, "pbgb_vbd_autotune: expected dt > 0, iterations >= 0, substeps >= 1");
    return guarded(h, [&] {
        int32_t l = 0, b = 0;
        float ms  = 0.f;
        h->sys.autotune(dt, iterations, substeps, &l, &b, &ms);
        if (lanes)
            *lanes = l;
        if (block_size)
            *block_size = b;
        if (ms_per_step)
            *ms_per_step = ms;
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_set_staged_sweep(pbgb_vbd* h, int32_t enable)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    h->sys.staged = enable != 0;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_staged_sweep(pbgb_vbd* h, int32_t* available, int32_t* enabled)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (available)
        *available = h->sys.stagedOk ? 1 : 0;
    if (enabled)
        *enabled = h->sys.staged ? 1 : 0;
    return kOk;
}

PBGB_API int pbgb_vbd_set_programmatic_launch(pbgb_vbd* h, int32_t enable)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    h->sys.pdl = enable != 0;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_set_persistent(pbgb_vbd* h, int32_t enable)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    h->sys.persistent = enable != 0;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_persistent(pbgb_vbd* h, int32_t* active)
{
    if (!h || !active)
        return fail(h, kInvalid, "null argument");
    *active = h->sys.persistentActive() ? 1 : 0;
    return kOk;
}

PBGB_API int pbgb_vbd_set_batch_tile(pbgb_vbd* h, int32_t subtiles)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (subtiles < 1 || subtiles > 64)
        return fail(h, kInvalid, "pbgb_vbd_set_batch_tile: expected 1 <= subtiles <= 64");
    h->sys.batchTile = subtiles;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_debug_batched_wait(pbgb_vbd* h, int64_t wait_ns, int32_t poison_item)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (wait_ns < 1000 || wait_ns > pbgb::kBatchWaitNs || poison_item < -1)
        return fail(h, kInvalid, "pbgb_debug_batched_wait: expected 1 us <= wait_ns <= 2 s and poison_item >= -1");
    h->sys.batchWaitNs = wait_ns;
    h->sys.batchPoison = poison_item;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_set_scene_bounding_box(pbgb_vbd* h, const float* min3, const float* max3)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (!min3 || !max3)
        return fail(h, kInvalid, "null bounding box");
    for (int k = 0; k < 3; ++k)
    {
        h->sys.sceneMin[k] = min3[k];
        h->sys.sceneMax[k] = max3[k];
    }
    return kOk;
}

PBGB_API int pbgb_vbd_set_sweep_timing(pbgb_vbd* h, int32_t enable)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    h->sys.profiling = enable != 0;
    h->sys.invalidate();
    return kOk;
}

PBGB_API int pbgb_vbd_sweep_timing(pbgb_vbd* h, double* milliseconds, int64_t* sweep_launches)
{
    if (!h || !milliseconds || !sweep_launches)
        return fail(h, kInvalid, "null argument");
    if (!h->sys.profiling || !h->sys.graphValid)
        return fail(h, kInvalid, "sweep timing is off or no step was taken since it was enabled");
    return guarded(h, [&] {
        auto& s = h->sys;
        check(cudaStreamSynchronize(s.stream), "cudaStreamSynchronize");
        *milliseconds = s.sweepMilliseconds(s.gIters, s.gSub);
        int64_t nonEmpty = 0;
        for (int32_t c = 0; c < s.nColors; ++c)
            nonEmpty += s.colorPtr[c + 1] > s.colorPtr[c] ? 1 : 0;
        *sweep_launches = nonEmpty * int64_t(s.gIters) * int64_t(s.gSub);
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_sizes(pbgb_vbd* h, int32_t* n_vertices, int32_t* n_tets, int32_t* n_free, int32_t* n_colors)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    if (n_vertices)
        *n_vertices = h->sys.nV;
    if (n_tets)
        *n_tets = h->sys.nT;
    if (n_free)
        *n_free = h->sys.nFree;
    if (n_colors)
        *n_colors = h->sys.nColors;
    return kOk;
}

PBGB_API int pbgb_vbd_launches_per_step(pbgb_vbd* h, int32_t iterations, int32_t substeps, int64_t* launches)
{
    if (!h || !launches)
        return fail(h, kInvalid, "null argument");
    *launches = h->sys.launchesPerStep(iterations, substeps);
    return kOk;
}

PBGB_API int pbgb_vbd_step_graph_kernels(pbgb_vbd* h, int64_t* kernels)
{
    if (!h || !kernels)
        return fail(h, kInvalid, "null argument");
    *kernels = h->sys.graphKernels;
    return kOk;
}

PBGB_API int pbgb_vbd_stream(pbgb_vbd* h, void** stream)
{
    if (!h || !stream)
        return fail(h, kInvalid, "null argument");
    *stream = static_cast<void*>(h->sys.stream);
    return kOk;
}

PBGB_API int pbgb_vbd_get_contacts(pbgb_vbd* h, int32_t* fc, uint8_t* active)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    return guarded(h, [&] {
        auto& s = h->sys;
        check(cudaStreamSynchronize(s.stream), "cudaStreamSynchronize");
        if (!s.contact)
        {
            if (fc)
                std::fill(fc, fc + size_t(s.nV) * pbgb::kMaxContacts, -1);
            return int(kOk);
        }
        if (fc)
            check(cudaMemcpy(fc, s.cFc.get(), sizeof(int32_t) * size_t(s.nV) * pbgb::kMaxContacts, cudaMemcpyDeviceToHost), "D2H");
        if (active)
            check(cudaMemcpy(active, s.cActive.get(), size_t(s.cmesh.nSurfV), cudaMemcpyDeviceToHost), "D2H");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_get_contact_bvh(
    pbgb_vbd* h,
    uint32_t* codes,
    int32_t* inds,
    int32_t* child,
    int32_t* parent,
    int32_t* rightmost,
    float* xpred,
    float* scene_box)
{
    if (!h)
        return fail(nullptr, kInvalid, "null handle");
    return guarded(h, [&] {
        auto& s = h->sys;
        if (!s.contact)
            throw std::invalid_argument("pbgb_vbd_get_contact_bvh: the integrator has no contact");
        check(cudaStreamSynchronize(s.stream), "cudaStreamSynchronize");
        auto const& B   = s.cstate.bvh;
        size_t const nF = size_t(s.cmesh.nF);
        auto get = [&](void* dst, void const* src, size_t bytes) {
            if (dst && bytes > 0)
                check(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), "D2H");
        };
        get(codes, B.codes, sizeof(uint32_t) * nF);
        get(inds, B.inds, sizeof(int32_t) * nF);
        if (nF > 1)
        {
            get(child, B.child, sizeof(int32_t) * 2 * (nF - 1));
            get(rightmost, B.rightmost, sizeof(int32_t) * 2 * (nF - 1));
        }
        get(parent, B.parent, sizeof(int32_t) * (2 * nF - 1));
        if (xpred)
        {
            std::vector<float4> const p4 = s.deviceToHost(s.xpred.get());
            for (size_t i = 0; i < p4.size(); ++i)
            {
                xpred[3 * i]     = p4[i].x;
                xpred[3 * i + 1] = p4[i].y;
                xpred[3 * i + 2] = p4[i].z;
            }
        }
        if (scene_box)
            for (int k = 0; k < 3; ++k)
            {
                scene_box[k]     = s.sceneMin[k];
                scene_box[3 + k] = s.sceneMax[k];
            }
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_objective(pbgb_vbd* h, double dt, double* f)
{
    if (!h || !f)
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        auto& s = h->sys;
        pbgb::check(pbgb::launch_objective(s.energyParams(dt, s.red.get()), s.stream), "objective");
        pbgb::check(cudaMemcpyAsync(f, s.red.get(), sizeof(double), cudaMemcpyDeviceToHost, s.stream), "D2H");
        pbgb::check(cudaStreamSynchronize(s.stream), "sync");
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_trust_region_log(pbgb_vbd* h, double* out, int32_t capacity, int32_t* count)
{
    if (!h || !count || capacity < 0)
        return fail(h, kInvalid, "null argument or negative capacity");
    return guarded(h, [&] {
        auto& s = h->sys;
        if (!s.trustLinear())
            throw std::invalid_argument("the integrator does not run the linear trust-region path");
        *count        = s.trLogEntries;
        int32_t const n = std::min(capacity, s.trLogEntries);
        if (out && n > 0)
        {
            pbgb::check(cudaMemcpyAsync(out, s.trLog.get(), sizeof(double) * pbgb::kTrustLogFields * size_t(n),
                                        cudaMemcpyDeviceToHost, s.stream),
                        "D2H");
            pbgb::check(cudaStreamSynchronize(s.stream), "sync");
        }
        return int(kOk);
    });
}

PBGB_API int pbgb_vbd_gradient(pbgb_vbd* h, double dt, double* grad)
{
    if (!h || !grad)
        return fail(h, kInvalid, "null argument");
    return guarded(h, [&] {
        auto& s = h->sys;
        if (s.gradBuf.size() < size_t(s.nV) * 3)
            s.gradBuf.allocate(size_t(s.nV) * 3);
        double* d = s.gradBuf.get();
        pbgb::check(cudaMemsetAsync(d, 0, sizeof(double) * 3 * size_t(s.nV), s.stream), "memset");
        pbgb::check(pbgb::launch_gradient(s.energyParams(dt, d), s.stream), "gradient");
        pbgb::check(cudaMemcpyAsync(grad, d, sizeof(double) * 3 * size_t(s.nV), cudaMemcpyDeviceToHost, s.stream), "D2H");
        pbgb::check(cudaStreamSynchronize(s.stream), "sync");
        return int(kOk);
    });
}

} // extern "C"

extern "C" {

PBGB_API int pbgb_vbd_gradient_noalloc(pbgb_vbd* h, double dt, double* grad)
{
    if (!h || !grad)
        return fail(h, kInvalid, "null argument");
    if (h->sys.nV > PBGB_NOALLOC_MAX_VERTICES)
        return fail(
            h,
            kInvalid,
            "pbgb_vbd_gradient_noalloc: " + std::to_string(h->sys.nV) + " vertices exceed the fixed scratch of " +
                std::to_string(PBGB_NOALLOC_MAX_VERTICES) + " vertices; use pbgb_vbd_gradient");
    if (!h->noallocScratch)
        return fail(h, kInternal, "pbgb_vbd_gradient_noalloc: the handle has no scratch address");
    return guarded(h, [&] {
        auto& s  = h->sys;
        double* d = h->noallocScratch;
        // Stream-ordered calls on the handle's own stream: no device switch is needed (the stream
        // belongs to the handle's device).  The used part of the shared array starts at zero.
        check(cudaMemsetAsync(d, 0, sizeof(double) * 3 * size_t(s.nV), s.stream), "cudaMemsetAsync");
        check(pbgb::launch_gradient(s.energyParams(dt, d), s.stream), "gradient");
        check(cudaMemcpyAsync(grad, d, sizeof(double) * 3 * size_t(s.nV), cudaMemcpyDeviceToHost, s.stream), "D2H");
        check(cudaStreamSynchronize(s.stream), "cudaStreamSynchronize");
        return int(kOk);
    });
}

PBGB_API const char* pbgb_last_error(pbgb_vbd* h)
{
    if (h)
        return h->sys.lastError.c_str();
    return pbgb::gLastError.c_str();
}

PBGB_API int pbgb_debug_vertex_triangle_contact(
    const float* xtv,
    const float* xv,
    const float* xtf,
    const float* xf,
    float dt,
    float muC,
    float muF,
    float epsv,
    float* g,
    float* H,
    float* energy)
{
    if (!xtv || !xv || !xtf || !xf || !g || !H)
        return fail(nullptr, kInvalid, "pbgb_debug_vertex_triangle_contact: null argument");
    float tf[3][3], f[3][3];
    for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r)
        {
            tf[k][r] = xtf[3 * k + r];
            f[k][r]  = xf[3 * k + r];
        }
    float Hs[6] = {H[0], H[3], H[6], H[4], H[7], H[8]};
    float const E = pbgb::vertex_triangle_contact(xtv, xv, tf, f, dt, muC, muF, epsv, FLT_EPSILON, g, Hs);
    H[0] = Hs[0], H[1] = Hs[1], H[2] = Hs[2];
    H[3] = Hs[1], H[4] = Hs[3], H[5] = Hs[4];
    H[6] = Hs[2], H[7] = Hs[4], H[8] = Hs[5];
    if (energy)
        *energy = E;
    return kOk;
}

PBGB_API int pbgb_debug_adjoint_tet(
    int32_t precision,
    const double* xe,
    const double* Xe,
    int32_t il,
    const double* w,
    const double* delta,
    double muw,
    double law,
    double* dphi,
    double* dlogmu,
    double* dloglambda)
{
    if (!xe || !Xe || !w || !delta || !dphi || !dlogmu || !dloglambda || il < 0 || il > 3 ||
        (precision != 32 && precision != 64))
        return fail(nullptr, kInvalid, "pbgb_debug_adjoint_tet: invalid argument");
    auto run = [&](auto zero) {
        using T = decltype(zero);
        T d[3][3], e[3][3], G[3][3], c[3][3];
        T const tw[3] = {T(w[0]), T(w[1]), T(w[2])};
        T const td[3] = {T(delta[0]), T(delta[1]), T(delta[2])};
        for (int m = 0; m < 3; ++m)
        {
            int const a = (il + 1 + m) & 3;
            for (int r = 0; r < 3; ++r)
            {
                d[m][r] = T(xe[3 * a + r]) - T(xe[3 * il + r]);
                e[m][r] = T(Xe[3 * a + r]) - T(Xe[3 * il + r]);
            }
        }
        pbgb::rest_gradients(e, G);
        T dm = T(0), dl = T(0);
        pbgb::adjoint_tet(d, e, G, tw, td, T(muw), T(law), c, dm, dl);
        for (int r = 0; r < 3; ++r)
            dphi[3 * il + r] = 0.0;
        for (int m = 0; m < 3; ++m)
        {
            int const a = (il + 1 + m) & 3;
            for (int r = 0; r < 3; ++r)
            {
                dphi[3 * a + r] = double(c[m][r]);
                dphi[3 * il + r] -= double(c[m][r]);
            }
        }
        *dlogmu     = double(dm);
        *dloglambda = double(dl);
    };
    if (precision == 64)
        run(0.0);
    else
        run(0.0f);
    return kOk;
}

PBGB_API int pbgb_debug_vertex_block(
    int32_t n,
    const double* xe,
    const double* GPs,
    const int32_t* il,
    const double* wg,
    const double* mu,
    const double* lambda,
    const double* xt,
    const double* xtilde,
    double m,
    double kD,
    double h,
    double h2,
    double detHZero,
    double* x,
    double* g,
    double* H)
{
    if (n < 0 || (n > 0 && (!xe || !GPs || !il || !wg || !mu || !lambda)) || !xt || !xtilde || !x)
        return fail(nullptr, kInvalid, "pbgb_debug_vertex_block: null argument");
    pbgb::VertexBlock<double> b;
    pbgb::zero(b);
    for (int32_t q = 0; q < n; ++q)
    {
        double const* xq = xe + 12 * size_t(q);
        double const* G4 = GPs + 12 * size_t(q);
        if (il[q] < 0 || il[q] > 3)
            return fail(nullptr, kInvalid, "local index out of range");
        // Same own-corner-relative form and per-tet record as the device sweep (in FP64).
        double d[3][3];
        for (int m = 0; m < 3; ++m)
        {
            int const a = (il[q] + 1 + m) & 3;
            for (int r = 0; r < 3; ++r)
                d[m][r] = xq[3 * a + r] - xq[3 * il[q] + r];
        }
        double w[8];
        pbgb::tet_stiffness_words(G4, wg[q], mu[q], lambda[q], w);
        double const bw[6] = {w[0], w[1], w[2], w[3], w[4], w[5]};
        double b0, b1, b2, kappa;
        pbgb::corner_stiffness(bw, w[7], il[q], b0, b1, b2, kappa);
        pbgb::accumulate_incidence(b, d, b0, b1, b2, w[6], kappa);
    }
    pbgb::newton_update(b, xt, xtilde, m, h, h2, kD, detHZero, x, g, H);
    return kOk;
}

} // extern "C"
