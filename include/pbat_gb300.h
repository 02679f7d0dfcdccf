/*
 * pbat_gb300.h — C ABI of the GB300-native Vertex Block Descent (VBD) library.
 *
 * One hot path of PhysicsBasedAnimationToolkit (PBAT) is implemented here: the VBD time step of
 * tetrahedral Stable Neo-Hookean meshes, with the reference's Chebyshev, Anderson, Broyden,
 * Nesterov and trust-region accelerations, vertex-triangle contact (and the LBVH it uses), a
 * batched multi-mesh form and a hand-written adjoint.  Every entry point takes plain pointers and sizes,
 * returns an int status (PBGB_OK = 0) and never lets a C++ exception cross the boundary.  Handles
 * are not thread-safe; each owns one CUDA stream.  Array layouts follow the reference's Eigen
 * column-major matrices: a "3 x n" array stores entity j at [3j, 3j+1, 3j+2].
 *
 * Reference interfaces replaced (paths relative to the reference's `source/pbat/`):
 *   pbgb_vbd_data_construct      sim::vbd::Data::Construct            sim/vbd/Data.cpp:179-308
 *   pbgb_vbd_create              gpu::vbd::Integrator(Data const&)    gpu/vbd/Integrator.cu:15-33
 *                                sim::vbd::Integrator(Data)           sim/vbd/Integrator.cpp:20
 *   pbgb_vbd_step                Integrator::Step(dt, iters, substeps) gpu/vbd/Integrator.cu:58-61,
 *                                                                     sim/vbd/Integrator.cpp:22-45
 *   pbgb_vbd_{get,set}_*         Get/SetPositions, Get/SetVelocities,  gpu/vbd/Integrator.h:95-144
 *                                SetExternalAcceleration, Set* knobs
 *   pbgb_vbd_objective/gradient  Integrator::ObjectiveFunction(Grad)  sim/vbd/Integrator.cpp:138-200
 *   pbgb_vbd_traced_step         Integrator::TracedStep               gpu/impl/vbd/Integrator.cu:105-148
 *   pbgb_vbd_trace_next_step     Integrator::TraceNextStep            sim/vbd/Integrator.cpp:47-52
 *   pbgb_vbd_trust_region_log    the trust-region decisions the reference logs through its
 *                                profiler                             gpu/impl/vbd/TrustRegionIntegrator.cu:71-160
 *   pbgb_bvh_*                   gpu::geometry::Bvh (build, overlaps, self-overlaps, nearest
 *                                simplices, visits) gpu/geometry/Bvh.cu, gpu/impl/geometry/Bvh.cu/.cuh
 *   pbgb_simplex_boxes           gpu::geometry::Aabb::Construct(P, S) gpu/geometry/Aabb.cu
 *   pbgb_ccd_*                   VertexTriangleMixedCcdDcd            gpu/impl/contact/VertexTriangleMixedCcdDcd.cu
 * Beyond the reference: pbgb_vbd_create_batched (many meshes, one persistent launch per step),
 * pbgb_vbd_step_record / pbgb_vbd_step_adjoint(_state) (reverse-mode derivatives), pbgb_vbd_save_state /
 * pbgb_vbd_load_state (checkpoints), *_device variants (device pointers), pbgb_vbd_autotune.
 */
#ifndef PBAT_GB300_H
#define PBAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define PBGB_API __declspec(dllexport)
#else
#define PBGB_API __attribute__((visibility("default")))
#endif

/* Status codes. */
#define PBGB_OK 0
#define PBGB_ERR_INVALID_ARGUMENT 1 /* null pointer, bad size, bad enum, rho outside (0,1) ... */
#define PBGB_ERR_CUDA 2             /* a CUDA runtime call failed (message in pbgb_last_error) */
#define PBGB_ERR_NONFINITE 3        /* the device detected a NaN/Inf position or velocity */
#define PBGB_ERR_DEGENERATE 4       /* a tetrahedron with non-positive volume */
#define PBGB_ERR_PALETTE 5          /* greedy colouring needed more than 128 colours */
#define PBGB_ERR_NO_DEVICE 6        /* no CUDA device */
#define PBGB_ERR_TIMEOUT 7          /* a bounded device wait gave up */
#define PBGB_ERR_INTERNAL 8

/* Enumerations (values match the reference's enums). */
/* sim/vbd/Enums.h:9-15 */
#define PBGB_INIT_POSITION 0
#define PBGB_INIT_INERTIA 1
#define PBGB_INIT_KINETIC_ENERGY_MINIMUM 2
#define PBGB_INIT_ADAPTIVE_VBD 3
#define PBGB_INIT_ADAPTIVE_PBAT 4
/* sim/vbd/Enums.h:21-28 (all six are implemented; which integrator runs a strategy follows the
   reference's dispatch: the GPU integrator runs plain VBD for Nesterov and Broyden) */
#define PBGB_ACCEL_NONE 0
#define PBGB_ACCEL_CHEBYSHEV 1
#define PBGB_ACCEL_ANDERSON 2 /* single mesh (contact allowed); window_size columns */
#define PBGB_ACCEL_NESTEROV 3 /* nesterov_lipschitz, nesterov_start; single mesh without contact (a
                                 CPU-integrator strategy) */
#define PBGB_ACCEL_BROYDEN 4 /* single mesh without contact (a CPU-integrator strategy); window_size columns */
#define PBGB_ACCEL_TRUST_REGION 5 /* tr_eta, tr_tau, tr_curved; single mesh (contact allowed) */
/* graph/Enums.h:20-33 */
#define PBGB_COLOR_ORDER_NATURAL 0
#define PBGB_COLOR_ORDER_SMALLEST_DEGREE 1
#define PBGB_COLOR_ORDER_LARGEST_DEGREE 2
#define PBGB_COLOR_SELECT_LEAST_USED 0
#define PBGB_COLOR_SELECT_FIRST_AVAILABLE 1
/* Integrator flavour: which reference integrator's step semantics to reproduce. */
#define PBGB_SEMANTICS_CPU 0 /* sim::vbd::Integrator: AdaptiveVbd sees vtm1 = v (Integrator.cpp:31-32) */
#define PBGB_SEMANTICS_GPU 1 /* gpu::vbd::Integrator: vtm1 = velocity of the previous step */
/* Chebyshev weight recurrence. */
#define PBGB_CHEBYSHEV_REFERENCE 0 /* omega_k = 4/4 - rho^2 omega_{k-1}, as written in Kernels.h:96-102 */
#define PBGB_CHEBYSHEV_TEXTBOOK 1  /* omega_k = 4/(4 - rho^2 omega_{k-1}) */

/* Maximum number of colours of the greedy colouring (graph/Color.h:45, palette capacity 128). */
#define PBGB_MAX_COLORS 128

/*
 * Data::Construct precompute on the host (FP64), sim/vbd/Data.cpp:179-243.
 *   X      : 3 x nV rest positions          T     : 4 x nT tetrahedra (int32)
 *   rhoe   : nT mass densities              dbc   : nDbc Dirichlet vertex indices
 *   ordering/selection: PBGB_COLOR_ORDER_* / PBGB_COLOR_SELECT_*
 * Outputs, caller-allocated:
 *   m[nV] lumped masses; GP[12 nT] shape-function gradients, per tet a row-major 4 x 3 block
 *   (row a = grad N_a); wg[nT] quadrature weights (volumes); GVGp[nV+1], GVGe[4nT],
 *   GVGilocal[4nT] vertex->tet adjacency; colors[nV]; Pptr[PBGB_MAX_COLORS+1] and Padj[nV] the
 *   colour partitions without Dirichlet vertices; *nPartitions, *nPadj their lengths.
 */
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
    int32_t* nPadj);

/*
 * A constructed VBD problem (the content of sim::vbd::Data after Construct).  Pointers are only
 * read during pbgb_vbd_create.
 */
typedef struct pbgb_vbd_desc
{
    int32_t n_vertices;
    int32_t n_tets;
    const double* x;      /* 3 x nV initial positions (required) */
    const int32_t* T;     /* 4 x nT tetrahedra (required) */
    const double* v;      /* 3 x nV velocities (NULL: zero) */
    const double* aext;   /* 3 x nV external accelerations (NULL: (0,0,-9.81)) */
    const double* m;      /* nV lumped masses (required) */
    const double* GP;     /* 12 nT shape-function gradients, row-major 4x3 per tet (optional: the
                             device recomputes them from the rest positions X) */
    const double* wg;     /* nT quadrature weights (required) */
    const double* mu;     /* nT first Lame coefficients (required) */
    const double* lambda; /* nT second Lame coefficients (required) */
    int32_t n_partitions; /* number of colours */
    const int32_t* Pptr;  /* n_partitions + 1 */
    const int32_t* Padj;  /* Pptr[n_partitions] free vertices, colour-major */
    int32_t init_strategy;     /* PBGB_INIT_* (reference default AdaptivePbat) */
    double kD;                 /* Rayleigh damping (default 0) */
    double detHZero;           /* near-singular Hessian threshold (default 1e-7) */
    int32_t acceleration;      /* PBGB_ACCEL_* */
    double rho;                /* Chebyshev spectral radius estimate, 0 < rho < 1 */
    int32_t chebyshev_formula; /* PBGB_CHEBYSHEV_* */
    int32_t semantics;         /* PBGB_SEMANTICS_* */
    const double* X;           /* 3 x nV rest positions (NULL: x) */
    /* Vertex-triangle contact (gpu/impl/vbd/Kernels.cuh:80-114,203-223; active set
     * gpu/impl/contact/VertexTriangleMixedCcdDcd.cu).  n_collision_triangles = 0 disables it; only
     * a single (non-batched) mesh may carry contact.  Bodies separate self-contact. */
    int32_t n_collision_vertices;  /* |V| */
    const int32_t* V;              /* collision vertices */
    int32_t n_collision_triangles; /* |F| */
    const int32_t* F;              /* 3 x |F| collision triangles */
    const int32_t* B;              /* nV body of each vertex (NULL: one body) */
    const double* XVA;             /* nV vertex areas (Data::XVA) */
    const double* FA;              /* |F| triangle areas (Data::FA) */
    double muC;                    /* contact penalty (default 1e6) */
    double muF;                    /* friction coefficient (default 0.3) */
    double epsv;                   /* IPC smooth friction velocity threshold (default 1e-3) */
    int32_t active_set_update_frequency; /* update the contact list every k substeps (default 1) */
    int32_t window_size; /* Anderson / Broyden window m, 1..16 (Data::mWindowSize, default 5) */
    double nesterov_lipschitz; /* L > 0 (Data::mNesterovLipschitzConstant, default 1) */
    int32_t nesterov_start;    /* accelerate iterations k > start >= 0 (default 3) */
    /* Trust-region acceleration (gpu/impl/vbd/TrustRegionIntegrator.cu; Data::eta, tau, bCurved). */
    double tr_eta;     /* energy-reduction ratio threshold, >= 0 (default 0.2) */
    double tr_tau;     /* radius growth factor, > 1 (default 2) */
    int32_t tr_curved; /* 1: curved path (its steps are plain VBD iterations), 0: linear path */
} pbgb_vbd_desc;

typedef struct pbgb_vbd pbgb_vbd; /* opaque integrator handle */

/* Upload a problem and build the device layout; *out receives the handle. */
PBGB_API int pbgb_vbd_create(const pbgb_vbd_desc* desc, pbgb_vbd** out);
/* Several independent meshes advanced together by one launch sequence per step (batched form).
 * Vertex/tet indices of each desc are local to its mesh; get/set address the concatenation. */
PBGB_API int pbgb_vbd_create_batched(const pbgb_vbd_desc* descs, int32_t n_meshes, pbgb_vbd** out);
PBGB_API int pbgb_vbd_destroy(pbgb_vbd* h);

/* Integrator::Step(dt, iterations, substeps).  Asynchronous on the handle's stream. */
PBGB_API int pbgb_vbd_step(pbgb_vbd* h, float dt, int32_t iterations, int32_t substeps);
/* Integrator::TracedStep (gpu/vbd/Integrator.h:79-93, gpu/impl/vbd/Integrator.cu:105-148): one
 * step of plain VBD iterations (whatever the acceleration, as the reference's TracedSolve) written
 * to `dir` as Matrix Market files: on t == 0 T.mtx (nT x 4), M.mtx, wg.mtx, GP.mtx (4 x 3 nT),
 * lame.mtx (nT x 2); per substep xtilde.t.{t}.s.{s}.mtx (nV x 3) and x.t.{t}.s.{s}.k.{k}.mtx for
 * k = 0 .. iterations.  Synchronous. */
PBGB_API int pbgb_vbd_traced_step(pbgb_vbd* h, float dt, int32_t iterations, int32_t substeps, int32_t t, const char* dir);
/* Integrator::TraceNextStep of the CPU integrator (sim/vbd/Integrator.cpp:47-52,202-235): the next
 * pbgb_vbd_step writes, per substep, {path}/{t}.{s}.f.mtx (objective at the iterates k = 0 ..
 * iterations), {t}.{s}.grad.mtx and {t}.{s}.x.mtx (3 nV x iterations+1, FP64 gradient and
 * positions), with the configured acceleration.  That step runs outside the step graph. */
PBGB_API int pbgb_vbd_trace_next_step(pbgb_vbd* h, const char* path, int32_t t);
/* Block until the handle's stream is idle; reports device-side non-finite detection. */
PBGB_API int pbgb_vbd_synchronize(pbgb_vbd* h);

/* Host copies (3 x nV, float32 like the reference's GpuMatrixX).  get_* synchronize. */
PBGB_API int pbgb_vbd_get_positions(pbgb_vbd* h, float* x);
PBGB_API int pbgb_vbd_set_positions(pbgb_vbd* h, const float* x);
PBGB_API int pbgb_vbd_get_velocities(pbgb_vbd* h, float* v);
PBGB_API int pbgb_vbd_set_velocities(pbgb_vbd* h, const float* v);
PBGB_API int pbgb_vbd_set_external_acceleration(pbgb_vbd* h, const float* aext);
/* Checkpoint / resume: the whole state a step reads (positions, velocities, the previous step's
 * velocities, external accelerations, and with contact the persistent active set, search radii and
 * contact lists) as one host blob with a header.  A handle built from the same descriptors that
 * loads the blob continues bit for bit.  pbgb_vbd_state_size gives the blob's size; save and load
 * synchronize; loading a blob of another system size is PBGB_ERR_INVALID_ARGUMENT. */
PBGB_API int pbgb_vbd_state_size(pbgb_vbd* h, size_t* bytes);
PBGB_API int pbgb_vbd_save_state(pbgb_vbd* h, void* blob, size_t bytes);
PBGB_API int pbgb_vbd_load_state(pbgb_vbd* h, const void* blob, size_t bytes);
/* Device-pointer variants (3 x nV float32 on the handle's device), stream-ordered. */
PBGB_API int pbgb_vbd_get_positions_device(pbgb_vbd* h, float* x_dev);
PBGB_API int pbgb_vbd_set_positions_device(pbgb_vbd* h, const float* x_dev);
PBGB_API int pbgb_vbd_get_velocities_device(pbgb_vbd* h, float* v_dev);
PBGB_API int pbgb_vbd_set_velocities_device(pbgb_vbd* h, const float* v_dev);
/* Per-tet Lame coefficients (host, nT each, system order), as Data::WithMaterial sets them
 * (sim/vbd/Data.cpp:60-75); masses and quadrature weights are kept.  Synchronizes. */
PBGB_API int pbgb_vbd_set_material(pbgb_vbd* h, const double* mu, const double* lambda);

/* Knobs (gpu/vbd/Integrator.h:110-134). */
PBGB_API int pbgb_vbd_set_detH_zero(pbgb_vbd* h, float zero);
PBGB_API int pbgb_vbd_set_damping(pbgb_vbd* h, float kD);
PBGB_API int pbgb_vbd_set_strategy(pbgb_vbd* h, int32_t strategy);
/* Threads per block of the vertex sweep (the reference clamps to [32, 256]). */
PBGB_API int pbgb_vbd_set_block_size(pbgb_vbd* h, int32_t block_size);
/* Lanes cooperating on one vertex: 1, 2, 4, 8, 16 or 32 (0 = autotuned). */
PBGB_API int pbgb_vbd_set_lanes_per_vertex(pbgb_vbd* h, int32_t lanes);
/* Autotuner: times one step of (dt, iterations, substeps) for every lanes-per-vertex in
 * {1,2,4,8,16,32} x block size in {64,128,256}, keeps the fastest for this handle and caches it per
 * size bucket (vertex and tet counts rounded up to powers of two, colours, iterations).  The
 * handle's positions and velocities are restored after each trial.  Outputs may be NULL. */
PBGB_API int pbgb_vbd_autotune(
    pbgb_vbd* h,
    float dt,
    int32_t iterations,
    int32_t substeps,
    int32_t* lanes,
    int32_t* block_size,
    float* ms_per_step);
/* Programmatic dependent launch of the colour sweeps (default on): each colour's kernel loads its
 * mesh tables while the previous colour drains, then waits before reading positions. */
PBGB_API int pbgb_vbd_set_programmatic_launch(pbgb_vbd* h, int32_t enable);
/* Staged colour sweep (default on): each vertex's distinct neighbours are loaded once into shared
 * memory instead of three corners per incident tet; same arithmetic, same results.  Unavailable
 * (the gathering sweep runs) when a vertex has more than 256 neighbours; a colour whose blocks
 * would need more than 200 KB of shared memory also runs the gathering sweep. */
PBGB_API int pbgb_vbd_set_staged_sweep(pbgb_vbd* h, int32_t enable);
PBGB_API int pbgb_vbd_staged_sweep(pbgb_vbd* h, int32_t* available, int32_t* enabled);
PBGB_API int pbgb_vbd_set_scene_bounding_box(pbgb_vbd* h, const float* min3, const float* max3);

/* Sizes and launch bookkeeping. */
PBGB_API int pbgb_vbd_sizes(pbgb_vbd* h, int32_t* n_vertices, int32_t* n_tets, int32_t* n_free, int32_t* n_colors);
/* Number of kernels one pbgb_vbd_step(iterations, substeps) launches. */
PBGB_API int pbgb_vbd_launches_per_step(pbgb_vbd* h, int32_t iterations, int32_t substeps, int64_t* launches);
/* Kernel nodes of the CUDA graph pbgb_vbd_step last captured: the launches a step replays, counted
 * from the graph itself (-1 before the first captured step; a traced step is not captured and
 * leaves the count as it was). */
PBGB_API int pbgb_vbd_step_graph_kernels(pbgb_vbd* h, int64_t* kernels);
/* Sweep timing (off by default): when enabled, each captured step records a CUDA event pair around
 * the colour sweeps of every iteration.  pbgb_vbd_sweep_timing returns, for the last step, the
 * summed sweep intervals in milliseconds and the number of sweep kernel launches they cover. */
PBGB_API int pbgb_vbd_set_sweep_timing(pbgb_vbd* h, int32_t enable);
PBGB_API int pbgb_vbd_sweep_timing(pbgb_vbd* h, double* milliseconds, int64_t* sweep_launches);
/* Persistent batched step (handles of several meshes; no counterpart in the reference, which steps
 * one mesh per integrator, gpu/impl/vbd/Integrator.cu:82-103).  On by default: one kernel launch
 * per step advances every mesh, each mesh moving to its next colour as soon as its own previous
 * colour is done (per-mesh completion counters, bounded waits: a wait that gives up makes the next
 * synchronizing call return PBGB_ERR_TIMEOUT).  Used for plain VBD and Chebyshev without contact
 * when every colour's neighbours fit in shared memory; otherwise, or when disabled, a batch steps
 * with one launch per colour.  pbgb_vbd_persistent reports whether the next step uses it.
 * pbgb_vbd_set_batch_tile: sweep work items of subtiles x (block / lanes) vertices (default 1). */
PBGB_API int pbgb_vbd_set_persistent(pbgb_vbd* h, int32_t enable);
PBGB_API int pbgb_vbd_persistent(pbgb_vbd* h, int32_t* active);
PBGB_API int pbgb_vbd_set_batch_tile(pbgb_vbd* h, int32_t subtiles);
/* The handle's CUDA stream (cudaStream_t) so callers can order their own work after a step. */
PBGB_API int pbgb_vbd_stream(pbgb_vbd* h, void** stream);

/* Contact lists after the last step: fc[8 nV] contact triangles per vertex (-1 = none) and
 * active[|V|] (1 if the collision vertex is in the active set).  Either may be NULL. */
PBGB_API int pbgb_vbd_get_contacts(pbgb_vbd* h, int32_t* fc, uint8_t* active);
/* The LBVH the last step built over the swept collision-triangle boxes (the active-set query of
 * VertexTriangleMixedCcdDcd, gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:51-136, on the
 * hierarchy of gpu/impl/geometry/Bvh.cu:130-229): codes[nF] sorted Morton codes, inds[nF] the
 * stable sort order, child[2(nF-1)], parent[2nF-1], rightmost[2(nF-1)] in the reference's node
 * numbering; xpred[3 x nV] the full-step prediction the boxes were swept to (from the positions
 * at the step's start) and scene_box[6] (min, max) the Morton normalisation box.  Any output may
 * be NULL.  PBGB_ERR_INVALID_ARGUMENT without contact. */
PBGB_API int pbgb_vbd_get_contact_bvh(
    pbgb_vbd* h,
    uint32_t* codes,
    int32_t* inds,
    int32_t* child,
    int32_t* parent,
    int32_t* rightmost,
    float* xpred,
    float* scene_box);

/* Backward-Euler objective f(x) = 1/2 |x - xtilde|_M^2 + dt^2 sum wg Psi and its gradient at
 * the current positions against the last step's inertial target; FP64 device reductions. */
PBGB_API int pbgb_vbd_objective(pbgb_vbd* h, double dt, double* f);
PBGB_API int pbgb_vbd_gradient(pbgb_vbd* h, double dt, double* grad /* 3 x nV */);

/* Trust-region decisions of the last step (PBGB_ACCEL_TRUST_REGION, linear path): 4 doubles per
 * (substep, iteration) entry, substep-major -- the step length t, the actual/predicted decrease
 * ratio rho (NaN when no stretched step was tried), the squared radius after the iteration and
 * flags (1: tried, 2: accepted); iterations 0 and 1 are plain.  These are the quantities the
 * reference's integrator logs through its profiler (gpu/impl/vbd/TrustRegionIntegrator.cu:71-160).
 * *count receives the number of entries; at most `capacity` are written to out (may be NULL). */
PBGB_API int pbgb_vbd_trust_region_log(pbgb_vbd* h, double* out, int32_t capacity, int32_t* count);

/*
 * pbgb_vbd_gradient without any device allocation.  This entry point has no counterpart in the
 * reference; it exists for callers that must not call cudaMalloc once their set-up is done, such
 * as applications whose device memory is owned and budgeted by another runtime or engine, or
 * frame loops that forbid allocation after start-up.  pbgb_vbd_gradient allocates its FP64
 * accumulation buffer on its first call; this variant accumulates in a fixed device array built
 * into the library instead (PBGB_NOALLOC_MAX_VERTICES x 3 doubles, 6 MiB per device).
 *   - The array is reserved on a device during set-up: pbgb_vbd_create (and _create_batched) looks
 *     up its device address there (cudaGetSymbolAddress, which loads the library's module on that
 *     device), and the device keeps the 6 MiB until the process exits.  This entry point's own
 *     calls allocate nothing and load nothing.
 *   - Meshes (or batches) with more than PBGB_NOALLOC_MAX_VERTICES vertices are rejected with
 *     PBGB_ERR_INVALID_ARGUMENT.
 *   - All calls share the one array: the used part is cleared at the start of every call, and
 *     calls whose work overlaps on the GPU (different handles or streams at the same time) race.
 *   - The address is kept by the handle: a device reset (cudaDeviceReset) invalidates the handle
 *     together with its other device resources; create a new handle after one.
 *   - Output and blocking behaviour are those of pbgb_vbd_gradient: grad (3 x nV, host) is
 *     written and the call returns once the handle's stream is idle.
 */
#define PBGB_NOALLOC_MAX_VERTICES 262144
PBGB_API int pbgb_vbd_gradient_noalloc(pbgb_vbd* h, double dt, double* grad /* 3 x nV */);

/*
 * Adjoint of the step (no counterpart in the reference, which has no differentiation).  The
 * adjoint is the exact derivative of the computed iterations: each colour sweep is reversed by the
 * same coloured block sweep on the transposed system (colours in reverse order), with the
 * curvature terms of the Stable Neo-Hookean energy that make it exact for the nonlinear update.
 * When the forward iterations converge it becomes the adjoint of the converged step,
 * (M/h^2 + d2E/dx2) lambda = dL/dx.
 *
 * Supported forward settings: plain VBD or Chebyshev acceleration (either weight recurrence), any
 * Rayleigh damping kD, every initial guess (Position, Inertia, KineticEnergyMinimum, AdaptiveVbd,
 * AdaptivePbat: the adaptive guesses' acceleration factor is differentiated on the branch the
 * forward took), CPU or GPU step semantics; no contact and no Anderson, Nesterov, Broyden or
 * trust-region acceleration (PBGB_ERR_INVALID_ARGUMENT).  AdaptivePbat's factor
 * |v.a| / (|v| |a|^2) has no derivative at v = 0 (it jumps), where its derivative is taken as zero.
 *
 *   pbgb_vbd_adjoint_reserve: device tape for `slots` recorded substeps of `iterations` iterations:
 *     per slot (iterations + 1) x nV iterates, the start positions, velocities and previous
 *     velocities, iterations x n_free inverse 3x3 Newton matrices, and with Chebyshev iterations x
 *     nV raw sweep results (16 (iterations + 4) nV + 32 iterations n_free bytes, plus 16 iterations
 *     nV with Chebyshev).
 *   pbgb_vbd_step_record: one pbgb_vbd_step(dt, iterations, substeps) (the same positions) that
 *     records substep s into slot `slot` + s.  Launched directly, not from the step's graph.
 *   pbgb_vbd_step_adjoint_state: reverses the substeps in slots slot + substeps - 1 down to slot.
 *     xbar_dev, vbar_dev, vprevbar_dev (device, 3 x nV): on entry the adjoints dL/dx, dL/dv and
 *     dL/dvprev of the state after the recorded step (vprev: the previous velocity the GPU
 *     semantics keep for AdaptiveVbd), on return those of the state before it.  dlogmu_dev,
 *     dloglambda_dev (device, nT, FP64): dL/dlog(mu), dL/dlog(lambda) of every tet, added to what
 *     they hold (with a fixed Poisson ratio, dL/dlog(E) is their sum).  Each is a sum over every
 *     iteration of terms that largely cancel, so it is accumulated in FP64; the terms are FP32.
 *   pbgb_vbd_step_adjoint: the same with the previous velocity's adjoint taken as zero and not
 *     returned; rejected for AdaptiveVbd with the GPU semantics, whose guess reads it.
 *   pbgb_vbd_{get,set}_previous_velocities_device: the previous velocities (3 x nV, device), for
 *     checkpoints of that state.
 * All are asynchronous on the handle's stream; the tape is overwritten by the next record into
 * the same slot.
 */
PBGB_API int pbgb_vbd_adjoint_reserve(pbgb_vbd* h, int32_t slots, int32_t iterations);
PBGB_API int pbgb_vbd_step_record(pbgb_vbd* h, float dt, int32_t iterations, int32_t substeps, int32_t slot);
PBGB_API int pbgb_vbd_step_adjoint(
    pbgb_vbd* h,
    int32_t slot,
    int32_t substeps,
    float* xbar_dev,
    float* vbar_dev,
    double* dlogmu_dev,
    double* dloglambda_dev);
PBGB_API int pbgb_vbd_step_adjoint_state(
    pbgb_vbd* h,
    int32_t slot,
    int32_t substeps,
    float* xbar_dev,
    float* vbar_dev,
    float* vprevbar_dev,
    double* dlogmu_dev,
    double* dloglambda_dev);
PBGB_API int pbgb_vbd_get_previous_velocities_device(pbgb_vbd* h, float* vprev_dev);
PBGB_API int pbgb_vbd_set_previous_velocities_device(pbgb_vbd* h, const float* vprev_dev);

/*
 * Linear BVH over axis-aligned boxes (reference: gpu::geometry::Bvh, gpu/geometry/Bvh.cu, and its
 * implementation gpu/impl/geometry/Bvh.cu:24-229, Bvh.cuh:205-588, Morton.cu:23-44).
 * Boxes are host arrays, 3 x n (box i at [3i, 3i+2]).  Node numbering as in the reference:
 * internal nodes 0..n-2 (root 0), leaves n-1..2n-2 in Morton order.
 */
typedef struct pbgb_bvh pbgb_bvh;
PBGB_API int pbgb_bvh_create(int32_t capacity, pbgb_bvh** out);
PBGB_API int pbgb_bvh_destroy(pbgb_bvh* b);
/* Morton codes of box centres normalised by the scene box [wmin, wmax] (30 bits), stable radix
 * sort of (code, box index), Karras hierarchy, bottom-up internal boxes.  Bvh::Build. */
PBGB_API int pbgb_bvh_build(pbgb_bvh* b, int32_t n, const float* lower, const float* upper, const float* wmin3, const float* wmax3);
/* New boxes for the same n boxes, topology kept (Bvh::ConstructBoxes after a box update). */
PBGB_API int pbgb_bvh_refit(pbgb_bvh* b, const float* lower, const float* upper);
/* Bvh::Build from device boxes (the reference builds from device Aabb buffers,
 * gpu/impl/geometry/Bvh.cu:116-137): lower4_dev, upper4_dev are n x 4 floats (x, y, z, unused),
 * 16-byte aligned, on the BVH's device; read during the call only.  Asynchronous on the BVH's
 * stream (pbgb_bvh_stream); errors of the device-side checks surface at the next host-buffer
 * call. */
PBGB_API int pbgb_bvh_build_device(pbgb_bvh* b, int32_t n, const float* lower4_dev, const float* upper4_dev, const float* wmin3, const float* wmax3);
PBGB_API int pbgb_bvh_stream(pbgb_bvh* b, void** stream);
/* Read-back: sorted codes[n], inds[n] (original box of each sorted leaf), child[2(n-1)]
 * (child[2i], child[2i+1]), parent[2n-1] (-1 at the root), rightmost[2(n-1)], internal boxes
 * 3 x (n-1).  Any output may be NULL. */
PBGB_API int pbgb_bvh_topology(
    pbgb_bvh* b,
    uint32_t* codes,
    int32_t* inds,
    int32_t* child,
    int32_t* parent,
    int32_t* rightmost,
    float* internal_lower,
    float* internal_upper);
/* All (query, box) pairs whose closed boxes overlap (Bvh::DetectOverlaps(leafAabbs, queryAabbs)):
 * pairs[2k] = query, pairs[2k+1] = box for k < min(*count, capacity); *count = pairs found. */
PBGB_API int pbgb_bvh_overlaps(
    pbgb_bvh* b,
    int32_t nq,
    const float* qlower,
    const float* qupper,
    int32_t* pairs,
    int64_t capacity,
    int64_t* count);
/* Self-overlaps of the built boxes (gpu/geometry/Bvh.cu:68-121, Bvh::DetectOverlaps with and
 * without a set; traversal gpu/impl/geometry/Bvh.cuh:206-281): each unordered pair once, as
 * (box of the leaf earlier in Morton order, other box), in no particular order.  set (nullable)
 * holds one int per box; pairs within one set are dropped.  pairs: 2 * capacity ints; count = all
 * pairs found (call again with a larger capacity when count > capacity). */
PBGB_API int pbgb_bvh_self_overlaps(pbgb_bvh* b, const int32_t* set, int32_t* pairs, int64_t capacity, int64_t* count);
/* Nearest simplex to each of nq points X (3 floats each) among the nS = built boxes' simplices
 * S (k = 3: triangles, gpu/geometry/Bvh.cu:123-190 PointTriangleNearestNeighbors; k = 4:
 * tetrahedra, :192-260 PointTetrahedronNearestNeighbors) over nP points P: nn[q] = simplex index,
 * among exact ties the one the reference's callback writes last. */
PBGB_API int pbgb_bvh_nearest_simplices(pbgb_bvh* b, int32_t nq, const float* X, int32_t nP, const float* P, int32_t nS,
                                        const int32_t* S, int32_t k, int32_t* nn);
/* Visit counters of the last box pass (n - 1 ints; gpu/geometry/Bvh.cu Visits, each 2 after a build). */
PBGB_API int pbgb_bvh_visits(pbgb_bvh* b, int32_t* visits);
/* Boxes of nS simplices of k (1..4) vertices over nP points (gpu/geometry/Aabb.cu:56-80,
 * Aabb::Construct(P, S)): lower / upper 3 floats per simplex. */
PBGB_API int pbgb_simplex_boxes(int32_t nP, const float* P, int32_t nS, const int32_t* S, int32_t k, float* lower, float* upper);
PBGB_API const char* pbgb_bvh_last_error(pbgb_bvh* b);

/*
 * Vertex-triangle contact detector (reference: gpu::impl::contact::VertexTriangleMixedCcdDcd,
 * gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:17-223).  V: collision vertices, F: 3 x |F|
 * triangles, B: nV bodies (NULL: one body; same-body pairs never collide).  Positions are host
 * arrays 3 x nV.
 */
typedef struct pbgb_ccd pbgb_ccd;
PBGB_API int pbgb_ccd_create(int32_t nV, int32_t nSurfV, const int32_t* V, int32_t nF, const int32_t* F, const int32_t* B, pbgb_ccd** out);
PBGB_API int pbgb_ccd_destroy(pbgb_ccd* c);
/* InitializeActiveSet(xt, x, wmin, wmax): swept vertices vs swept triangles. */
PBGB_API int pbgb_ccd_initialize(pbgb_ccd* c, const float* xt, const float* x, const float* wmin3, const float* wmax3);
/* UpdateActiveSet(x): nearest triangles (<= 8, ties within FLT_EPSILON) of active vertices. */
PBGB_API int pbgb_ccd_update(pbgb_ccd* c, const float* x);
/* FinalizeActiveSet(x): keep the vertices that lie behind their nearest triangle's plane. */
PBGB_API int pbgb_ccd_finalize(pbgb_ccd* c, const float* x);
/* active[|V|], nn[8 |V|] (-1 = none), dupper[|V|] (squared search radius), *n_active. */
PBGB_API int pbgb_ccd_get(pbgb_ccd* c, uint8_t* active, int32_t* nn, float* dupper, int32_t* n_active);
PBGB_API const char* pbgb_ccd_last_error(pbgb_ccd* c);

/* Message of the last failing call on h (or of the last failing handle-less call if h is NULL). */
PBGB_API const char* pbgb_last_error(pbgb_vbd* h);

/* Host self-check of the per-tet adjoint term of the device's adjoint sweep (adjoint_tet): for one
 * tet with solved corner o, xe (4 x 3 current positions, row a = corner a), Xe (4 x 3 rest
 * positions), il = o's local index, w and delta (3 each), muw = wg mu, law = wg lambda, writes
 * dphi (4 x 3, row a = d(phi_e)/d(x_a), o's row included) and d(phi_e)/dlog(mu),
 * d(phi_e)/dlog(lambda).  precision 64 evaluates in double, 32 in float like the device. */
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
    double* dloglambda);

/* Test hook of the persistent batched step's bounded waits: the time limit of one wait (1 us ..
 * 2 s; default 2 s) and one work item whose requirement is never met (-1: none), for the steps that
 * follow.  With a poisoned item the step's wait gives up after wait_ns, the step ends with invalid
 * positions and the next synchronizing call returns PBGB_ERR_TIMEOUT; the context stays usable. */
PBGB_API int pbgb_debug_batched_wait(pbgb_vbd* h, int64_t wait_ns, int32_t poison_item);

/* Host self-check of the closed-form vertex block (FP64): accumulates n incident tets and
 * applies damping, inertia and the Newton step exactly like the device sweep.  Arguments as the
 * oracle's per-vertex solve: xe n x 12 (3x4 column-major per tet), GPs n x 12 (row-major 4x3). */
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
    double* H);

/* Host self-check of one vertex-triangle contact term (FP32), the arithmetic of the device sweep
 * (sim/vbd/Kernels.h:215-302).  xtf, xf: 3 x 3 corners (corner-major); adds to g[3] and to the
 * symmetric H[9] (column-major); *energy (may be NULL) receives the contact energy. */
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
    float* energy);

#ifdef __cplusplus
}
#endif

#endif /* PBAT_GB300_H */
