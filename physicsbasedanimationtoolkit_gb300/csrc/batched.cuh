// Persistent step of a batch of meshes (no counterpart in the reference, which steps one mesh
// per integrator, gpu/impl/vbd/Integrator.cu:82-103).
//
// One kernel launch advances every mesh of the batch through a whole time step.  The step is cut
// into work items: per mesh and substep, the inertial target / initial guess of a range of its
// vertices (begin), a tile of one colour's solve entries for one iteration (sweep), and the
// velocity update of a range of vertices (end).  A mesh's items form a chain of stages -- begin,
// then (iteration k, colour c) for k, c ascending, then end -- and every item of a stage needs
// every item of the mesh's previous stage finished.  Items sit in one array, ordered by stage
// time (substep, iteration, colour) and then by mesh, and blocks take them in that order from an
// atomic ticket; a block waits (bounded) until the mesh's completion counter reaches the item's
// requirement, runs the item, and adds one to the counter.  So a mesh moves to its next colour as
// soon as its own previous colour is done, whatever the other meshes are doing, and no launch or
// grid-wide barrier separates colours.
//
// Progress: a block holds at most two tickets, the item it runs and the next one it took; the
// lowest unfinished item is always some block's running item (the other ticket a block holds is
// higher than its running one), and its requirements are lower items, all finished.  So the
// waits end, whatever the number of resident blocks.  Every wait is also bounded in time: one
// that gives up raises flags[1] and an abort flag that makes every later wait return at once, and
// the launch ends.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_kernels.cuh"

namespace pbgb {

int constexpr kBatchBegin = 0; // inertial target and initial guess of vertices [begin, end)
int constexpr kBatchSweep = 1; // colour sweep of solve entries [begin, end)
int constexpr kBatchEnd   = 2; // velocity update of vertices [begin, end)

// One work item, two int4: (mesh, kind | iteration << 2, begin, end), (need, 0, 0, 0); need =
// completed items of the mesh required before it starts.
struct BatchItemWords
{
    int4 a;
    int4 b;
};

struct BatchedStepParams
{
    SweepParams sweep;    // tables and step constants; x / hprev / hcur / k / omega per item
    SubstepParams sub;    // begin and end of substep
    float4* H0;           // two-buffer sweep (Chebyshev): iterate buffers, nullptr for one buffer
    float4* H1;
    float const* omega;   // Chebyshev weight of each iteration
    BatchItemWords const* items;
    int32_t nItems;
    int32_t* control;     // [0] ticket, [1] abort; cleared before every launch
    int32_t* done;        // per mesh: completed items; cleared before every launch
    int32_t* flags;       // flags[1] |= 1 when a wait gave up
    long long waitNs;     // time limit of one wait
    int32_t poison;       // item whose requirement is never met (tests of the time limit); -1: none
};

// Time limit of one wait in a normal step (a wait normally lasts well under a millisecond).
long long constexpr kBatchWaitNs = 2000000000LL;

// Launches the persistent step: grid blocks of `block` threads, `lanes` lanes per vertex,
// `smem` bytes of dynamic shared memory (the largest neighbour slab of any sweep tile).
cudaError_t launch_batched_step(BatchedStepParams const& p, int lanes, int block, int grid, size_t smem, bool chebyshev, cudaStream_t s);
// Resident blocks per SM of that launch (0 if it cannot run).
int batched_step_blocks_per_sm(int lanes, int block, size_t smem, bool chebyshev);
// Allows the kernels the staged sweep's shared-memory maximum on the current device.
cudaError_t prepare_batched_step();

} // namespace pbgb
