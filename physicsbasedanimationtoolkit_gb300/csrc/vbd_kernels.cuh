// Device kernels of the VBD step.  Layout in HBM (all arrays of the whole, possibly batched,
// system; indices global):
//
//   x, xt, xtilde, v, aext, vprev : float4 per vertex (xyz, w unused except xt.w = lumped mass)
//   h0, h1: float4 per vertex, the Chebyshev iterate history (allocated with acceleration only)
//   X     : float4 per vertex, rest positions (the shape-function gradients are recomputed from
//           them, which keeps a tet record at 32 bytes)
//   tets  : one 32-byte TetRecord per tet (below)
//   solve : free vertices, colour-major; inside a colour sorted by decreasing degree
//   incPtr: offsets of each solved vertex's incidences; inc: (tet << 2 | local index), tets
//           ascending
//
// A tet record is read by each of its 4 vertices in 4 different colour passes of an iteration;
// being 32-byte aligned it costs exactly one sector per visit, and the records, incidences and
// position tables of a ~1.5M-tet mesh fit in the 129 MB L2 together.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vbd_math.cuh"

namespace pbgb {

// One tetrahedron.  v.{x,y,z,w}: vertex indices in bits 0-29; bits 30-31 hold the vertex's rank
// (0..3) by colour inside the tet, which tells a vertex solve whether a neighbour was already
// updated in the current iteration (lower rank) or not (higher rank).
//   mat = (wg*mu, wg*lambda, alpha = 1 + mu/lambda, unused)
struct __align__(32) TetRecord
{
    uint4 v;
    float4 mat;
};

uint32_t constexpr kIndexMask = 0x3FFFFFFFu;

struct SweepParams
{
    float4* __restrict__ x;            // positions (with Chebyshev: raw sweep results)
    float4 const* __restrict__ hprev;  // Chebyshev: accelerated iterate k-1 (read)
    float4* __restrict__ hcur;         // Chebyshev: iterate k-2 in, accelerated iterate k out
    float4 const* __restrict__ xt;     // .w = lumped mass
    float4 const* __restrict__ xtilde; // inertial target
    TetRecord const* __restrict__ tets;
    int32_t const* __restrict__ solve;
    int32_t const* __restrict__ incPtr;
    uint32_t const* __restrict__ inc;
    int32_t begin;
    int32_t end;
    float h;
    float h2;
    float kD;
    float detHZero;
    int32_t k;   // iteration index (Chebyshev)
    float omega; // Chebyshev weight of iteration k
    // Vertex-triangle contact (fc == nullptr: none).  Contact triangles' corners are read with
    // the same colour rule as mesh neighbours: colour < `color` from x, otherwise from hprev.
    int32_t const* __restrict__ fc;     // nV x 8 contact triangles, -1 = none
    int4 const* __restrict__ F;         // collision triangles
    float const* __restrict__ XVA;      // nV vertex areas
    float const* __restrict__ FA;       // triangle areas
    int32_t const* __restrict__ vcolor; // nV colour of each vertex (-1 for pinned ones)
    int32_t color;                      // colour of this launch
    // Contact records, rebuilt at each active-set update (launch_contact_records): per vertex and
    // slot, the triangle's corners with bit 31 set when the corner's colour is below the vertex's
    // (read from x, else from hprev) and w = the triangle (-1: none); cpen = its penalty
    // XVA_i muC FA_f / sum of the listed FA.  The listed triangles come first; ccount holds how
    // many a vertex has, so that the vertices without contact read no record.
    int4 const* __restrict__ crec;
    float const* __restrict__ cpen;
    int32_t const* __restrict__ ccount;
    float muC;
    float muF;
    float epsv;
    // Per-incidence stiffness (solve order, TetStiffness resolved for the incidence's own corner):
    // stiff[k] = (b0, b1, b2, kappa_o); incPack[k] = (neighbour slots, sigma as bits): the three
    // other corners' positions in the vertex's neighbour list in bytes 0-2 of .x (corner order
    // (local + 1 + m) & 3; staged sweep only).  Every incidence reads these instead of rest
    // positions.
    float4 const* __restrict__ stiff;
    uint2 const* __restrict__ incPack;
    // Neighbour staging (staged sweep only): for solve-list entry s, its distinct neighbours
    // nbr[nbrPtr[s] .. nbrPtr[s+1]) (vertex index in bits 0-29, bit 31 set when the neighbour has a
    // lower colour, so that the two-buffer sweep reads it from x rather than hprev).
    int32_t const* __restrict__ nbrPtr;
    uint32_t const* __restrict__ nbr;
    // Applied Newton increments (one-buffer sweeps only, nullptr: not written): step[i] = x_new -
    // x_old for every solved vertex, the residual Anderson acceleration mixes (exact to FP32
    // relative precision, unlike the difference of two rounded positions).
    float4* __restrict__ step;
    // Adjoint tape of this iteration (recording sweeps only): for solve-list entry s, the inverse
    // of the vertex's 3x3 Newton matrix (xx xy xz yy | yz zz 0 0) in tape[2s], tape[2s+1]; zero
    // when the Newton step was skipped.
    float4* __restrict__ tape;
};

struct SubstepParams
{
    float4* __restrict__ x;
    float4* __restrict__ xt;
    float4* __restrict__ xtilde;
    float4* __restrict__ v;
    float4 const* __restrict__ aext;
    float4* __restrict__ vprev;
    float4* __restrict__ h0; // Chebyshev history (nullptr without acceleration)
    float4* __restrict__ h1;
    float4 const* __restrict__ result; // buffer holding the final iterate at end of substep
    float const* __restrict__ m;
    int32_t* __restrict__ flags;
    int32_t n;
    float h;
    float h2;
    int32_t strategy;
    int32_t gpuSemantics;
};

struct EnergyParams
{
    float4 const* __restrict__ x;
    float4 const* __restrict__ xtilde;
    float const* __restrict__ m;
    float4 const* __restrict__ X;
    TetRecord const* __restrict__ tets;
    int32_t nV;
    int32_t nT;
    double dt2;
    double* __restrict__ out; // objective: out[0]; gradient: 3 x nV
    // Objective only: kObjectiveMaxBlocks per-block partial sums, added in block order into out[0]
    // (a fixed grid and fixed orders make the value identical from run to run).
    double* __restrict__ partials;
    // sum_e wg_e mu_e^2 / (2 lambda_e): the elastic energy of the rest state, which the objective
    // adds once (times dt^2) so that per-tet terms carry only what varies with x.
    double restEnergy;
};

// Launchers (defined in vbd_kernels.cu).  Each returns the launch status.
// pdl: launch with programmatic stream serialization, so that the kernel's mesh-table prologue
// overlaps the tail of the previous launch on the stream (the kernel waits before reading
// positions).
// stagedBytes > 0: the staged sweep (neighbours in shared memory), stagedBytes from
// staged_sweep_bytes (each variant launches with its own slot size, at most that much dynamic
// shared memory per block); 0: the sweep that gathers every incidence's corners.  Both
// compute the same arithmetic in the same order.
cudaError_t launch_sweep(SweepParams const& p, int lanes, int block, bool chebyshev, bool pdl, cudaStream_t s, size_t stagedBytes = 0);
// The sweep that also writes p.tape (no contact); the same arithmetic as launch_sweep with the same
// chebyshev flag, so a recorded step reproduces an unrecorded one.
cudaError_t launch_sweep_record(SweepParams const& p, int lanes, int block, bool chebyshev, bool pdl, cudaStream_t s, size_t stagedBytes = 0);
// Dynamic shared memory of the staged sweep over solve entries [begin, end) with `lanes` lanes per
// vertex and `block` threads per block: 16 bytes per staged neighbour of the block that stages the
// most (nbrPtr on the host).
size_t staged_sweep_bytes(int32_t const* nbrPtr, int32_t begin, int32_t end, int lanes, int block);
// Largest dynamic shared memory a staged sweep may use (set on the current device by
// prepare_staged_sweeps); larger launches fall back to the gathering sweep.
size_t constexpr kStagedMaxBytes = 200 * 1024;
// Bytes of one staged neighbour: its current position (float4).
size_t constexpr kStagedSlotBytes = sizeof(float4);
cudaError_t prepare_staged_sweeps();
cudaError_t launch_begin_substep(SubstepParams const& p, cudaStream_t s);
cudaError_t launch_end_substep(SubstepParams const& p, cudaStream_t s);
// Blocks of the objective's reduction grid (p.partials holds this many doubles).
int constexpr kObjectiveMaxBlocks = 1024;
// Writes the objective to p.out[0] (no prior clearing needed); deterministic.
cudaError_t launch_objective(EnergyParams const& p, cudaStream_t s);
cudaError_t launch_gradient(EnergyParams const& p, cudaStream_t s);
// origin (nullable, one float4 per vertex): positions are stored relative to it (pack subtracts,
// unpack adds).
cudaError_t launch_pack3(float const* in3, float4* out4, int32_t n, cudaStream_t s, float4 const* origin = nullptr);
// Contact records of all nV vertices from their lists fc (see SweepParams::crec).
cudaError_t launch_contact_records(int32_t nV, int32_t const* fc, int4 const* F, float const* FA, float const* XVA,
                                   int32_t const* vcolor, float muC, int4* crec, float* cpen, int32_t* ccount,
                                   cudaStream_t s);
cudaError_t launch_unpack3(float4 const* in4, float* out3, int32_t n, cudaStream_t s, float4 const* origin = nullptr);

} // namespace pbgb
