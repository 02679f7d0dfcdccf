// Trust-region accelerated VBD, linear accelerated path
// (gpu/impl/vbd/TrustRegionIntegrator.cu:48-165).
//
// The reference decides every iteration on the host from objective values it reduces with thrust
// and copies back.  Here the scalars live in device memory (TrustState) and every decision is
// taken by the last block of the reduction that produces its input, so a whole step, decisions
// included, is one stream-ordered sequence that a CUDA graph replays without a host round trip.
// Kernels whose work a decision skips read the decision from TrustState and return at once.
//
// Per VBD iteration k >= 2 (k < 2 are plain sweeps that record f and t):
//   trust_begin      x_{k-1} <- x; block 0 builds the quadratic model m(t) through the last three
//                    (t, f) pairs and shifts them (ConstructModel, UpdateIterates)
//   colour sweeps    x <- VBD iterate
//   trust_step_size  |x - x_{k-1}|^2; last block: radius, t = clamp(t*, 1, R/|dx|), try flag
//   trust_apply      if try: x <- x_{k-1} + t (x - x_{k-1})
//   trust_objective  if try: f(x); last block: accept when (f_{k-1} - f)/(m(0) - m(t)) > eta
//   trust_apply      if rejected after a try: x <- x_{k-1} + (x - x_{k-1}) / t
//   trust_objective  if rejected: f(x) -> f_k
// All scalars are FP64; reductions are deterministic (fixed grid, per-block partials summed in
// block order by the last block).
#pragma once

#include "vbd_kernels.cuh"

#include <cuda_runtime.h>
#include <cstdint>

namespace pbgb {

struct TrustState
{
    double fk, fkm1, fkm2;
    double tk, tkm1, tkm2;
    double R2;
    double aQ[3];
    double t, upper;
    int32_t tryStep, accepted, rollback, needObjective;
    uint32_t ticket; // blocks of the running reduction that have published their partial
    int32_t pad;
};

struct TrustParams
{
    float4* x;
    float4* xkm1;
    EnergyParams energy; // positions, inertial targets, masses, rest positions, tets, dt^2
    TrustState* state;
    double* partials; // kTrustMaxBlocks
    int32_t nV;
    double eta, tau;
    float4* xh; // with contact: the two-buffer sweep's copy of the iterate, updated with x (or null)
    // With contact: the contact energy of the active vertices joins the objective
    // (gpu/impl/vbd/TrustRegionIntegrator.cu:265-360); nActive = null without contact.
    int32_t const* nActive;
    int32_t const* av;  // active collision vertices (indices into cV)
    int32_t const* cV;  // collision vertex -> system vertex
    int32_t const* fc;  // 8 contact triangles per system vertex (-1 = none)
    int4 const* cF;     // triangles
    float const* FA;    // triangle areas
    float const* XVA;   // vertex areas
    float4 const* xt;   // positions at t
    float muC, muF, epsv, h;
    // Decision log of the step, 4 doubles per (substep, iteration) entry: t, the decrease ratio
    // rho (NaN when no stretched step was tried), the squared radius after the iteration, and
    // flags (1: stretched step tried, 2: accepted).  Iterations 0 and 1 log t = 0, flags 0.
    double* log;
};

int constexpr kTrustLogFields = 4;

int constexpr kTrustMaxBlocks = 1024;

enum TrustObjectivePhase : int32_t
{
    kTrustInitial = 0, // f_k <- f(x) before the first iteration
    kTrustPlain   = 1, // iterations 0 and 1: f_k <- f(x), t_k <- k
    kTrustTrial   = 2, // after a stretched step: accept or reject
    kTrustFinal   = 3, // after a rejection: f_k <- f(x)
};

// entry: index of this (substep, iteration) in p.log.
cudaError_t launch_trust_begin(TrustParams const& p, int32_t k, cudaStream_t s);
cudaError_t launch_trust_step_size(TrustParams const& p, int32_t entry, cudaStream_t s);
cudaError_t launch_trust_apply(TrustParams const& p, bool rollback, cudaStream_t s);
cudaError_t launch_trust_objective(TrustParams const& p, TrustObjectivePhase phase, int32_t k, int32_t entry, cudaStream_t s);

} // namespace pbgb
