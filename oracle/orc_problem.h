// Problem description shared by the FP64 oracle (vbd_oracle.cpp) and the reference harness
// (ref_harness.cpp).  TEST INFRASTRUCTURE ONLY.  Mirrored by ctypes in tests/oracle_lib.py.
#pragma once
#include <cstdint>

extern "C" {
struct orc_problem
{
    int32_t nV;
    int32_t nT;
    double const* X;  // nV x 3 rest positions
    int32_t const* T; // nT x 4
    double const* m;  // nV lumped masses
    double const* GP; // nT x 4 x 3 shape function gradients (row a = grad N_a)
    double const* wg; // nT quadrature weights (tet volumes)
    double const* mu; // nT first Lame coefficients
    double const* lambda;
    int32_t const* GVGp; // nV+1
    int32_t const* GVGe; // Sum deg
    int32_t const* GVGilocal;
    int32_t nPartitions;
    int32_t const* Pptr; // nPartitions+1
    int32_t const* Padj; // free vertices, colour-major
    double const* aext;  // nV x 3
    int32_t strategy;    // EInitializationStrategy (sim/vbd/Enums.h:9-15)
    double kD;
    double detHZero;
    int32_t acceleration;      // 0 none, 1 Chebyshev, 2 Anderson, 3 Nesterov, 5 trust region
    double rho;                // Chebyshev spectral radius estimate
    int32_t chebyshev_formula; // 0: reference weights (sim/vbd/Kernels.h:96-102), 1: textbook
    int32_t semantics;         // 0: CPU integrator (vtm1 = v), 1: GPU integrator (vtm1 = v(t-1))
    int32_t nthreads;          // <= 0: OpenMP default
    int32_t window;            // Anderson window (acceleration 2)
    double nesterov_L;         // Nesterov Lipschitz constant (acceleration 3)
    int32_t nesterov_start;    // Nesterov: accelerate iterations k > start
    double tr_eta;             // trust region (acceleration 5): energy-reduction ratio threshold
    double tr_tau;             // trust region: radius growth factor
    int32_t tr_curved;         // trust region: curved path (1) or linear path (0)
    double const* tr_forced;   // trust region: NULL, or 4 doubles per (step, substep, iteration) --
                               // t, rho, R^2, flags (1 tried, 2 accepted) -- whose t and flags
                               // replace the oracle's own decisions (replays a logged run)
    double* tr_log;            // trust region: NULL, or receives the oracle's own decisions in the
                               // same layout
};
}
