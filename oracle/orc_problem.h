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
    int32_t acceleration;      // 0 none, 1 Chebyshev, 2 Anderson
    double rho;                // Chebyshev spectral radius estimate
    int32_t chebyshev_formula; // 0: reference weights (sim/vbd/Kernels.h:96-102), 1: textbook
    int32_t semantics;         // 0: CPU integrator (vtm1 = v), 1: GPU integrator (vtm1 = v(t-1))
    int32_t nthreads;          // <= 0: OpenMP default
    int32_t window;            // Anderson window (acceleration 2)
};
}
