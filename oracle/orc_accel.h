// Acceleration loops of the FP64 oracle, shared by the plain step (vbd_oracle.cpp) and the
// contact-enabled step (contact_oracle.cpp).  TEST INFRASTRUCTURE ONLY.
#pragma once

#include "orc_problem.h"

#include <cstdint>
#include <functional>

namespace orc {

using Sweep     = std::function<void()>;   // one VBD iteration over every colour, in place on x
using Objective = std::function<double()>; // the backward-Euler objective at the current x

// AndersonIntegrator::Solve (sim/vbd/AndersonIntegrator.cpp:24-57) over 3 nV doubles.
void anderson_solve(orc_problem const& P, double* x, int32_t nV, int32_t iterations, Sweep const& sweep);

// TrustRegionIntegrator::SolveWithLinearAcceleratedPath (gpu/impl/vbd/TrustRegionIntegrator.cu:
// 48-165).  forced: NULL or a logged run's decisions to replay (4 doubles per iteration); log: NULL
// or receives this run's decisions.
void trust_region_solve(orc_problem const& P, double* x, int32_t nV, int32_t iterations, Sweep const& sweep,
                        Objective const& objective, double const* forced, double* log);

} // namespace orc
