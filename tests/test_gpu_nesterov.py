"""Nesterov-accelerated VBD on the device (sim/vbd/NesterovIntegrator.cpp:16-43) against the FP64
oracle restatement of the same iteration.  Nesterov is a CPU-integrator strategy in the reference,
so it runs through ``pbat.sim.vbd.Integrator`` (the GPU integrator runs plain VBD for it).

The reference keeps x_{k-1} at the solve's start iterate, so accelerated iterations pull the
iterate back towards that start; over many steps the iteration diverges.  Parity is therefore
checked on short runs (one to five steps) where the oracle's own sensitivity to a 1e-6 input
perturbation stays at the perturbation's size."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

pytestmark = pytest.mark.gpu


def data_for(w, L, start, strategy=2):
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
         .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(strategy))
    if L is not None:
        d = d.with_nesterov_acceleration(L, start)
    return d.construct()


@pytest.mark.parametrize("L,start,iterations,steps", [(1.0, 3, 8, 1), (4.0, 3, 8, 1), (1.0, 5, 10, 2),
                                                      (2.0, 6, 10, 3), (1.0, 8, 10, 5)])
def test_unit_cube_matches_oracle(L, start, iterations, steps):
    w = meshgen.unit_cube_workload(n=7, seed=3)
    I = pbat.sim.vbd.Integrator(data_for(w, L, start))
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2, semantics=0,
                    nesterov=(L, start))
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    for _ in range(steps):
        I.step(1 / 60, iterations, 1)
    R.step(1 / 60, iterations, 1, steps)
    assert np.abs(R.x - w["X"]).max() > 1e-3  # the run moved
    err = np.abs(I.x.T - R.x).max() / diag
    assert err <= 1e-4, err


def test_substeps_match_oracle():
    w = meshgen.unit_cube_workload(n=5, seed=2)
    I = pbat.sim.vbd.Integrator(data_for(w, 2.0, 4))
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2, semantics=0,
                    nesterov=(2.0, 4))
    for _ in range(2):
        I.step(1 / 60, 7, 2)
    R.step(1 / 60, 7, 2, 2)
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    assert np.abs(I.x.T - R.x).max() / diag <= 1e-4


def test_without_accelerated_iterations_equals_plain_vbd():
    """start >= iterations - 1 leaves every iteration unaccelerated: the same sweeps as plain VBD,
    bit for bit."""
    w = meshgen.unit_cube_workload(n=6, seed=4)
    A = pbat.sim.vbd.Integrator(data_for(w, 1.0, 9))
    B = pbat.sim.vbd.Integrator(data_for(w, None, 0))
    for _ in range(4):
        A.step(1 / 60, 10, 1)
        B.step(1 / 60, 10, 1)
    np.testing.assert_array_equal(A.x, B.x)
    np.testing.assert_array_equal(A.v, B.v)



def test_gpu_integrator_runs_plain_vbd_for_nesterov():
    """gpu/vbd/Integrator.cu:15-33 builds the base integrator for Nesterov data."""
    w = meshgen.unit_cube_workload(n=5, seed=1)
    A = pbat.gpu.vbd.Integrator(data_for(w, 1.0, 2))
    B = pbat.gpu.vbd.Integrator(data_for(w, None, 0))
    for _ in range(3):
        A.step(1 / 60, 10, 1)
        B.step(1 / 60, 10, 1)
    np.testing.assert_array_equal(A.x, B.x)
