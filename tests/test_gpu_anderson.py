"""Anderson-accelerated VBD on the device (sim/vbd/AndersonIntegrator.cpp,
gpu/impl/vbd/AndersonIntegrator.cu) against the FP64 oracle restatement."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

pytestmark = pytest.mark.gpu


def data_for(w, window, strategy=2):
    return (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
            .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(strategy)
            .with_anderson_acceleration(window).construct())


def test_reference_doctest_properties_on_device():
    """The 5-tet cube, window 5, one step of 10 iterations at dt = 1e-2: vertices fall and only
    fall, the FP64 objective gradient is below 1e-4 and the objective decreased."""
    P, T, _, _ = meshgen.cube5()
    d = pbat.sim.vbd.Data().with_volume_mesh(P, T).with_anderson_acceleration(5).construct()
    I = pbat.sim.vbd.Integrator(d)
    dt = 1e-2
    f0 = None
    I.step(dt, 0, 1)  # zero iterations: the objective at the initial guess against this step's target
    I.x = P
    f0 = I.objective(dt)
    I.x = P
    I.v = np.zeros_like(P)
    I.step(dt, 10, 1)
    dx = I.x - P
    assert (dx[2] < 0).all()
    assert (np.abs(dx[:2]) < 1e-4).all()
    assert np.linalg.norm(I.gradient(dt)) < 1e-4
    assert I.objective(dt) < f0


@pytest.mark.parametrize("window", [1, 3, 5, 8])
def test_unit_cube_matches_oracle(window):
    w = meshgen.unit_cube_workload(n=7, seed=3)
    I = pbat.gpu.vbd.Integrator(data_for(w, window))
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2, semantics=1,
                    anderson_window=window)
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    for _ in range(10):
        I.step(1 / 60, 15, 1)
    R.step(1 / 60, 15, 1, 10)
    err = np.abs(I.x.T - R.x).max() / diag
    assert err <= 1e-4, err


def test_beam_with_substeps_matches_oracle():
    X, T = meshgen.hex_grid(12, 3, 3, hi=(4.0, 1.0, 1.0))
    nT = T.shape[0]
    mu, lam = meshgen.lame(np.full(nT, 5e5), np.full(nT, 0.48))
    w = dict(X=X, T=T, dbc=meshgen.face_vertices(X, 0, 0.0), rho=np.full(nT, 1000.0), mu=mu, lam=lam)
    I = pbat.gpu.vbd.Integrator(data_for(w, 5))
    R = O.OracleVbd(X, T, w["rho"], mu, lam, w["dbc"], strategy=2, semantics=1, anderson_window=5)
    for _ in range(6):
        I.step(1 / 60, 12, 2)
    R.step(1 / 60, 12, 2, 6)
    diag = np.linalg.norm(X.max(0) - X.min(0))
    assert np.abs(I.x.T - R.x).max() / diag <= 1e-4


def test_anderson_reduces_the_residual_faster_than_plain_vbd():
    w = meshgen.unit_cube_workload(n=8, seed=1)

    def grad_norm(window):
        d = data_for(w, window) if window else (
            pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
            .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(2).construct())
        I = pbat.sim.vbd.Integrator(d)
        I.step(1 / 60, 15, 1)
        g = I.gradient(1 / 60).reshape(-1, 3)
        g[w["dbc"]] = 0.0
        return np.linalg.norm(g)

    assert grad_norm(5) < 0.5 * grad_norm(None)


def test_anderson_rejects_batched_contact_and_bad_windows():
    w = meshgen.unit_cube_workload(n=3)
    with pytest.raises(_capi.PbgbError):
        pbat.gpu.vbd.BatchedIntegrator([data_for(w, 5), data_for(w, 5)])
    with pytest.raises(_capi.PbgbError):
        pbat.gpu.vbd.Integrator(data_for(w, 17))
