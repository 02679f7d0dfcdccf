"""Descent-path traces in the reference's Matrix Market formats: the GPU integrator's
TracedStep (gpu/impl/vbd/Integrator.cu:105-148,284-301) and the CPU integrator's TraceNextStep
(sim/vbd/Integrator.cpp:47-52,202-235), read back with scipy.io.mmread."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

sio = pytest.importorskip("scipy.io")
pytestmark = pytest.mark.gpu


def data_for(w, **kw):
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
         .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(2))
    if "rho" in kw:
        d = d.with_chebyshev_acceleration(kw["rho"])
    return d.construct()


def test_gpu_traced_step_files(tmp_path):
    w = meshgen.unit_cube_workload(n=4, seed=2)
    d = data_for(w, rho=0.9)
    I = pbat.gpu.vbd.Integrator(d)
    x0 = I.x.copy()
    dt, iters = 1 / 60, 6
    I.traced_step(dt, iters, 2, t=0, dir=str(tmp_path))
    nV, nT = w["X"].shape[0], w["T"].shape[0]
    np.testing.assert_array_equal(sio.mmread(tmp_path / "T.mtx"), w["T"])
    np.testing.assert_allclose(np.asarray(sio.mmread(tmp_path / "M.mtx")).ravel(), d.m, rtol=1e-15)
    np.testing.assert_allclose(np.asarray(sio.mmread(tmp_path / "wg.mtx")).ravel(), d.wg, rtol=1e-15)
    np.testing.assert_allclose(sio.mmread(tmp_path / "GP.mtx"), d.GP, rtol=1e-15)
    np.testing.assert_allclose(sio.mmread(tmp_path / "lame.mtx"), d.lame.T, rtol=1e-15)
    for s in range(2):
        assert sio.mmread(tmp_path / f"xtilde.t.0.s.{s}.mtx").shape == (nV, 3)
        for k in range(iters + 1):
            assert sio.mmread(tmp_path / f"x.t.0.s.{s}.k.{k}.mtx").shape == (nV, 3)
    # Substep 0: xtilde = x + h v + h^2 a (v = 0), the KineticEnergyMinimum guess equals it.
    h = dt / 2
    a = np.zeros_like(x0.T)
    a[:, 2] = -9.81
    a[w["dbc"]] = 0.0
    xt_expected = x0.T.astype(np.float64) + h * h * a
    np.testing.assert_allclose(sio.mmread(tmp_path / "xtilde.t.0.s.0.mtx"), xt_expected, atol=1e-6)
    np.testing.assert_allclose(sio.mmread(tmp_path / "x.t.0.s.0.k.0.mtx"), xt_expected, atol=1e-6)
    # Plain iterations (as the reference's TracedSolve), whatever the acceleration: the last
    # iterate equals a plain integrator's step from the same state, and the integrator advanced.
    P = pbat.gpu.vbd.Integrator(data_for(w))
    P.step(dt, iters, 2)
    last = sio.mmread(tmp_path / f"x.t.0.s.1.k.{iters}.mtx").astype(np.float32)
    np.testing.assert_array_equal(last, P.x.T)
    np.testing.assert_array_equal(I.x, P.x)
    # Frame > 0 writes no mesh files again.
    (tmp_path / "T.mtx").unlink()
    I.traced_step(dt, iters, 1, t=1, dir=str(tmp_path))
    assert not (tmp_path / "T.mtx").exists()
    assert (tmp_path / f"x.t.1.s.0.k.{iters}.mtx").exists()


@pytest.mark.parametrize("rho", [None, 0.9])
def test_cpu_trace_next_step_files(tmp_path, rho):
    w = meshgen.unit_cube_workload(n=4, seed=3)
    kw = {} if rho is None else {"rho": rho}
    I = pbat.sim.vbd.Integrator(data_for(w, **kw))
    J = pbat.sim.vbd.Integrator(data_for(w, **kw))
    dt, iters = 1 / 60, 8
    xt = I.x.T.astype(np.float64).copy()
    I.trace_next_step(str(tmp_path), 5)
    I.step(dt, iters, 1)
    J.step(dt, iters, 1)
    np.testing.assert_array_equal(I.x, J.x)  # a traced step computes the same positions
    f = np.asarray(sio.mmread(tmp_path / "5.0.f.mtx")).ravel()
    G = np.asarray(sio.mmread(tmp_path / "5.0.grad.mtx"))
    X = np.asarray(sio.mmread(tmp_path / "5.0.x.mtx"))
    nV = w["X"].shape[0]
    assert f.shape == (iters + 1,) and G.shape == (3 * nV, iters + 1) and X.shape == (3 * nV, iters + 1)
    np.testing.assert_array_equal(X[:, -1].astype(np.float32), I.x.T.ravel())
    assert f[-1] < f[0]
    # Objective and gradient against the FP64 oracle at the traced positions (the device sums FP32
    # per-element terms in FP64 against its FP32 inertial target).
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2)
    xtilde = xt + dt * R.v + dt * dt * R.aext
    for k in (0, iters // 2, iters):
        xk = X[:, k].reshape(-1, 3)
        assert abs(R.objective(xk, xtilde, dt) - f[k]) <= 1e-5 * abs(f[k])
        gk = R.gradient(xk, xtilde, dt)
        assert np.abs(gk - G[:, k]).max() <= 1e-3 * np.abs(gk).max()
    # Only the next step is traced.
    I.step(dt, iters, 1)
    assert not (tmp_path / "5.1.f.mtx").exists()
