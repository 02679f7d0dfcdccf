"""The adjoint on the device (pbat.gpu.vbd.rollout): a recorded step equals an unrecorded one, the
FP32 device gradient agrees with the FP64 oracle adjoint, and with FP64 central differences of the
oracle's forward integrator on the differentiation beam (40 x 10 x 10 hexes, 30 steps of 20
iterations, dt = 1/60, 32 seeded directions, eps = 1e-5)."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def gpu_integrator(w, strategy=2, **extra):
    nT = w["T"].shape[0]
    mu, lam = meshgen.lame(np.exp(w["logE"]), np.full(nT, w["nu"]))
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], mu, lam)
         .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(strategy))
    if "rho_chebyshev" in extra:
        d = d.with_chebyshev_acceleration(extra["rho_chebyshev"])
    if "kD" in extra:
        d = d.with_rayleigh_damping(extra["kD"])
    return pbat.gpu.vbd.Integrator(d.construct())


def device_gradients(w, v0, dt, iters, steps, strategy=2, every=5, x0=None):
    """(loss, dL/dlogE, dL/dv0, dL/dx0) from the device rollout."""
    I = gpu_integrator(w, strategy)
    nu = w["nu"]
    logE = torch.tensor(w["logE"], dtype=torch.float64, requires_grad=True)
    E = torch.exp(logE)
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    x0 = torch.tensor(w["X"] if x0 is None else x0, dtype=torch.float32, device="cuda", requires_grad=True)
    v0t = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    xT, vT = pbat.gpu.vbd.rollout(I, mu, lam, x0, v0t, dt=dt, iterations=iters, steps=steps, checkpoint_every=every)
    tip = torch.tensor(w["tip"], device="cuda")
    target = torch.tensor(w["target"], dtype=torch.float32, device="cuda")
    L = ((xT[tip] - target) ** 2).sum()
    L.backward()
    return (float(L.detach()), logE.grad.numpy().copy(), v0t.grad.cpu().numpy().astype(np.float64),
            x0.grad.cpu().numpy().astype(np.float64))


def oracle_of(w, logE, v0, strategy=2):
    nT = w["T"].shape[0]
    mu, lam = meshgen.lame(np.exp(logE), np.full(nT, w["nu"]))
    return O.OracleVbd(w["X"], w["T"], w["rho"], mu, lam, w["dbc"], v=v0, strategy=strategy, semantics=1)


def oracle_gradients(w, v0, dt, iters, steps, strategy=2):
    I = oracle_of(w, w["logE"], v0, strategy)
    I.step(dt, iters, 1, steps)
    xb = np.zeros_like(w["X"])
    xb[w["tip"]] = 2.0 * (I.x[w["tip"]] - w["target"])
    gx, gv, gmu, gla = oracle_of(w, w["logE"], v0, strategy).adjoint(dt, iters, 1, steps, xb, np.zeros_like(xb))
    return np.sum((I.x[w["tip"]] - w["target"]) ** 2), gmu + gla, gv, gx


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_recorded_step_reproduces_the_step():
    w = meshgen.adjoint_beam_workload(nx=12, ny=3, nz=3)
    A = gpu_integrator(w)
    B = gpu_integrator(w)
    B.adjoint_reserve(2, 15)
    for _ in range(4):
        A.step(1 / 60, 15, 2)
        B.step_record(1 / 60, 15, 2, 0)
    np.testing.assert_array_equal(A.x, B.x)
    np.testing.assert_array_equal(A.v, B.v)


@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_device_adjoint_matches_oracle_adjoint(strategy):
    w = meshgen.adjoint_beam_workload(nx=8, ny=2, nz=2, seed=2)
    v0 = np.random.default_rng(2).uniform(-0.5, 0.5, w["X"].shape)
    v0[w["dbc"]] = 0.0
    L, gE, gv, gx = device_gradients(w, v0, 1 / 60, 10, 5, strategy=strategy, every=2)
    Lr, gEr, gvr, gxr = oracle_gradients(w, v0, 1 / 60, 10, 5, strategy=strategy)
    assert abs(L - Lr) <= 1e-4 * Lr
    assert rel(gE, gEr) <= 1e-3
    assert rel(gv, gvr) <= 1e-3
    assert rel(gx, gxr) <= 1e-3


def test_checkpoint_interval_does_not_change_the_gradient():
    """Recomputed segments reproduce the forward bit for bit; what differs between two backward
    passes is only the order of the FP32 atomic additions into the neighbours' adjoints."""
    w = meshgen.adjoint_beam_workload(nx=8, ny=2, nz=2, seed=6)
    v0 = np.zeros_like(w["X"])
    g1 = device_gradients(w, v0, 1 / 60, 8, 6, every=1)
    g6 = device_gradients(w, v0, 1 / 60, 8, 6, every=6)
    assert g1[0] == g6[0]
    for a, b in zip(g1[1:], g6[1:]):
        assert rel(a, b) <= 1e-3


def test_adjoint_beam_gradients_match_fp64_finite_differences():
    """The differentiation workload: gradients w.r.t. per-tet log E, v0 and x0."""
    w = meshgen.adjoint_beam_workload()
    dt, iters, steps = 1 / 60, 20, 30
    v0 = np.zeros_like(w["X"])
    L, gE, gv, gx = device_gradients(w, v0, dt, iters, steps)
    Lr, gEr, gvr, gxr = oracle_gradients(w, v0, dt, iters, steps)
    assert abs(L - Lr) <= 1e-3 * Lr
    assert rel(gE, gEr) <= 1e-3
    assert rel(gv, gvr) <= 1e-3
    assert rel(gx, gxr) <= 1e-3
    rng = np.random.default_rng(20261203)
    eps = 1e-5
    ad, fd = [], []
    for _ in range(32):
        dE = rng.standard_normal(gE.size)
        dv = rng.standard_normal(v0.shape)
        dv[w["dbc"]] = 0.0

        def f(s):
            I = oracle_of(w, w["logE"] + s * dE, v0 + s * dv)
            I.step(dt, iters, 1, steps)
            return np.sum((I.x[w["tip"]] - w["target"]) ** 2)

        fd.append((f(eps) - f(-eps)) / (2 * eps))
        ad.append(gE @ dE + np.sum(gv * dv))
    ad, fd = np.array(ad), np.array(fd)
    err = np.abs(ad - fd) / np.abs(fd)
    assert np.all(err <= 1e-3), (err.max(), ad, fd)


def test_rollout_rejects_unsupported_settings():
    w = meshgen.adjoint_beam_workload(nx=4, ny=2, nz=2)
    nT = w["T"].shape[0]
    mu = torch.ones(nT, dtype=torch.float64)
    x0 = torch.tensor(w["X"], dtype=torch.float32, device="cuda")
    for I in (gpu_integrator(w, strategy=4), gpu_integrator(w, rho_chebyshev=0.9), gpu_integrator(w, kD=1e-3)):
        with pytest.raises(_capi.PbgbError):
            pbat.gpu.vbd.rollout(I, mu * 1e5, mu * 1e6, x0, torch.zeros_like(x0), steps=1)
