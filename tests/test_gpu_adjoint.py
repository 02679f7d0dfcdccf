"""The adjoint on the device (pbat.gpu.vbd.rollout): a recorded step equals an unrecorded one, the
FP32 device gradient agrees with the FP64 oracle adjoint (every initial guess, Rayleigh damping,
Chebyshev), and with FP64 central differences of the oracle's forward integrator on the
differentiation beam (40 x 10 x 10 hexes, 30 steps of 20 iterations, dt = 1/60, 32 seeded
directions, eps = 1e-5), with KineticEnergyMinimum and with the reference Data's default initial
guess, AdaptivePbat."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def gpu_integrator(w, strategy=2, **extra):
    """strategy None: the Data builder's default initial guess (AdaptivePbat, as the reference's)."""
    nT = w["T"].shape[0]
    mu, lam = meshgen.lame(np.exp(w["logE"]), np.full(nT, w["nu"]))
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], mu, lam)
         .with_dirichlet_vertices(w["dbc"]))
    if strategy is not None:
        d = d.with_initialization_strategy(strategy)
    if "rho_chebyshev" in extra:
        d = d.with_chebyshev_acceleration(extra["rho_chebyshev"], extra.get("formula", "reference"))
    if "kD" in extra:
        d = d.with_rayleigh_damping(extra["kD"])
    if "anderson" in extra:
        d = d.with_anderson_acceleration(extra["anderson"])
    return pbat.gpu.vbd.Integrator(d.construct())


def device_gradients(w, v0, dt, iters, steps, strategy=2, every=5, x0=None, **extra):
    """(loss, dL/dlogE, dL/dv0, dL/dx0) from the device rollout."""
    I = gpu_integrator(w, strategy, **extra)
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


def oracle_kw(extra):
    kw = {}
    if "rho_chebyshev" in extra:
        kw["rho_chebyshev"] = extra["rho_chebyshev"]
        kw["chebyshev_formula"] = 1 if extra.get("formula") == "textbook" else 0
    if "kD" in extra:
        kw["kD"] = extra["kD"]
    return kw


def oracle_of(w, logE, v0, strategy=2, **extra):
    nT = w["T"].shape[0]
    mu, lam = meshgen.lame(np.exp(logE), np.full(nT, w["nu"]))
    return O.OracleVbd(w["X"], w["T"], w["rho"], mu, lam, w["dbc"], v=v0, strategy=4 if strategy is None else strategy,
                       semantics=1, **oracle_kw(extra))


def oracle_gradients(w, v0, dt, iters, steps, strategy=2, **extra):
    I = oracle_of(w, w["logE"], v0, strategy, **extra)
    I.step(dt, iters, 1, steps)
    xb = np.zeros_like(w["X"])
    xb[w["tip"]] = 2.0 * (I.x[w["tip"]] - w["target"])
    gx, gv, gmu, gla = oracle_of(w, w["logE"], v0, strategy, **extra).adjoint(dt, iters, 1, steps, xb,
                                                                              np.zeros_like(xb))
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


@pytest.mark.parametrize("extra", [dict(), dict(kD=1e-2), dict(rho_chebyshev=0.9),
                                   dict(rho_chebyshev=0.85, formula="textbook", kD=5e-3)])
@pytest.mark.parametrize("strategy", [0, 1, 2, 3, 4])
def test_device_adjoint_matches_oracle_adjoint(strategy, extra):
    w = meshgen.adjoint_beam_workload(nx=8, ny=2, nz=2, seed=2)
    v0 = np.random.default_rng(2).uniform(-0.5, 0.5, w["X"].shape)
    v0[w["dbc"]] = 0.0
    L, gE, gv, gx = device_gradients(w, v0, 1 / 60, 10, 5, strategy=strategy, every=2, **extra)
    Lr, gEr, gvr, gxr = oracle_gradients(w, v0, 1 / 60, 10, 5, strategy=strategy, **extra)
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


@pytest.mark.parametrize("every", [2, 5])
def test_a_second_backward_re_records_the_taped_segment(every):
    """The forward pass tapes its last segment and the first backward reverses it directly; the
    other segments reuse the tape's slots, so a second backward (retain_graph) records every segment
    again and must give the same gradients."""
    w = meshgen.adjoint_beam_workload(nx=8, ny=2, nz=2, seed=4)
    I = gpu_integrator(w)
    nu = w["nu"]
    logE = torch.tensor(w["logE"], dtype=torch.float64, requires_grad=True)
    E = torch.exp(logE)
    mu, lam = E / (2 * (1 + nu)), E * nu / ((1 + nu) * (1 - 2 * nu))
    x0 = torch.tensor(w["X"], dtype=torch.float32, device="cuda", requires_grad=True)
    v0 = torch.zeros_like(x0, requires_grad=True)
    xT, _ = pbat.gpu.vbd.rollout(I, mu, lam, x0, v0, dt=1 / 60, iterations=8, steps=5, checkpoint_every=every)
    L = (xT ** 2).sum()
    L.backward(retain_graph=True)
    g1 = (logE.grad.clone(), x0.grad.clone(), v0.grad.clone())
    logE.grad, x0.grad, v0.grad = None, None, None
    L.backward()
    for a, b in zip(g1, (logE.grad, x0.grad, v0.grad)):
        assert rel(b.cpu().numpy(), a.cpu().numpy()) <= 1e-4


def fd_check(w, v0, gE, gv, gx, dt, iters, steps, strategy, directions=32, with_v=True, with_x=False, eps=1e-5):
    rng = np.random.default_rng(20261203)
    ad, fd = [], []
    for _ in range(directions):
        dE = rng.standard_normal(gE.size)
        dv = rng.standard_normal(v0.shape) if with_v else np.zeros_like(v0)
        dv[w["dbc"]] = 0.0
        dx = 0.01 * rng.standard_normal(v0.shape) if with_x else np.zeros_like(v0)

        def f(s):
            I = oracle_of(w, w["logE"] + s * dE, v0 + s * dv, strategy)
            I.x = I.x + s * dx
            I.step(dt, iters, 1, steps)
            return np.sum((I.x[w["tip"]] - w["target"]) ** 2)

        fd.append((f(eps) - f(-eps)) / (2 * eps))
        ad.append(gE @ dE + np.sum(gv * dv) + np.sum(gx * dx))
    ad, fd = np.array(ad), np.array(fd)
    # Relative to the directional derivative, but to no less than a tenth of the largest one: a
    # direction nearly orthogonal to the gradient (a derivative 100x below the others) is a
    # difference of large FP32 terms, and its relative error says nothing of the gradient's.
    err = np.abs(ad - fd) / np.maximum(np.abs(fd), 0.1 * np.abs(fd).max())
    assert np.all(err <= 1e-3), (err.max(), ad, fd)


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
    fd_check(w, v0, gE, gv, gx, dt, iters, steps, 2)


def test_adjoint_beam_default_initial_guess_matches_fp64_finite_differences():
    """The same workload with the reference Data's default initial guess, AdaptivePbat
    (x0 = xt + h v + h^2 min(|v.a| / (|v| |a|^2), 1) a).  Its factor jumps at v = 0, where the
    workload's initial velocities sit, so the directions there perturb log E only; the velocity
    directions are checked from a seeded non-zero start (|v| <= 0.05 m/s).  The x0 gradient is
    compared with the FP64 adjoint.

    The factor's |v.a| has a kink wherever a vertex's velocity turns perpendicular to gravity, and
    over 30 steps of 4961 vertices some velocity passes within 1e-5 of one: a central difference
    of step 1e-5 straddles a kink in most directions (errors up to 20 %), one of step 1e-6 in
    almost none (1e-7 agreement on the FP64 oracle), so the velocity directions use 1e-6."""
    w = meshgen.adjoint_beam_workload()
    dt, iters, steps = 1 / 60, 20, 30
    v0 = np.zeros_like(w["X"])
    L, gE, gv, gx = device_gradients(w, v0, dt, iters, steps, strategy=None)
    Lr, gEr, gvr, gxr = oracle_gradients(w, v0, dt, iters, steps, strategy=None)
    assert abs(L - Lr) <= 1e-3 * Lr
    assert rel(gE, gEr) <= 1e-3
    assert rel(gx, gxr) <= 1e-3
    fd_check(w, v0, gE, gv, gx, dt, iters, steps, None, directions=16, with_v=False)
    v1 = np.random.default_rng(7).uniform(-0.05, 0.05, w["X"].shape)
    v1[w["dbc"]] = 0.0
    L, gE, gv, gx = device_gradients(w, v1, dt, iters, steps, strategy=None)
    Lr, gEr, gvr, gxr = oracle_gradients(w, v1, dt, iters, steps, strategy=None)
    assert rel(gv, gvr) <= 1e-3
    fd_check(w, v1, gE, gv, gx, dt, iters, steps, None, directions=16, eps=1e-6)


def test_rollout_rejects_unsupported_settings():
    w = meshgen.adjoint_beam_workload(nx=4, ny=2, nz=2)
    nT = w["T"].shape[0]
    mu = torch.ones(nT, dtype=torch.float64)
    x0 = torch.tensor(w["X"], dtype=torch.float32, device="cuda")
    I = gpu_integrator(w, anderson=3)
    with pytest.raises(_capi.PbgbError):
        pbat.gpu.vbd.rollout(I, mu * 1e5, mu * 1e6, x0, torch.zeros_like(x0), steps=1)


def test_adaptive_vbd_needs_the_state_entry_point():
    """AdaptiveVbd under the GPU semantics reads the previous velocity: the entry point without its
    adjoint refuses it, the state entry point carries it."""
    w = meshgen.adjoint_beam_workload(nx=4, ny=2, nz=2)
    I = gpu_integrator(w, strategy=3)
    I.adjoint_reserve(1, 4)
    I.step_record(1 / 60, 4, 1, 0)
    n, nT = I.n_vertices, I.n_tets
    xb = torch.zeros((n, 3), device="cuda")
    vb, pb = torch.zeros_like(xb), torch.zeros_like(xb)
    dm = torch.zeros(nT, dtype=torch.float64, device="cuda")
    dl = torch.zeros_like(dm)
    with pytest.raises(_capi.PbgbError):
        I.step_adjoint(0, 1, xb.data_ptr(), vb.data_ptr(), dm.data_ptr(), dl.data_ptr())
    I.step_adjoint(0, 1, xb.data_ptr(), vb.data_ptr(), dm.data_ptr(), dl.data_ptr(), pb.data_ptr())
    I.synchronize()
