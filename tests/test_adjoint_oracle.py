"""The FP64 oracle adjoint against FP64 central differences of the oracle's forward step (the
restated reference integrator).  No reference counterpart exists: the reference has no adjoint, so
the finite differences pin it."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen


def small_beam(seed=3):
    w = meshgen.adjoint_beam_workload(nx=8, ny=2, nz=2, seed=seed)
    rng = np.random.default_rng(seed)
    v0 = rng.uniform(-0.5, 0.5, w["X"].shape)
    v0[w["dbc"]] = 0.0
    return w, v0


def oracle(w, logE, v0, strategy, semantics=1, **kw):
    nT = w["T"].shape[0]
    mu, lam = meshgen.lame(np.exp(logE), np.full(nT, w["nu"]))
    return O.OracleVbd(w["X"], w["T"], w["rho"], mu, lam, w["dbc"], v=v0, strategy=strategy, semantics=semantics, **kw)


# (strategy, semantics, extra settings): every initial guess with both step semantics where they
# differ, Rayleigh damping and Chebyshev (the reference's weight recurrence and the textbook one).
SETTINGS = [
    (0, 1, {}), (1, 1, {}), (2, 1, {}),
    (3, 1, {}), (3, 0, {}), (4, 1, {}), (4, 0, {}),
    (2, 1, dict(kD=1e-2)), (4, 1, dict(kD=5e-3)),
    (2, 1, dict(rho_chebyshev=0.9)), (4, 1, dict(rho_chebyshev=0.9, chebyshev_formula=1)),
    (3, 1, dict(rho_chebyshev=0.85, kD=1e-2)),
]


@pytest.mark.parametrize("strategy,semantics,kw", SETTINGS)
def test_oracle_adjoint_matches_central_differences(strategy, semantics, kw):
    """Loss of the tip vertices after 5 steps; central differences along 6 random directions of
    (log E, v0, x0, and the previous velocity for AdaptiveVbd under the GPU integrator's semantics,
    which reads it).  Random non-zero initial velocities keep AdaptivePbat away from v = 0, where
    its clamp factor |v.a| / (|v| |a|^2) is not differentiable."""
    w, v0 = small_beam()
    rng0 = np.random.default_rng(17)
    p0 = rng0.uniform(-0.5, 0.5, v0.shape)
    p0[w["dbc"]] = 0.0
    dt, iters, nsteps = 1 / 60, 10, 5
    tip, target = w["tip"], w["target"]

    def make(logE, v, p):
        I = oracle(w, logE, v, strategy, semantics, **kw)
        I.vprev[:] = p
        return I

    def loss(logE, v, dx, p):
        I = make(logE, v, p)
        I.x = I.x + dx
        I.step(dt, iters, 1, nsteps)
        return np.sum((I.x[tip] - target) ** 2), I

    L0, I = loss(w["logE"], v0, 0.0, p0)
    xb = np.zeros_like(w["X"])
    xb[tip] = 2.0 * (I.x[tip] - target)
    gx, gv, gmu, gla, gp = make(w["logE"], v0, p0).adjoint(dt, iters, 1, nsteps, xb, np.zeros_like(xb),
                                                            with_vprev=True)
    if not (strategy == 3 and semantics == 1):
        assert not gp.any()
    glogE = gmu + gla
    rng = np.random.default_rng(11)
    eps = 1e-5
    for _ in range(6):
        dE = rng.standard_normal(glogE.size)
        dv = rng.standard_normal(v0.shape)
        dv[w["dbc"]] = 0.0
        dp = rng.standard_normal(v0.shape)
        dp[w["dbc"]] = 0.0
        dx = 0.01 * rng.standard_normal(v0.shape)
        fp = loss(w["logE"] + eps * dE, v0 + eps * dv, eps * dx, p0 + eps * dp)[0]
        fm = loss(w["logE"] - eps * dE, v0 - eps * dv, -eps * dx, p0 - eps * dp)[0]
        fd = (fp - fm) / (2 * eps)
        ad = glogE @ dE + np.sum(gv * dv) + np.sum(gx * dx) + np.sum(gp * dp)
        assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-9, (ad, fd)


def test_oracle_adjoint_with_substeps():
    w, v0 = small_beam(seed=4)
    dt, iters, substeps, nsteps = 1 / 30, 6, 2, 3
    tip, target = w["tip"], w["target"]

    def loss(logE):
        I = oracle(w, logE, v0, 2)
        I.step(dt, iters, substeps, nsteps)
        return np.sum((I.x[tip] - target) ** 2), I

    _, I = loss(w["logE"])
    xb = np.zeros_like(w["X"])
    xb[tip] = 2.0 * (I.x[tip] - target)
    _, _, gmu, gla = oracle(w, w["logE"], v0, 2).adjoint(dt, iters, substeps, nsteps, xb, np.zeros_like(xb))
    dE = np.random.default_rng(5).standard_normal(gmu.size)
    eps = 1e-5
    fd = (loss(w["logE"] + eps * dE)[0] - loss(w["logE"] - eps * dE)[0]) / (2 * eps)
    assert abs((gmu + gla) @ dE - fd) <= 1e-6 * abs(fd)


def test_oracle_adjoint_rejects_unsupported_settings():
    w, v0 = small_beam()
    nT = w["T"].shape[0]
    mu, lam = meshgen.lame(np.exp(w["logE"]), np.full(nT, w["nu"]))
    for kw in (dict(anderson_window=3), dict(broyden_window=3)):
        I = O.OracleVbd(w["X"], w["T"], w["rho"], mu, lam, w["dbc"], v=v0, semantics=1, strategy=2, **kw)
        with pytest.raises(RuntimeError):
            I.adjoint(1 / 60, 5, 1, 1, np.zeros_like(v0), np.zeros_like(v0))


def phi_tet(xe, Xe, il, w, delta, mu, lam):
    """phi_e = w . (g_e - H_e delta) for corner il of one tet, from the oracle's Stable Neo-Hookean
    gradient and 9x9 Hessian (the reference's own derivatives, pinned in test_oracle)."""
    Dm = np.stack([Xe[1] - Xe[0], Xe[2] - Xe[0], Xe[3] - Xe[0]], axis=1)
    wg = np.linalg.det(Dm) / 6.0
    Ji = np.linalg.inv(Dm)
    G = np.zeros((4, 3))
    G[1:] = Ji
    G[0] = -Ji.sum(axis=0)
    F = xe.T @ G  # sum_a x_a G_a^T
    gF = np.zeros(9)
    HF = np.zeros(81)
    O.lib().orc_snh_grad_hessian(np.ascontiguousarray(F.ravel(order="F")), mu, lam, gF, HF)
    HF = HF.reshape(9, 9)
    go = G[il]
    g = wg * gF.reshape(3, 3, order="F") @ go
    H = np.zeros((3, 3))
    for k in range(3):
        for l in range(3):
            H += wg * go[k] * go[l] * HF[3 * k:3 * k + 3, 3 * l:3 * l + 3]
    return w @ (g - H @ delta), wg


def debug_adjoint_tet(prec, xe, Xe, il, w, delta, muw, law):
    from physicsbasedanimationtoolkit_gb300 import _capi
    import ctypes as C
    dphi = np.zeros(12)
    dm, dl = C.c_double(), C.c_double()
    rc = _capi.lib().pbgb_debug_adjoint_tet(prec, np.ascontiguousarray(xe, np.float64).ctypes.data,
                                            np.ascontiguousarray(Xe, np.float64).ctypes.data, il,
                                            np.ascontiguousarray(w, np.float64).ctypes.data,
                                            np.ascontiguousarray(delta, np.float64).ctypes.data, muw, law,
                                            dphi.ctypes.data, C.byref(dm), C.byref(dl))
    assert rc == 0
    return dphi.reshape(4, 3), dm.value, dl.value


@pytest.mark.parametrize("seed", range(6))
def test_adjoint_tet_matches_finite_differences_of_the_reference_derivatives(seed):
    """The closed-form per-tet adjoint term of the device sweep (FP64 host instantiation) against
    central differences of phi_e built from the reference's SNH gradient and Hessian."""
    rng = np.random.default_rng(seed)
    Xe = rng.standard_normal((4, 3)) * 0.1
    while np.linalg.det(np.stack([Xe[1] - Xe[0], Xe[2] - Xe[0], Xe[3] - Xe[0]], axis=1)) < 1e-4:
        Xe = rng.standard_normal((4, 3)) * 0.1
    xe = Xe + 0.03 * rng.standard_normal((4, 3))
    il = int(rng.integers(0, 4))
    w, delta = rng.standard_normal(3), 0.01 * rng.standard_normal(3)
    mu, lam = rng.uniform(1e4, 1e6), rng.uniform(1e5, 1e7)
    _, wg = phi_tet(xe, Xe, il, w, delta, mu, lam)
    dphi, dm, dl = debug_adjoint_tet(64, xe, Xe, il, w, delta, wg * mu, wg * lam)
    h = 1e-6
    fd = np.zeros((4, 3))
    for a in range(4):
        for r in range(3):
            xp, xm = xe.copy(), xe.copy()
            xp[a, r] += h
            xm[a, r] -= h
            fd[a, r] = (phi_tet(xp, Xe, il, w, delta, mu, lam)[0] - phi_tet(xm, Xe, il, w, delta, mu, lam)[0]) / (2 * h)
    np.testing.assert_allclose(dphi, fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())
    s = 1e-6
    fmu = (phi_tet(xe, Xe, il, w, delta, mu * np.exp(s), lam)[0] - phi_tet(xe, Xe, il, w, delta, mu * np.exp(-s), lam)[0]) / (2 * s)
    fla = (phi_tet(xe, Xe, il, w, delta, mu, lam * np.exp(s))[0] - phi_tet(xe, Xe, il, w, delta, mu, lam * np.exp(-s))[0]) / (2 * s)
    assert abs(dm - fmu) <= 1e-5 * abs(fmu) + 1e-8 * abs(wg * mu)
    assert abs(dl - fla) <= 1e-5 * abs(fla) + 1e-8 * abs(wg * lam)


def test_adjoint_tet_material_terms_keep_precision_in_fp32_at_small_strain():
    """At strain 1e-4 far from the origin, the FP32 material sensitivities stay within 1e-3 of
    FP64: they are formed from the displacement gradient, not as differences of O(1) terms."""
    rng = np.random.default_rng(9)
    worst = 0.0
    for _ in range(50):
        Xe = np.array([4.0, 0.5, 0.5]) + 0.1 * np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]) + 0.01 * rng.standard_normal((4, 3))
        Xe = Xe.astype(np.float32).astype(np.float64)
        xe = (Xe + 1e-5 * rng.standard_normal((4, 3))).astype(np.float32).astype(np.float64)
        w, delta = rng.standard_normal(3), 1e-6 * rng.standard_normal(3)
        _, dm64, dl64 = debug_adjoint_tet(64, xe, Xe, 0, w, delta, 1e3, 1e4)
        _, dm32, dl32 = debug_adjoint_tet(32, xe, Xe, 0, w, delta, 1e3, 1e4)
        worst = max(worst, abs(dm32 - dm64) / abs(dm64), abs(dl32 - dl64) / abs(dl64))
    assert worst <= 1e-3, worst
