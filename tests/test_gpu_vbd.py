"""GPU parity of the VBD step against the FP64 oracle, through the C ABI (pbat.* wrappers).

Tolerance: positions within 1e-4 of the bounding-box diagonal after the configured steps (FP32
device arithmetic against the FP64 oracle on the same mesh, colouring and iteration count)."""

import json
import pathlib

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

pytestmark = pytest.mark.gpu

TOL = 1e-4  # of the bounding-box diagonal
GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def make_data(w, strategy=None, kD=0.0, rho=None, formula="reference"):
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T)
         .with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
         .with_velocity(w["v"].T))
    if strategy is not None:
        d = d.with_initialization_strategy(strategy)
    if kD:
        d = d.with_rayleigh_damping(kD)
    if rho is not None:
        d = d.with_chebyshev_acceleration(rho, formula)
    return d.construct()


def oracle_for(w, strategy=4, kD=0.0, rho=None, formula=0, semantics=0):
    return O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], v=w["v"], strategy=strategy,
                       kD=kD, rho_chebyshev=rho, chebyshev_formula=formula, semantics=semantics)


def rel_err(xg, xo, X):
    diag = np.linalg.norm(X.max(0) - X.min(0))
    return np.abs(xg - xo).max() / diag


def test_unit_cube_30_steps_matches_oracle():
    """10x10x10 hex grid (1331 vertices, 6000 tets), 30 steps x 20 iterations, dt = 1/60."""
    w = meshgen.unit_cube_workload()
    I = pbat.sim.vbd.Integrator(make_data(w))
    for _ in range(30):
        I.step(1 / 60, 20, 1)
    R = oracle_for(w)
    R.step(1 / 60, 20, 1, 30)
    err = rel_err(I.x.T, R.x, w["X"])
    assert err <= TOL, err
    g = np.load(GOLD / "trajectories.npz")
    assert rel_err(I.x.T, g["cube10_x"], w["X"]) <= TOL
    # Something actually moved (the cube sags under gravity by several centimetres).
    assert (w["X"][:, 2] - I.x.T[:, 2]).max() > 1e-2


@pytest.mark.parametrize("strategy", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("semantics", ["sim", "gpu"])
def test_initialization_strategies_and_semantics(strategy, semantics):
    w = meshgen.unit_cube_workload(n=5, seed=11)
    w["v"] = np.random.default_rng(2).uniform(-0.2, 0.2, w["X"].shape)
    d = make_data(w, strategy=strategy, kD=1e-3 if strategy % 2 else 0.0)
    I = (pbat.sim.vbd.Integrator if semantics == "sim" else pbat.gpu.vbd.Integrator)(d)
    for _ in range(6):
        I.step(1 / 60, 10, 2)
    R = oracle_for(w, strategy=strategy, kD=1e-3 if strategy % 2 else 0.0, semantics=0 if semantics == "sim" else 1)
    R.step(1 / 60, 10, 2, 6)
    x = I.x if semantics == "sim" else I.x.astype(np.float64)
    assert rel_err(x.T, R.x, w["X"]) <= TOL


@pytest.mark.parametrize("formula", ["reference", "textbook"])
def test_chebyshev_beam_matches_oracle(formula):
    X, T = meshgen.hex_grid(16, 4, 4, hi=(4.0, 1.0, 1.0))
    dbc = meshgen.face_vertices(X, 0, 0.0)
    mu, lam = meshgen.lame(np.full(T.shape[0], 5e5), np.full(T.shape[0], 0.48))
    v = np.random.default_rng(1).uniform(-0.1, 0.1, X.shape)
    w = dict(X=X, T=T, dbc=dbc, rho=np.full(T.shape[0], 1000.0), mu=mu, lam=lam, v=v)
    I = pbat.sim.vbd.Integrator(make_data(w, rho=0.95, formula=formula))
    for _ in range(20):
        I.step(1 / 60, 30, 1)
    R = oracle_for(w, rho=0.95, formula=0 if formula == "reference" else 1)
    R.step(1 / 60, 30, 1, 20)
    assert rel_err(I.x.T, R.x, X) <= TOL


def test_small_beam_fixture_from_reference_kernels():
    g = np.load(GOLD / "trajectories.npz")
    X, T = meshgen.hex_grid(12, 3, 3, hi=(4.0, 1.0, 1.0))
    dbc = meshgen.face_vertices(X, 0, 0.0)
    mu, lam = meshgen.lame(np.full(T.shape[0], 5e5), np.full(T.shape[0], 0.48))
    w = dict(X=X, T=T, dbc=dbc, rho=np.full(T.shape[0], 1000.0), mu=mu, lam=lam, v=g["beam_v0"])
    I = pbat.sim.vbd.Integrator(make_data(w, strategy=3, kD=1e-3, rho=0.95))
    for _ in range(6):
        I.step(1 / 60, 15, 2)
    assert rel_err(I.x.T, g["beam_x"], X) <= TOL


def test_reference_cube_falls_and_only_falls():
    """gpu/impl/vbd/Integrator.cu:384-432 and sim/vbd/Integrator.cpp:245-293 on the device."""
    kat = json.loads((GOLD / "kat.json").read_text())["vbd_cube"]
    P, T, V, F = meshgen.cube5()
    for cheb in (None, kat["rho_chebyshev"]):
        d = pbat.sim.vbd.Data().with_volume_mesh(P, T).with_surface_mesh(V, F)
        if cheb:
            d = d.with_chebyshev_acceleration(cheb)
        d = d.construct()
        vbd = pbat.gpu.vbd.Integrator(d)
        vbd.scene_bounding_box = (P.min(axis=1), P.max(axis=1))
        xtilde = P + kat["dt"] * d.v + kat["dt"] ** 2 * d.aext
        vbd.step(kat["dt"], kat["iterations"], kat["substeps"])
        dx = vbd.x - P
        assert np.all(dx[2] < 0)
        assert np.all(np.abs(dx[:2]) < kat["zero"])
        # The objective decreased and the solution agrees with the FP64 oracle's, whose
        # gradient norm is below 1e-4.
        f = vbd.objective(kat["dt"])
        R = O.OracleVbd(P.T.copy(), T.T.copy(), np.full(5, 1000.0),
                        *meshgen.lame(np.full(5, 1e6), np.full(5, 0.45)), dbc=np.zeros(0, np.int32),
                        rho_chebyshev=cheb)
        f0 = R.objective(P.T.copy(), xtilde.T.copy(), kat["dt"])
        R.step(kat["dt"], kat["iterations"], kat["substeps"])
        assert f < f0
        np.testing.assert_allclose(vbd.x.T, R.x, atol=TOL * np.sqrt(3))


def test_objective_and_gradient_fp64_reductions_match_oracle():
    w = meshgen.unit_cube_workload(n=6)
    I = pbat.sim.vbd.Integrator(make_data(w))
    I.step(1 / 60, 5, 1)
    R = oracle_for(w)
    R.x = I.x.T.copy()
    xtilde = w["X"] + (1 / 60) * 0 + (1 / 60) ** 2 * R.aext
    f_gpu = I.objective(1 / 60)
    f_orc = R.objective(R.x, xtilde, 1 / 60)
    assert abs(f_gpu - f_orc) <= 1e-5 * abs(f_orc)
    g_gpu = I.gradient(1 / 60)
    g_orc = R.gradient(R.x, xtilde, 1 / 60)
    assert np.abs(g_gpu - g_orc).max() <= 1e-3 * np.abs(g_orc).max()


def test_objective_is_deterministic():
    """Fixed grid, fixed summation orders: repeated evaluations give the same bits."""
    w = meshgen.unit_cube_workload(n=12, seed=6)
    I = pbat.gpu.vbd.Integrator(make_data(w))
    I.step(1 / 60, 10, 1)
    f = [I.objective(1 / 60) for _ in range(8)]
    assert all(np.float64(v).tobytes() == np.float64(f[0]).tobytes() for v in f), f


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32])
def test_lanes_per_vertex_do_not_change_results(lanes):
    w = meshgen.unit_cube_workload(n=6, seed=4)
    I = pbat.sim.vbd.Integrator(make_data(w))
    I.lanes_per_vertex = lanes
    for _ in range(5):
        I.step(1 / 60, 10, 1)
    R = oracle_for(w)
    R.step(1 / 60, 10, 1, 5)
    assert rel_err(I.x.T, R.x, w["X"]) <= TOL


def test_batched_equals_individual_meshes():
    meshes = meshgen.batch_workload(n_meshes=5, nmin=3, nmax=7, seed=3)
    datas = [make_data(m) for m in meshes]
    B = pbat.gpu.vbd.BatchedIntegrator(datas)
    B.lanes_per_vertex = 4
    singles = []
    for d in datas:
        s = pbat.gpu.vbd.Integrator(d)
        s.lanes_per_vertex = 4
        singles.append(s)
    for _ in range(4):
        B.step(1 / 60, 10, 1)
        for s in singles:
            s.step(1 / 60, 10, 1)
    xb = B.x
    off = B.vertex_offsets
    for b, s in enumerate(singles):
        np.testing.assert_array_equal(xb[:, off[b]: off[b + 1]], s.x)
    # And each mesh matches its own oracle.
    for b, m in enumerate(meshes):
        R = oracle_for(m)
        R.step(1 / 60, 10, 1, 4)
        assert rel_err(xb[:, off[b]: off[b + 1]].T.astype(np.float64), R.x, m["X"]) <= TOL


def test_positions_velocities_roundtrip_and_external_acceleration():
    w = meshgen.unit_cube_workload(n=3)
    I = pbat.gpu.vbd.Integrator(make_data(w))
    x = np.asfortranarray(np.random.default_rng(0).standard_normal((3, w["X"].shape[0])).astype(np.float32))
    I.x = x
    np.testing.assert_array_equal(I.x, x)
    I.v = 2 * x
    np.testing.assert_array_equal(I.v, 2 * x)
    # Zero gravity, zero velocity, rest positions: nothing moves.
    I.x = w["X"].T
    I.v = np.zeros_like(x)
    I.a = np.zeros_like(x)
    I.step(1 / 60, 10, 1)
    np.testing.assert_allclose(I.x, w["X"].T, atol=1e-6)


def test_nonfinite_state_is_reported():
    w = meshgen.unit_cube_workload(n=3)
    I = pbat.gpu.vbd.Integrator(make_data(w))
    x = w["X"].T.astype(np.float32).copy()
    x[0, 5] = np.nan
    I.x = x
    I.step(1 / 60, 2, 1)
    with pytest.raises(_capi.PbgbError) as e:
        I.synchronize()
    assert e.value.code == 3
    # The flag is cleared once reported; the handle stays usable.
    I.x = w["X"].T
    I.v = np.zeros((3, w["X"].shape[0]), np.float32)
    I.step(1 / 60, 2, 1)
    I.synchronize()


def test_invalid_step_arguments():
    w = meshgen.unit_cube_workload(n=2)
    I = pbat.gpu.vbd.Integrator(make_data(w))
    with pytest.raises(_capi.PbgbError):
        I.step(-1.0, 10, 1)
    with pytest.raises(_capi.PbgbError):
        I.step(0.01, 10, 0)
    with pytest.raises(ValueError):
        I.x = np.zeros((3, 2))


def test_autotuner_restores_state_and_keeps_parity():
    w = meshgen.unit_cube_workload(n=5, seed=21)
    I = pbat.sim.vbd.Integrator(make_data(w, rho=0.9))
    I.step(1 / 60, 10, 1)
    x_before = I.x.copy()
    v_before = I.v.copy()
    lanes, block, ms = I.autotune(1 / 60, 10, 1)
    assert lanes in (1, 2, 4, 8, 16, 32) and block in (64, 96, 128, 160, 192, 224, 256) and ms > 0
    np.testing.assert_array_equal(I.x, x_before)
    np.testing.assert_array_equal(I.v, v_before)
    for _ in range(4):
        I.step(1 / 60, 10, 1)
    R = oracle_for(w, rho=0.9)
    R.step(1 / 60, 10, 1, 5)
    assert rel_err(I.x.T, R.x, w["X"]) <= TOL


def test_block_size_does_not_change_results():
    """Every vertex's arithmetic is independent of how the colour is cut into blocks: warp-multiple
    block sizes that are not powers of two (the autotuner's 96 ... 224) give the positions of
    block 256 bit for bit, with and without the staged sweep's shared-memory slabs."""
    w = meshgen.unit_cube_workload(n=8, seed=3)
    outs = {}
    for block in (256, 96, 160, 224):
        for lanes in (4, 8):
            I = pbat.sim.vbd.Integrator(make_data(w, rho=0.9))
            I.lanes_per_vertex = lanes
            _capi.check(_capi.lib().pbgb_vbd_set_block_size(I.handle, block), I.handle)
            for _ in range(3):
                I.step(1 / 60, 10, 1)
            outs[(block, lanes)] = I.x.copy()
    for (block, lanes), x in outs.items():
        np.testing.assert_array_equal(x, outs[(256, lanes)])


@pytest.mark.parametrize("pdl", [0, 1])
def test_programmatic_launch_does_not_change_results(pdl):
    w = meshgen.unit_cube_workload(n=6, seed=5)
    I = pbat.sim.vbd.Integrator(make_data(w, rho=0.9))
    _capi.check(_capi.lib().pbgb_vbd_set_programmatic_launch(I.handle, pdl), I.handle)
    for _ in range(5):
        I.step(1 / 60, 10, 1)
    R = oracle_for(w, rho=0.9)
    R.step(1 / 60, 10, 1, 5)
    assert rel_err(I.x.T, R.x, w["X"]) <= TOL


def _run_pair(make, steps, step):
    """Two integrators built by `make`, one with the staged sweep and one with the gathering sweep,
    advanced identically; returns both."""
    A, B = make(), make()
    assert A.staged_sweep == (True, True)
    B.staged_sweep = False
    for _ in range(steps):
        step(A)
        step(B)
    return A, B


@pytest.mark.parametrize("lanes", [1, 4, 32])
@pytest.mark.parametrize("mode", ["plain", "chebyshev", "damped_substeps"])
def test_staged_sweep_equals_gathering_sweep(mode, lanes):
    """Neighbours staged in shared memory: the same arithmetic in the same order as gathering
    every incidence's corners, hence the same positions bit for bit."""
    w = meshgen.unit_cube_workload(n=7, seed=9)
    kw = {"plain": {}, "chebyshev": {"rho": 0.9}, "damped_substeps": {"kD": 1e-3, "strategy": 3}}[mode]
    sub = 2 if mode == "damped_substeps" else 1

    def make():
        I = pbat.gpu.vbd.Integrator(make_data(w, **kw))
        I.lanes_per_vertex = lanes
        return I

    A, B = _run_pair(make, 4, lambda I: I.step(1 / 60, 10, sub))
    np.testing.assert_array_equal(A.x, B.x)
    np.testing.assert_array_equal(A.v, B.v)


def test_staged_sweep_batched_and_recorded():
    meshes = meshgen.batch_workload(n_meshes=4, nmin=3, nmax=6, seed=8)
    datas = [make_data(m, strategy=2) for m in meshes]
    A, B = _run_pair(lambda: pbat.gpu.vbd.BatchedIntegrator(datas), 3, lambda I: I.step(1 / 60, 8, 1))
    np.testing.assert_array_equal(A.x, B.x)
    # The recording sweep is staged too and still reproduces the unrecorded step.
    w = meshgen.unit_cube_workload(n=5, seed=2)
    C = pbat.gpu.vbd.Integrator(make_data(w, strategy=2))
    D = pbat.gpu.vbd.Integrator(make_data(w, strategy=2))
    D.adjoint_reserve(1, 9)
    for _ in range(3):
        C.step(1 / 60, 9, 1)
        D.step_record(1 / 60, 9, 1, 0)
    np.testing.assert_array_equal(C.x, D.x)
