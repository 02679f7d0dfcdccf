"""Trust-region accelerated VBD on the device (gpu/impl/vbd/TrustRegionIntegrator.cu) against the
FP64 oracle restatement of the same iteration."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

pytestmark = pytest.mark.gpu


def data_for(w, tr=None, strategy=2):
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
         .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(strategy))
    if tr is not None:
        d = d.with_trust_region_acceleration(*tr)
    return d.construct()


@pytest.mark.parametrize("eta,tau", [(0.2, 2.0), (0.1, 2.0), (0.5, 1.5), (0.0, 4.0)])
def test_linear_path_matches_oracle_on_the_device_decisions(eta, tau):
    """The oracle replays the device's logged decisions (step lengths, tries, acceptances): the
    positions then agree within 1e-4 of the bounding-box diagonal over 8 steps of 15 iterations.
    This pins every kernel's arithmetic independently of how close the decisions themselves are
    (see the trajectory test below)."""
    w = meshgen.unit_cube_workload(n=7, seed=3)
    I = pbat.gpu.vbd.Integrator(data_for(w, (eta, tau, False)))
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2, semantics=1,
                    trust_region=(eta, tau, False))
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    tried = 0
    for _ in range(8):
        I.step(1 / 60, 15, 1)
        log = I.trust_region_log()
        assert log.shape == (15, 4)
        flags = log[:, 3].astype(int)
        assert set(flags[:2]) == {0} and set(flags) <= {0, 1, 3}
        assert np.all(np.isnan(log[flags == 0, 1])) and np.all(log[flags > 0, 0] > 1.0)
        tried += int((flags > 0).sum())
        R.step(1 / 60, 15, 1, 1, trust_region_log=log)
        err = np.abs(I.x.T - R.x).max() / diag
        assert err <= 1e-4, err
    assert tried > 0


def test_linear_path_trajectory_follows_oracle():
    """Free-running trajectories (8 steps of 15 iterations at the reference's defaults eta 0.2,
    tau 2), each side taking its own decisions, agree within 1e-3 of the diagonal.  The bound is
    looser than the replay test's because the step length t* = -b / 2a comes from a quadratic fit
    through objective values whose differences are ~1e-7 of f: a 1e-10 relative change of f moves
    t* by ~1e-4, and FP32 iterates alone differ from FP64 ones by more than that, so the two sides'
    step lengths drift apart by 1e-4..1e-1 relative over a step (measured on this cube) and
    positions by ~2e-4 of the diagonal after 8 steps.  The FP64 oracle itself moves by up to 6e-4
    under a 1e-8 relative perturbation of its objective (eta 0.1)."""
    w = meshgen.unit_cube_workload(n=7, seed=3)
    I = pbat.gpu.vbd.Integrator(data_for(w, (0.2, 2.0, False)))
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2, semantics=1,
                    trust_region=(0.2, 2.0, False))
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    for _ in range(8):
        I.step(1 / 60, 15, 1)
    R.step(1 / 60, 15, 1, 8)
    err = np.abs(I.x.T - R.x).max() / diag
    assert err <= 1e-3, err


def test_beam_with_substeps_matches_oracle():
    X, T = meshgen.hex_grid(12, 3, 3, hi=(4.0, 1.0, 1.0))
    nT = T.shape[0]
    mu, lam = meshgen.lame(np.full(nT, 5e5), np.full(nT, 0.48))
    w = dict(X=X, T=T, dbc=meshgen.face_vertices(X, 0, 0.0), rho=np.full(nT, 1000.0), mu=mu, lam=lam)
    I = pbat.gpu.vbd.Integrator(data_for(w, (0.2, 2.0, False)))
    R = O.OracleVbd(X, T, w["rho"], mu, lam, w["dbc"], strategy=2, semantics=1, trust_region=(0.2, 2.0, False))
    for _ in range(6):
        I.step(1 / 60, 12, 2)
    R.step(1 / 60, 12, 2, 6)
    diag = np.linalg.norm(X.max(0) - X.min(0))
    assert np.abs(I.x.T - R.x).max() / diag <= 1e-4


def test_curved_path_moves_like_plain_vbd():
    """The curved path's constraint solve returns 0 (TrustRegionIntegrator.cu:700-703), so it never
    tries an accelerated step: its positions are the plain VBD iterates, bit for bit."""
    w = meshgen.unit_cube_workload(n=6, seed=2)
    A = pbat.gpu.vbd.Integrator(data_for(w, (0.2, 2.0, True)))
    B = pbat.gpu.vbd.Integrator(data_for(w))
    for _ in range(4):
        A.step(1 / 60, 12, 1)
        B.step(1 / 60, 12, 1)
    np.testing.assert_array_equal(A.x, B.x)
    np.testing.assert_array_equal(A.v, B.v)


def test_cpu_integrator_runs_plain_vbd_for_trust_region():
    """The reference's CPU integrator builds the base integrator for trust-region data."""
    w = meshgen.unit_cube_workload(n=5, seed=1)
    A = pbat.sim.vbd.Integrator(data_for(w, (0.2, 2.0, False)))
    B = pbat.sim.vbd.Integrator(data_for(w))
    for _ in range(3):
        A.step(1 / 60, 10, 1)
        B.step(1 / 60, 10, 1)
    np.testing.assert_array_equal(A.x, B.x)


def test_linear_path_lowers_the_objective_further_than_plain_vbd():
    """At equal iterations (one step of 40) the accelerated solve ends at a lower objective than
    plain VBD, on the device as in the oracle."""
    w = meshgen.unit_cube_workload(n=8, seed=1)
    dt = 1 / 60

    def device(tr):
        I = pbat.gpu.vbd.Integrator(data_for(w, tr))
        I.step(dt, 40, 1)
        return I.objective(dt)

    def oracle(tr):
        R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=2, semantics=1,
                        **({"trust_region": tr} if tr else {}))
        xtilde = R.x + dt * R.v + dt * dt * R.aext
        R.step(dt, 40, 1, 1)
        return R.objective(R.x, xtilde, dt)

    gain_device = device(None) - device((0.2, 2.0, False))
    gain_oracle = oracle(None) - oracle((0.2, 2.0, False))
    assert gain_oracle > 0
    assert gain_device > 0.5 * gain_oracle


def test_step_graph_replays_identically():
    """All decisions are taken on the device: two integrators replaying the same captured step
    produce the same positions, bit for bit."""
    w = meshgen.unit_cube_workload(n=6, seed=5)
    A = pbat.gpu.vbd.Integrator(data_for(w, (0.2, 2.0, False)))
    B = pbat.gpu.vbd.Integrator(data_for(w, (0.2, 2.0, False)))
    for _ in range(5):
        A.step(1 / 60, 15, 1)
        B.step(1 / 60, 15, 1)
    np.testing.assert_array_equal(A.x, B.x)
