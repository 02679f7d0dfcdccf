"""The persistent batched step: one launch per step, each mesh advancing through its own colours.

Its positions must equal, bit for bit, those of the colour-launch batch and of one single-mesh
integrator per mesh (the per-vertex arithmetic, its order and the lanes are the same), and match
the FP64 oracle per mesh; a bounded wait that is made to run out must end the step with
PBGB_ERR_TIMEOUT and leave the context usable."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

pytestmark = pytest.mark.gpu

TOL = 1e-4


def make_datas(meshes, rho=None):
    out = []
    for m in meshes:
        d = (pbat.sim.vbd.Data().with_volume_mesh(m["X"].T, m["T"].T).with_material(m["rho"], m["mu"], m["lam"])
             .with_dirichlet_vertices(m["dbc"]))
        if rho is not None:
            d = d.with_chebyshev_acceleration(rho)
        out.append(d.construct())
    return out


@pytest.mark.parametrize("rho", [None, 0.9])
@pytest.mark.parametrize("lanes,block,tile", [(1, 64, 1), (2, 128, 1), (4, 224, 2), (8, 256, 3), (32, 256, 1)])
def test_persistent_equals_colour_launches_and_single_meshes(rho, lanes, block, tile):
    meshes = meshgen.batch_workload(n_meshes=9, nmin=2, nmax=9, seed=lanes + block)
    datas = make_datas(meshes, rho)
    P = pbat.gpu.vbd.BatchedIntegrator(datas)
    U = pbat.gpu.vbd.BatchedIntegrator(datas)
    for I in (P, U):
        I.lanes_per_vertex = lanes
        _capi.check(_capi.lib().pbgb_vbd_set_block_size(I.handle, block), I.handle)
    P.batch_tile = tile
    U.persistent = False
    assert P.persistent and not U.persistent
    singles = []
    for d in datas:
        s = pbat.gpu.vbd.Integrator(d)
        s.lanes_per_vertex = lanes
        _capi.check(_capi.lib().pbgb_vbd_set_block_size(s.handle, block), s.handle)
        singles.append(s)
    for _ in range(3):
        for I in (P, U, *singles):
            I.step(1 / 60, 7, 2)
    P.synchronize()
    assert P.launches_per_step(7, 2) == 1
    xp, xu = P.x, U.x
    np.testing.assert_array_equal(xp, xu)
    np.testing.assert_array_equal(P.v, U.v)
    off = P.vertex_offsets
    for b, s in enumerate(singles):
        np.testing.assert_array_equal(xp[:, off[b]: off[b + 1]], s.x)


def test_persistent_batch_matches_oracle_per_mesh():
    meshes = meshgen.batch_workload(n_meshes=12, nmin=3, nmax=10, seed=21)
    B = pbat.gpu.vbd.BatchedIntegrator(make_datas(meshes))
    assert B.persistent
    for _ in range(5):
        B.step(1 / 60, 20, 1)
    x = B.x
    off = B.vertex_offsets
    for b, m in enumerate(meshes):
        R = O.OracleVbd(m["X"], m["T"], m["rho"], m["mu"], m["lam"], m["dbc"], v=m["v"], strategy=4, semantics=1)
        R.step(1 / 60, 20, 1, 5)
        diag = np.linalg.norm(m["X"].max(0) - m["X"].min(0))
        assert np.abs(x[:, off[b]: off[b + 1]].T.astype(np.float64) - R.x).max() / diag <= TOL


def test_a_batch_of_one_mesh_uses_colour_launches():
    w = meshgen.unit_cube_workload(n=3)
    d = make_datas([dict(X=w["X"], T=w["T"], rho=w["rho"], mu=w["mu"], lam=w["lam"], dbc=w["dbc"])])
    S = pbat.gpu.vbd.BatchedIntegrator(d)  # a batch of one mesh: colour launches
    assert not S.persistent


def test_a_wait_that_runs_out_reports_a_timeout_and_the_context_survives():
    """One work item's requirement is made unreachable (a counter that nothing raises far
    enough) with a 1 ms limit: the step ends, the next synchronizing call reports
    PBGB_ERR_TIMEOUT, and after the hook is cleared the same step from the same state gives the
    same positions as a batch that never timed out."""
    meshes = meshgen.batch_workload(n_meshes=6, nmin=3, nmax=6, seed=2)
    datas = make_datas(meshes)
    A = pbat.gpu.vbd.BatchedIntegrator(datas)
    Ref = pbat.gpu.vbd.BatchedIntegrator(datas)
    x0, v0 = A.x.copy(), A.v.copy()
    L = _capi.lib()
    # Item 40 lies in the first iteration's colour sweeps (6 meshes: 6 begin items come first).
    _capi.check(L.pbgb_debug_batched_wait(A.handle, 1_000_000, 40), A.handle)
    A.step(1 / 60, 10, 1)
    with pytest.raises(_capi.PbgbError) as err:
        A.synchronize()
    assert err.value.code == 7
    # The flag was cleared by the report; the context still works.
    _capi.check(L.pbgb_debug_batched_wait(A.handle, 2_000_000_000, -1), A.handle)
    A.x, A.v = x0, v0
    A.step(1 / 60, 10, 1)
    A.synchronize()
    Ref.step(1 / 60, 10, 1)
    np.testing.assert_array_equal(A.x, Ref.x)


def test_debug_hook_rejects_out_of_range_limits():
    meshes = meshgen.batch_workload(n_meshes=2, nmin=2, nmax=3, seed=1)
    B = pbat.gpu.vbd.BatchedIntegrator(make_datas(meshes))
    L = _capi.lib()
    assert L.pbgb_debug_batched_wait(B.handle, 10, -1) == 1
    assert L.pbgb_debug_batched_wait(B.handle, 5_000_000_000, -1) == 1
    assert L.pbgb_debug_batched_wait(B.handle, 1_000_000, -2) == 1

