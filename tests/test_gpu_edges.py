"""Edge cases of the VBD step on the device against the FP64 oracle: a single tetrahedron, a mesh
whose every vertex is pinned (no free vertex, no colour to sweep), zero iterations (the initial
guess alone) and a ragged batch (a one-tet mesh beside a cube)."""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

pytestmark = pytest.mark.gpu


def one_tet():
    X = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    T = np.array([[0, 1, 2, 3]])
    mu, lam = meshgen.lame(np.full(1, 1e6), np.full(1, 0.45))
    return dict(X=X, T=T, rho=np.full(1, 1000.0), mu=mu, lam=lam, dbc=np.array([0]), v=np.zeros_like(X))


def data_of(w, strategy=2):
    return (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
            .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(strategy).construct())


def oracle_of(w, strategy=2):
    return O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], strategy=strategy, semantics=1)


def test_single_tetrahedron_matches_oracle():
    w = one_tet()
    I = pbat.gpu.vbd.Integrator(data_of(w))
    R = oracle_of(w)
    for _ in range(10):
        I.step(1 / 60, 10, 1)
    R.step(1 / 60, 10, 1, 10)
    assert np.abs(I.x.T - R.x).max() / np.sqrt(3) <= 1e-4
    assert np.abs(I.x.T[0] - w["X"][0]).max() == 0.0  # the pinned vertex stays


def test_all_vertices_pinned():
    w = meshgen.unit_cube_workload(n=3, seed=2)
    w = dict(w, dbc=np.arange(w["X"].shape[0]))
    d = data_of(w)
    assert d.Padj.size == 0
    I = pbat.gpu.vbd.Integrator(d)
    for _ in range(3):
        I.step(1 / 60, 5, 2)
    np.testing.assert_array_equal(I.x.T, w["X"].astype(np.float32))
    np.testing.assert_array_equal(I.v, 0.0)


@pytest.mark.parametrize("strategy", [0, 1, 2])
def test_zero_iterations_give_the_initial_guess(strategy):
    w = meshgen.unit_cube_workload(n=4, seed=5)
    I = pbat.gpu.vbd.Integrator(data_of(w, strategy))
    R = oracle_of(w, strategy)
    for _ in range(2):
        I.step(1 / 60, 0, 1)
    R.step(1 / 60, 0, 1, 2)
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    assert np.abs(I.x.T - R.x).max() / diag <= 1e-6


def test_ragged_batch_equals_individual_meshes():
    meshes = [one_tet(), dict(meshgen.unit_cube_workload(n=5, seed=1), v=None), one_tet()]
    datas = [data_of(m) for m in meshes]
    B = pbat.gpu.vbd.BatchedIntegrator(datas)
    singles = [pbat.gpu.vbd.Integrator(d) for d in datas]
    B.lanes_per_vertex = 4
    for s in singles:
        s.lanes_per_vertex = 4
    for _ in range(3):
        B.step(1 / 60, 8, 1)
        for s in singles:
            s.step(1 / 60, 8, 1)
    off = B.vertex_offsets
    for b, s in enumerate(singles):
        np.testing.assert_array_equal(B.x[:, off[b]: off[b + 1]], s.x)
