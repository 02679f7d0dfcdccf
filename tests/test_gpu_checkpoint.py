"""Checkpoint / resume of the step state: a second handle built from the same data that loads a
saved state continues bit for bit."""

import numpy as np
import pytest

from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

pytestmark = pytest.mark.gpu


def test_resume_plain_and_adaptive_guess():
    w = meshgen.unit_cube_workload(n=5, seed=7)
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
         .with_dirichlet_vertices(w["dbc"]).with_initialization_strategy(3).construct())
    A = pbat.gpu.vbd.Integrator(d)  # GPU semantics: AdaptiveVbd reads the previous step's velocity
    for _ in range(3):
        A.step(1 / 60, 10, 1)
    blob = A.save_state()
    for _ in range(4):
        A.step(1 / 60, 10, 1)
    B = pbat.gpu.vbd.Integrator(d)
    B.load_state(blob)
    for _ in range(4):
        B.step(1 / 60, 10, 1)
    np.testing.assert_array_equal(A.x, B.x)
    np.testing.assert_array_equal(A.v, B.v)


def test_resume_with_contact_state():
    w = meshgen.contact_scene_workload(n_cubes_side=2, cube_hexes=3, slab_hexes=(8, 8, 1), gap=0.01)
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
         .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
         .with_contact_parameters(1e7, 0.3, 1e-3).with_initialization_strategy(2).construct())
    A = pbat.gpu.vbd.Integrator(d)
    for _ in range(12):
        A.step(1 / 60, 15, 1)
    blob = A.save_state()
    for _ in range(5):
        A.step(1 / 60, 15, 1)
    B = pbat.gpu.vbd.Integrator(d)
    B.load_state(blob)
    for _ in range(5):
        B.step(1 / 60, 15, 1)
    np.testing.assert_array_equal(A.x, B.x)
    fa, aa = A.contacts()
    fb, ab = B.contacts()
    np.testing.assert_array_equal(fa, fb)
    np.testing.assert_array_equal(aa, ab)


def test_state_of_another_system_is_rejected():
    a = meshgen.unit_cube_workload(n=3)
    b = meshgen.unit_cube_workload(n=4)
    mk = lambda w: pbat.gpu.vbd.Integrator(
        pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
        .with_dirichlet_vertices(w["dbc"]).construct())
    A, B = mk(a), mk(b)
    with pytest.raises(_capi.PbgbError) as e:
        B.load_state(A.save_state())
    assert e.value.code == 1
