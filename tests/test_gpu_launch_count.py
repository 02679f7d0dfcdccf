"""The launch count each integrator claims for a step (pbgb_vbd_launches_per_step, the source of the
benchmark's gpu_launches) against the kernel nodes of the CUDA graph the step actually captured."""

import pytest

from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

pytestmark = pytest.mark.gpu


def cube_data(acceleration=None, n=4, seed=0):
    w = meshgen.unit_cube_workload(n=n, seed=seed)
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
         .with_dirichlet_vertices(w["dbc"]))
    if acceleration == "chebyshev":
        d = d.with_chebyshev_acceleration(0.9)
    elif acceleration == "anderson":
        d = d.with_anderson_acceleration(4)
    elif acceleration == "trust_region":
        d = d.with_trust_region_acceleration(0.2, 2.0, False)
    return d.construct()


def contact_data():
    w = meshgen.contact_scene_workload(n_cubes_side=2, cube_hexes=3, slab_hexes=(8, 8, 1), gap=0.01)
    return (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
            .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
            .with_contact_parameters(1e7, 0.3, 1e-3).with_initialization_strategy(2).construct())


def check(I, iterations, substeps):
    assert I.step_graph_kernels() == -1
    I.step(1 / 60, iterations, substeps)
    I.synchronize()
    assert I.step_graph_kernels() == I.launches_per_step(iterations, substeps)


@pytest.mark.parametrize("acceleration", [None, "chebyshev", "anderson", "trust_region"])
@pytest.mark.parametrize("iterations,substeps", [(1, 1), (7, 2)])
def test_single_mesh(acceleration, iterations, substeps):
    check(pbat.gpu.vbd.Integrator(cube_data(acceleration)), iterations, substeps)


@pytest.mark.parametrize("substeps", [1, 3])
def test_contact(substeps):
    check(pbat.gpu.vbd.Integrator(contact_data()), 6, substeps)


@pytest.mark.parametrize("persistent", [True, False])
def test_batch(persistent):
    B = pbat.gpu.vbd.BatchedIntegrator([cube_data(n=n, seed=n) for n in (2, 5, 3, 4)])
    B.persistent = persistent
    check(B, 5, 2)
