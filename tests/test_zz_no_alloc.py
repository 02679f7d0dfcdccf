"""The allocation-free gradient entry point (pbgb_vbd_gradient_noalloc).

Callers whose device memory is owned by another runtime, or whose frame loop must not allocate
after start-up, use this variant: it accumulates in a fixed device array built into the library
instead of allocating a buffer.  Its result must equal that of pbgb_vbd_gradient, on repeated
calls too (the shared array keeps the previous call's contents and must be cleared each time),
and a call must leave the device's free memory unchanged.

This file is collected last on purpose; it passes alone in a fresh process as well.
"""

import ctypes as C

import numpy as np
import pytest

from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

pytestmark = pytest.mark.gpu


def _data(n=6, extra_pinned=0, seed=9):
    w = meshgen.unit_cube_workload(n=n, seed=seed)
    X, T, dbc = w["X"], w["T"], w["dbc"]
    if extra_pinned:
        # Unconnected, pinned vertices: they enlarge the vertex count without any tets.
        far = 10.0 + np.random.default_rng(0).uniform(0.0, 1.0, (extra_pinned, 3))
        dbc = np.concatenate([dbc, np.arange(X.shape[0], X.shape[0] + extra_pinned)])
        X = np.vstack([X, far])
    return (pbat.sim.vbd.Data().with_volume_mesh(X.T, T.T).with_material(w["rho"], w["mu"], w["lam"])
            .with_dirichlet_vertices(dbc).with_chebyshev_acceleration(0.9).construct())


def _integrator(n=6, extra_pinned=0):
    return pbat.gpu.vbd.Integrator(_data(n, extra_pinned))


def _noalloc_gradient(I, dt):
    g = np.full(3 * I.n_vertices, np.nan)
    rc = _capi.lib().pbgb_vbd_gradient_noalloc(I.handle, C.c_double(dt), g.ctypes.data)
    _capi.check(rc, I.handle)
    return g


def test_gradient_without_allocation_matches_the_allocating_entry_point():
    dt = 1 / 60
    I = _integrator()
    for step in range(2):
        I.step(dt, 10, 1)
        expected = I.gradient(dt)
        scale = np.abs(expected).max()
        assert scale > 0
        # Two calls in a row: the second must not see the first one's accumulators.
        for _ in range(2):
            g = _noalloc_gradient(I, dt)
            np.testing.assert_allclose(g, expected, rtol=1e-9, atol=1e-12 * scale)


def test_a_call_leaves_device_memory_unchanged():
    """On a fresh handle that never called the allocating entry point: after one warm-up call
    (which loads the gradient kernel's code), a second call changes the device's free memory by
    nothing."""
    torch = pytest.importorskip("torch")
    dt = 1 / 60
    I = _integrator(n=7)
    I.step(dt, 10, 1)
    g0 = _noalloc_gradient(I, dt)
    I.synchronize()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    g1 = _noalloc_gradient(I, dt)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    np.testing.assert_array_equal(np.isfinite(g1), np.ones_like(g1, bool))
    np.testing.assert_allclose(g1, g0, rtol=1e-9, atol=1e-12 * np.abs(g0).max())
    # Only now the allocating entry point, for the comparison.
    expected = I.gradient(dt)
    np.testing.assert_allclose(g1, expected, rtol=1e-9, atol=1e-12 * np.abs(expected).max())


def test_ragged_batch_matches_the_allocating_entry_point():
    """A batched handle of meshes of different sizes (one system of concatenated vertices)."""
    dt = 1 / 60
    B = pbat.gpu.vbd.BatchedIntegrator([_data(n=3, seed=1), _data(n=6, seed=2), _data(n=4, seed=3)])
    B.step(dt, 8, 1)
    B.synchronize()
    for _ in range(2):
        g = np.full(3 * B.n_vertices, np.nan)
        _capi.check(_capi.lib().pbgb_vbd_gradient_noalloc(B.handle, C.c_double(dt), g.ctypes.data), B.handle)
        expected = np.zeros(3 * B.n_vertices)
        _capi.check(_capi.lib().pbgb_vbd_gradient(B.handle, C.c_double(dt), expected.ctypes.data), B.handle)
        np.testing.assert_allclose(g, expected, rtol=1e-9, atol=1e-12 * np.abs(expected).max())


def test_meshes_beyond_the_fixed_scratch_are_rejected():
    I = _integrator(n=2, extra_pinned=262_200)
    assert I.n_vertices > 262_144
    g = np.zeros(3 * I.n_vertices)
    rc = _capi.lib().pbgb_vbd_gradient_noalloc(I.handle, C.c_double(1 / 60), g.ctypes.data)
    assert rc == 1
    assert b"262144" in _capi.lib().pbgb_last_error(I.handle)
    # The allocating entry point still serves it.
    assert np.isfinite(I.gradient(1 / 60)).all()
