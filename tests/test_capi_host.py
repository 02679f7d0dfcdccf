"""C-ABI surface and host-side logic of the product library (no GPU needed)."""

import ctypes as C
import pathlib
import re

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"PBGB_API\s+[\w\s\*]+?\b(pbgb_\w+)\s*\(", h.read_text()))
    return names


def test_library_exports_every_declared_symbol():
    L = _capi.lib()
    declared = declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    # The Python binding covers the whole header.
    assert declared == set(_capi.SYMBOLS)


def test_library_has_no_cpu_fallback_symbols():
    # The only compute entry point usable without a device is the documented host self-check.
    L = _capi.lib()
    h = C.c_void_p()
    d = _capi.VbdDesc()
    rc = L.pbgb_vbd_create(C.byref(d), C.byref(h))
    assert rc != 0


def _construct_product(X, T, rho, dbc, o=2, s=0):
    d = (pbat.sim.vbd.Data().with_volume_mesh(X.T, T.T).with_material(rho, np.ones_like(rho), np.ones_like(rho))
         .with_dirichlet_vertices(dbc).with_vertex_coloring_strategy(o, s).construct())
    return d


@pytest.mark.parametrize("n", [1, 3, 10])
def test_product_construct_matches_oracle(n):
    w = meshgen.unit_cube_workload(n=n, seed=n)
    for o in range(3):
        for s in range(2):
            d = _construct_product(w["X"], w["T"], w["rho"], w["dbc"], o, s)
            r = O.construct(w["X"], w["T"], w["rho"], w["dbc"], o, s)
            np.testing.assert_array_equal(d.colors, r["colors"])
            np.testing.assert_array_equal(d.Pptr, r["Pptr"])
            np.testing.assert_array_equal(d.Padj, r["Padj"])
            np.testing.assert_array_equal(d.GVGp, r["GVGp"])
            np.testing.assert_array_equal(d.GVGe, r["GVGe"])
            np.testing.assert_array_equal(d.GVGilocal, r["GVGilocal"])
            np.testing.assert_allclose(d.m, r["m"], rtol=1e-13)
            np.testing.assert_allclose(d.wg, r["wg"], rtol=1e-13)
            np.testing.assert_allclose(d._GP_rows.reshape(-1, 4, 3), r["GP"], rtol=1e-12, atol=1e-9)


def test_product_construct_reference_gp_layout():
    P, T, V, F = meshgen.cube5()
    d = pbat.sim.vbd.Data().with_volume_mesh(P, T).with_surface_mesh(V, F).construct()
    assert d.GP.shape == (4, 15)
    # Column 3e+k of GP holds d/dX_k of the 4 shape functions of element e.
    r = O.construct(P.T, T.T, np.full(5, 1000.0), np.zeros(0, np.int32))
    for e in range(5):
        np.testing.assert_allclose(d.GP[:, 3 * e: 3 * e + 3], r["GP"][e], atol=1e-14)
    assert d.XVA.shape == (8,) and d.FA.shape == (12,)
    assert abs(d.FA.sum() - 6.0) < 1e-12


def test_product_coloring_matches_reference_fixture():
    g = np.load(ROOT / "tests" / "golden" / "coloring.npz")
    X = meshgen.hex_grid(10, 10, 10)[0]
    T = g["cube10_T"]
    for o in range(3):
        for s in range(2):
            d = _construct_product(X, T, np.full(T.shape[0], 1000.0), np.zeros(0, np.int64), o, s)
            np.testing.assert_array_equal(d.colors, g[f"cube10_{o}_{s}"])


def test_construct_rejects_bad_meshes():
    X, T = meshgen.hex_grid(2, 2, 2)
    bad = T.copy()
    bad[0, [1, 2]] = bad[0, [2, 1]]  # inverted tet
    with pytest.raises(_capi.PbgbError) as e:
        _construct_product(X, bad, np.full(T.shape[0], 1000.0), np.zeros(0, np.int64))
    assert e.value.code == 4
    oob = T.copy()
    oob[3, 0] = X.shape[0] + 5
    with pytest.raises(_capi.PbgbError) as e:
        _construct_product(X, oob, np.full(T.shape[0], 1000.0), np.zeros(0, np.int64))
    assert e.value.code == 1
    with pytest.raises(_capi.PbgbError):
        _construct_product(X, T, np.full(T.shape[0], 1000.0), np.array([X.shape[0] + 1]))


def test_chebyshev_rho_validation():
    P, T, _, _ = meshgen.cube5()
    with pytest.raises(ValueError):
        pbat.sim.vbd.Data().with_volume_mesh(P, T).with_chebyshev_acceleration(1.0).construct()


def test_closed_form_vertex_block_matches_reference_fixture():
    """The device sweep's closed-form 3x3 block (host FP64 build of the same code) against the
    reference's full 9x9 SNH contraction."""
    g = np.load(ROOT / "tests" / "golden" / "vertex_solve.npz")
    L = _capi.lib()
    for c in range(int(g["count"])):
        a = {k.split("_", 1)[1]: g[k] for k in g.files if k.startswith(f"c{c}_")}
        x = a["x"].astype(np.float64).copy()
        gg = np.zeros(3)
        H = np.zeros(9)
        arrs = [np.ascontiguousarray(a[k]) for k in ("xe", "GPs")]
        il = np.ascontiguousarray(a["il"], dtype=np.int32)
        rc = L.pbgb_debug_vertex_block(int(a["n"]), arrs[0].ctypes.data, arrs[1].ctypes.data, il.ctypes.data,
                                       a["wg"].ctypes.data, a["mu"].ctypes.data, a["lam"].ctypes.data,
                                       a["xt"].ctypes.data, a["xtilde"].ctypes.data, float(a["m"]),
                                       float(a["kD"]), float(a["h"]), float(a["h"]) ** 2, 1e-7,
                                       x.ctypes.data, gg.ctypes.data, H.ctypes.data)
        assert rc == 0
        scale = np.abs(a["H"]).max()
        np.testing.assert_allclose(H.reshape(3, 3).T.ravel(), a["H"], rtol=1e-10, atol=1e-10 * scale)
        np.testing.assert_allclose(gg, a["g"], rtol=1e-8, atol=1e-9 * scale)
        np.testing.assert_allclose(x, a["x_out"], rtol=0, atol=1e-11)


def test_integrator_creation_without_device_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    P, T, _, _ = meshgen.cube5()
    d = pbat.sim.vbd.Data().with_volume_mesh(P, T).construct()
    with pytest.raises(_capi.PbgbError) as e:
        pbat.gpu.vbd.Integrator(d)
    assert e.value.code == 6


def _desc_with_contact(accel):
    """A GPU-semantics descriptor of the 5-tet cube with its surface mesh, acceleration forced."""
    from physicsbasedanimationtoolkit_gb300 import _integrator as I

    P, T, V, F = meshgen.cube5()
    d = pbat.sim.vbd.Data().with_volume_mesh(P, T).with_surface_mesh(V, F).construct()
    desc, keep = I.make_desc(d, I.SEMANTICS_GPU)
    assert desc.n_collision_triangles > 0
    desc.acceleration = accel
    return desc, keep


@pytest.mark.parametrize("accel,name", [(3, "Nesterov"), (4, "Broyden")])
def test_cpu_strategies_need_a_single_mesh_without_contact(accel, name):
    """Nesterov and Broyden are CPU-integrator strategies, whose integrator has no contact."""
    desc, keep = _desc_with_contact(accel)
    desc.nesterov_lipschitz = 1.0
    desc.window_size = 5
    h = C.c_void_p()
    rc = _capi.lib().pbgb_vbd_create(C.byref(desc), C.byref(h))
    assert rc == 1
    assert name in _capi.lib().pbgb_last_error(None).decode()


@pytest.mark.parametrize("accel", [2, 5])
def test_gpu_strategies_accept_contact(accel):
    """The reference's GPU integrator runs Anderson and the trust region with contact: the
    descriptor passes validation (creation then needs a device)."""
    desc, keep = _desc_with_contact(accel)
    desc.tr_eta, desc.tr_tau, desc.tr_curved = 0.2, 2.0, 0
    desc.window_size = 5
    h = C.c_void_p()
    rc = _capi.lib().pbgb_vbd_create(C.byref(desc), C.byref(h))
    if rc == 0:
        _capi.lib().pbgb_vbd_destroy(h)
    assert rc in (0, 6), _capi.lib().pbgb_last_error(None)


def test_cpu_integrator_has_no_contact():
    """sim/vbd/Integrator.cpp:98-136 has no contact terms: with CPU semantics the surface mesh
    does not turn contact on; with GPU semantics it does."""
    from physicsbasedanimationtoolkit_gb300 import _integrator as I

    P, T, V, F = meshgen.cube5()
    d = pbat.sim.vbd.Data().with_volume_mesh(P, T).with_surface_mesh(V, F).with_broyden_acceleration(5).construct()
    assert I.make_desc(d, I.SEMANTICS_CPU)[0].n_collision_triangles == 0
    assert I.make_desc(d, I.SEMANTICS_GPU)[0].n_collision_triangles > 0


@pytest.mark.parametrize("accel,cpu,gpu", [("none", 0, 0), ("chebyshev", 1, 1), ("anderson", 2, 2),
                                           ("nesterov", 3, 0), ("broyden", 4, 0), ("trust_region", 0, 5)])
def test_acceleration_dispatch_follows_the_reference(accel, cpu, gpu):
    """The CPU integrator runs Chebyshev, Anderson, Broyden and Nesterov and the base integrator
    otherwise; the GPU integrator runs Anderson, Chebyshev and trust region and the base
    integrator otherwise."""
    from physicsbasedanimationtoolkit_gb300 import _integrator as I

    P, T, _, _ = meshgen.cube5()
    d = pbat.sim.vbd.Data().with_volume_mesh(P, T)
    d = {"none": lambda: d, "chebyshev": lambda: d.with_chebyshev_acceleration(0.5),
         "anderson": lambda: d.with_anderson_acceleration(5), "nesterov": lambda: d.with_nesterov_acceleration(1.0, 3),
         "broyden": lambda: d.with_broyden_acceleration(5),
         "trust_region": lambda: d.with_trust_region_acceleration(0.2, 2.0, False)}[accel]().construct()
    for sem, want in ((I.SEMANTICS_CPU, cpu), (I.SEMANTICS_GPU, gpu)):
        if want is None:
            with pytest.raises(NotImplementedError):
                I.make_desc(d, sem)
        else:
            assert I.make_desc(d, sem)[0].acceleration == want


def test_trust_region_settings_are_validated():
    P, T, V, F = meshgen.cube5()
    with pytest.raises(ValueError):
        pbat.sim.vbd.Data().with_volume_mesh(P, T).with_trust_region_acceleration(-0.1, 2.0, False).construct()
    with pytest.raises(ValueError):
        pbat.sim.vbd.Data().with_volume_mesh(P, T).with_trust_region_acceleration(0.2, 1.0, True).construct()


def _cube_data():
    w = meshgen.unit_cube_workload(n=3, seed=1)
    return (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
            .with_dirichlet_vertices(w["dbc"]).construct())


@pytest.mark.parametrize("defect", ["colouring", "duplicate", "nan_x", "zero_wg", "negative_lambda"])
def test_descriptor_errors_are_reported_without_a_device(defect):
    """Host validation runs before the device query, so a bad descriptor is an invalid argument
    (with its message) whether or not a GPU is present."""
    d = _cube_data()
    if defect == "colouring":
        # Move a vertex into the colour of one of its neighbours.
        ptr, adj = d.Pptr.copy(), d.Padj.copy()
        T = np.asarray(d.E).T
        v = int(adj[ptr[0]])
        nb = next(int(u) for t in T if v in t for u in t if u != v and u in adj[ptr[1]:ptr[2]])
        k = int(np.nonzero(adj == nb)[0][0])
        adj[k] = v
        adj[ptr[0]] = nb
        d.Padj = adj
        expect = "invalid colouring"
    elif defect == "duplicate":
        adj = d.Padj.copy()
        adj[1] = adj[0]
        d.Padj = adj
        expect = "more than one partition"
    elif defect == "nan_x":
        x = np.array(d.x, dtype=np.float64)
        x[0, 3] = np.nan
        d.x = x
        expect = "non-finite"
    elif defect == "zero_wg":
        wg = d.wg.copy()
        wg[2] = 0.0
        d.wg = wg
        expect = "quadrature weights"
    else:
        lame = np.array(d.lame, dtype=np.float64)
        lame[1, 0] = -1.0
        d.lame = lame
        expect = "Lame"
    with pytest.raises(_capi.PbgbError) as e:
        pbat.gpu.vbd.Integrator(d)
    assert e.value.code == 1, e.value
    assert expect in str(e.value)


def test_nesterov_settings_are_validated():
    P, T, _, _ = meshgen.cube5()
    with pytest.raises(ValueError):
        pbat.sim.vbd.Data().with_volume_mesh(P, T).with_nesterov_acceleration(0.0, 3).construct()
    with pytest.raises(ValueError):
        pbat.sim.vbd.Data().with_volume_mesh(P, T).with_nesterov_acceleration(1.0, -1).construct()


def test_bvh_queries_validate_arguments_before_the_device():
    """The LBVH query entry points refuse bad arguments with PBGB_ERR_INVALID_ARGUMENT before any
    device work: null handles, simplices indexing past the points, unsupported simplex sizes."""
    L = _capi.lib()
    count = C.c_int64()
    assert L.pbgb_bvh_self_overlaps(None, None, None, 0, C.byref(count)) == 1
    assert L.pbgb_bvh_nearest_simplices(None, 0, None, 0, None, 0, None, 3, None) == 1
    assert L.pbgb_bvh_visits(None, None) == 1
    P = np.zeros((4, 3), np.float32)
    S = np.array([[0, 1, 2], [1, 2, 7]], np.int32)  # index 7 is past the 4 points
    lo = np.zeros((2, 3), np.float32)
    hi = np.zeros((2, 3), np.float32)
    rc = L.pbgb_simplex_boxes(4, P.ctypes.data, 2, S.ctypes.data, 3, lo.ctypes.data, hi.ctypes.data)
    assert rc == 1 and b"out of range" in L.pbgb_bvh_last_error(None)
    rc = L.pbgb_simplex_boxes(4, P.ctypes.data, 2, S.ctypes.data, 5, lo.ctypes.data, hi.ctypes.data)
    assert rc == 1
    with pytest.raises(ValueError):
        pbat.gpu.geometry.Aabb(2, 4)
    with pytest.raises(ValueError):
        pbat.gpu.geometry.Aabb(3, 0).construct(np.zeros((3, 4), np.float32), np.zeros((5, 2), np.int32))
