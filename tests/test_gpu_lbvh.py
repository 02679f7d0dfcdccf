"""GPU LBVH against the oracle: Morton codes, sort order, topology and internal boxes bit-exact;
overlap pair sets equal to brute force."""

import json
import pathlib

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

pytestmark = pytest.mark.gpu

GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def gpu_build(lo, hi, wmin, wmax):
    bvh = pbat.gpu.geometry.Bvh(lo.shape[0], 0)
    bvh.build(lo.T, hi.T, wmin, wmax)
    return bvh, bvh._topology()


def assert_same(g, o):
    np.testing.assert_array_equal(g["codes"], o["codes"])
    np.testing.assert_array_equal(g["inds"], o["inds"])
    np.testing.assert_array_equal(g["child"], o["child"])
    np.testing.assert_array_equal(g["parent"], o["parent"])
    np.testing.assert_array_equal(g["rightmost"], o["rightmost"])
    np.testing.assert_array_equal(g["ilo"], o["ilo"])
    np.testing.assert_array_equal(g["ihi"], o["ihi"])


def test_cube_topology_known_answer_on_device():
    kat = json.loads((GOLD / "kat.json").read_text())["bvh_cube5"]
    P, T, _, _ = meshgen.cube5()
    X = P.T.astype(np.float32)
    pts = X[T.T]
    lo, hi = pts.min(axis=1), pts.max(axis=1)
    _, g = gpu_build(lo, hi, X.min(axis=0), X.max(axis=0))
    np.testing.assert_array_equal(g["child"], np.array(kat["child"]))
    np.testing.assert_array_equal(g["parent"], np.array(kat["parent"]))
    np.testing.assert_array_equal(g["rightmost"], np.array(kat["rightmost"]))


def test_morton_codes_match_reference_fixture_on_device():
    g = np.load(GOLD / "morton.npz")
    _, t = gpu_build(g["lo"], g["hi"], g["wmin"], g["wmax"])
    expected = np.sort(g["codes"], kind="stable")
    np.testing.assert_array_equal(t["codes"], expected)
    np.testing.assert_array_equal(t["inds"], np.argsort(g["codes"], kind="stable"))


def scene_boxes(swept):
    w = meshgen.contact_scene_workload()
    X = w["X"].astype(np.float32)
    Xn = None
    if swept:
        Xn = (X + np.random.default_rng(1).uniform(-0.01, 0.01, X.shape) + np.array([0, 0, -0.02])).astype(np.float32)
    lo, hi = meshgen.triangle_boxes(X, w["F"], Xn)
    lo, hi = lo.astype(np.float32), hi.astype(np.float32)
    allp = X if Xn is None else np.vstack([X, Xn])
    return w, lo, hi, allp.min(axis=0), allp.max(axis=0)


@pytest.mark.parametrize("swept", [False, True])
def test_scene_triangle_bvh_bit_exact(swept):
    """66,560 surface triangles of the 16-cube contact scene."""
    w, lo, hi, wmin, wmax = scene_boxes(swept)
    assert lo.shape[0] == 66560
    _, g = gpu_build(lo, hi, wmin, wmax)
    o = O.bvh_build(lo, hi, wmin, wmax)
    assert_same(g, o)


@pytest.mark.parametrize("n", [2, 3, 1000, 1024, 1025, 2049, 200_000, 1_100_000])
def test_random_boxes_with_duplicate_codes(n):
    rng = np.random.default_rng(n)
    lo = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    hi = (lo + rng.uniform(0, 0.01, (n, 3))).astype(np.float32)
    lo[: n // 3] = lo[n // 3: 2 * (n // 3)]
    hi[: n // 3] = hi[n // 3: 2 * (n // 3)]
    _, g = gpu_build(lo, hi, [0, 0, 0], [1.01, 1.01, 1.01])
    assert_same(g, O.bvh_build(lo, hi, [0, 0, 0], [1.01, 1.01, 1.01]))


def test_overlap_pairs_equal_brute_force():
    w, lo, hi, wmin, wmax = scene_boxes(True)
    X = w["X"].astype(np.float32)
    rng = np.random.default_rng(7)
    V = w["V"][rng.choice(w["V"].size, 4000, replace=False)]
    Xn = X + np.array([0, 0, -0.03], np.float32)
    qlo = np.minimum(X[V], Xn[V])
    qhi = np.maximum(X[V], Xn[V])
    bvh, _ = gpu_build(lo, hi, wmin, wmax)
    got = bvh.overlaps(qlo.T, qhi.T)
    exp = O.overlaps(lo, hi, qlo, qhi)
    assert exp.shape[0] > 1000
    assert {tuple(p) for p in got.T} == {tuple(p) for p in exp}
    assert got.shape[1] == exp.shape[0]


def test_refit_matches_oracle_boxes_for_same_topology():
    w, lo, hi, wmin, wmax = scene_boxes(False)
    bvh, g0 = gpu_build(lo, hi, wmin, wmax)
    X = w["X"].astype(np.float32) + np.random.default_rng(3).uniform(-0.02, 0.02, w["X"].shape).astype(np.float32)
    lo2, hi2 = meshgen.triangle_boxes(X, w["F"])
    lo2, hi2 = lo2.astype(np.float32), hi2.astype(np.float32)
    bvh.refit(lo2.T, hi2.T)
    g = bvh._topology()
    np.testing.assert_array_equal(g["child"], g0["child"])
    ilo, ihi = O.bvh_boxes(g["child"], g["inds"], lo2, hi2)
    np.testing.assert_array_equal(g["ilo"], ilo)
    np.testing.assert_array_equal(g["ihi"], ihi)


def test_build_from_device_boxes_equals_host_build():
    """pbgb_bvh_build_device (boxes already on the device) gives the same codes, order, topology
    and boxes as the host-buffer build, and both equal the oracle."""
    import ctypes as C

    import torch

    from physicsbasedanimationtoolkit_gb300 import _capi

    rng = np.random.default_rng(21)
    n = 20000
    c = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    e = rng.uniform(0, 0.01, (n, 3)).astype(np.float32)
    lo, hi = (c - e).astype(np.float32), (c + e).astype(np.float32)
    wmin, wmax = np.zeros(3, np.float32), np.ones(3, np.float32)
    bvh, host = gpu_build(lo, hi, wmin, wmax)
    lo4 = torch.zeros((n, 4), device="cuda")
    hi4 = torch.zeros((n, 4), device="cuda")
    lo4[:, :3] = torch.from_numpy(lo).cuda()
    hi4[:, :3] = torch.from_numpy(hi).cuda()
    torch.cuda.synchronize()
    L = _capi.lib()
    _capi.check_bvh(L.pbgb_bvh_build_device(bvh._h, n, C.c_void_p(lo4.data_ptr()), C.c_void_p(hi4.data_ptr()),
                                            wmin.ctypes.data, wmax.ctypes.data), bvh._h)
    dev = bvh._topology()
    assert_same(dev, host)
    assert_same(dev, O.bvh_build(lo, hi, wmin, wmax))


# ---------------------------------------------------------------------------------------------
# The reference binding's remaining queries (bindings/pypbat/gpu/geometry/Bvh.cpp, Aabb.cpp).

def _brute_self_overlaps(lo, hi, sets=None):
    """Unordered pairs {i, j}, i != j, of closed boxes that overlap (numpy, exact comparisons)."""
    ov = np.all((lo[:, None, :] <= hi[None, :, :]) & (lo[None, :, :] <= hi[:, None, :]), axis=2)
    i, j = np.nonzero(np.triu(ov, 1))
    keep = np.ones(i.size, bool) if sets is None else sets[i] != sets[j]
    return {frozenset((a, b)) for a, b in zip(i[keep].tolist(), j[keep].tolist())}


def test_detect_overlaps_between_sets_reference_case():
    """The reference's doctest (gpu/geometry/Bvh.cu:336-404): three edges (set 0) and one
    triangle (set 1); the triangle overlaps edges 1 and 0, each pair reported once."""
    V = np.array([[0, 1, 2, 3, 0, 2, 0], [0, 0.1, 0.2, 0.3, 0, 0.1, 0], [0, 10, 20, 30, 0, 10, 0]], np.float32)
    E1 = np.array([[1, 0, 2], [2, 1, 3]])
    F2 = np.array([[4], [5], [6]])
    edges, tris = pbat.gpu.geometry.Aabb(3, 3), pbat.gpu.geometry.Aabb(3, 1)
    edges.construct(V, E1)
    tris.construct(V, F2)
    L = np.hstack([edges.min, tris.min])
    U = np.hstack([edges.max, tris.max])
    aabbs = pbat.gpu.geometry.Aabb(3, 4)
    aabbs.construct(L, U)
    sets = np.array([0, 0, 0, 1], np.int32)
    bvh = pbat.gpu.geometry.Bvh(4, 4)
    bvh.build(aabbs, L.min(axis=1), U.max(axis=1))
    O2 = bvh.detect_overlaps(aabbs, sets)
    assert O2.shape == (2, 2)
    assert {frozenset(c) for c in O2.T.tolist()} == {frozenset((3, 1)), frozenset((3, 0))}
    assert (bvh.visits == 2).all()


@pytest.mark.parametrize("n", [2, 3, 50, 2000])
def test_self_overlaps_equal_brute_force(n):
    rng = np.random.default_rng(n)
    c = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    r = rng.uniform(0.005, 0.05, (n, 3)).astype(np.float32)
    lo, hi = c - r, c + r
    lo[: n // 10] = lo[n // 10: 2 * (n // 10)]  # duplicated boxes (equal Morton codes)
    hi[: n // 10] = hi[n // 10: 2 * (n // 10)]
    bvh = pbat.gpu.geometry.Bvh(n, 16)
    bvh.build(lo.T, hi.T, lo.min(axis=0), hi.max(axis=0))
    O1 = bvh.detect_overlaps(lo.T, upper=hi.T)
    got = [frozenset(p) for p in O1.T.tolist()]
    assert len(got) == len(set(got))  # each pair once
    assert set(got) == _brute_self_overlaps(lo, hi)
    sets = rng.integers(0, 3, n).astype(np.int32)
    O2 = bvh.detect_overlaps(lo.T, sets, upper=hi.T)
    got2 = [frozenset(p) for p in O2.T.tolist()]
    assert len(got2) == len(set(got2))
    assert set(got2) == _brute_self_overlaps(lo, hi, sets)


def _np_point_triangle(p, a, b, c):
    """FP64 point-triangle distance by Voronoi regions (independent of the device code)."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = ab @ ap, ac @ ap
    if d1 <= 0 and d2 <= 0:
        return np.linalg.norm(p - a)
    bp = p - b
    d3, d4 = ab @ bp, ac @ bp
    if d3 >= 0 and d4 <= d3:
        return np.linalg.norm(p - b)
    vc = d1 * d4 - d3 * d2
    if vc <= 0 and d1 >= 0 and d3 <= 0:
        return np.linalg.norm(p - (a + d1 / (d1 - d3) * ab))
    cp = p - c
    d5, d6 = ab @ cp, ac @ cp
    if d6 >= 0 and d5 <= d6:
        return np.linalg.norm(p - c)
    vb = d5 * d2 - d1 * d6
    if vb <= 0 and d2 >= 0 and d6 <= 0:
        return np.linalg.norm(p - (a + d2 / (d2 - d6) * ac))
    va = d3 * d6 - d5 * d4
    if va <= 0 and (d4 - d3) >= 0 and (d5 - d6) >= 0:
        return np.linalg.norm(p - (b + (d4 - d3) / ((d4 - d3) + (d5 - d6)) * (c - b)))
    den = 1.0 / (va + vb + vc)
    return np.linalg.norm(p - (a + ab * vb * den + ac * vc * den))


def _np_point_tet(p, a, b, c, d):
    def outside(u, v, w):
        return (p - u) @ np.cross(v - u, w - u) > 0
    if not (outside(a, b, d) or outside(b, c, d) or outside(c, a, d) or outside(a, c, b)):
        return 0.0
    return min(_np_point_triangle(p, a, b, d), _np_point_triangle(p, b, c, d), _np_point_triangle(p, c, a, d),
               _np_point_triangle(p, a, c, b))


def test_point_triangle_nearest_neighbours_are_nearest():
    """Nearest surface triangle of a jittered cube to points inside, near and far from it: the
    triangle returned is at the FP64 brute-force minimum distance (to FP32 rounding)."""
    w = meshgen.unit_cube_workload(n=6, seed=4)
    X = w["X"].astype(np.float64)
    F = meshgen.boundary_faces(w["T"]).astype(np.int32)
    aabbs = pbat.gpu.geometry.Aabb(3, F.shape[0])
    aabbs.construct(X.T, F.T)
    lo, hi = aabbs.min, aabbs.max
    np.testing.assert_array_equal(lo, X[F].min(axis=1).T.astype(np.float32))
    np.testing.assert_array_equal(hi, X[F].max(axis=1).T.astype(np.float32))
    bvh = pbat.gpu.geometry.Bvh(F.shape[0], 0)
    bvh.build(aabbs, lo.min(axis=1) - 1, hi.max(axis=1) + 1)
    rng = np.random.default_rng(2)
    P = np.vstack([rng.uniform(-0.5, 1.5, (300, 3)), rng.uniform(0.1, 0.9, (100, 3))]).astype(np.float32)
    nn = bvh.point_triangle_nearest_neighbours(aabbs, P.T, X.T, F.T)
    X32 = X.astype(np.float32).astype(np.float64)
    for q, f in enumerate(nn):
        d = np.array([_np_point_triangle(P[q].astype(np.float64), *X32[F[j]]) for j in range(F.shape[0])])
        assert 0 <= f < F.shape[0]
        assert d[f] <= d.min() + 1e-5


def test_point_tetrahedron_nearest_neighbours_are_nearest():
    """Nearest tetrahedron of a jittered cube: points inside get a tetrahedron that contains them
    (distance 0), points outside one at the FP64 brute-force minimum distance."""
    w = meshgen.unit_cube_workload(n=4, seed=6)
    X = w["X"].astype(np.float32)
    T = w["T"].astype(np.int32)
    aabbs = pbat.gpu.geometry.Aabb(3, T.shape[0])
    aabbs.construct(X.T, T.T)
    bvh = pbat.gpu.geometry.Bvh(T.shape[0], 0)
    bvh.build(aabbs, aabbs.min.min(axis=1), aabbs.max.max(axis=1))
    rng = np.random.default_rng(3)
    P = np.vstack([rng.uniform(0.05, 0.95, (200, 3)), rng.uniform(-0.4, 1.4, (100, 3))]).astype(np.float32)
    nn = bvh.point_tetrahedron_nearest_neighbours(aabbs, P.T, X.T, T.T)
    X64 = X.astype(np.float64)
    for q, t in enumerate(nn):
        d = np.array([_np_point_tet(P[q].astype(np.float64), *X64[T[j]]) for j in range(T.shape[0])])
        assert 0 <= t < T.shape[0]
        assert d[t] <= d.min() + 1e-5
