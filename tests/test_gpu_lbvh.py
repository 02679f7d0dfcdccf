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


@pytest.mark.parametrize("n", [2, 3, 1000, 200_000])
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
