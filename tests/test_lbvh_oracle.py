"""LBVH oracle pinned to the reference: the 5-tet cube topology of the reference's doctest, the
reference's Morton3D on FP32-normalised box centres (fixture), and structural invariants."""

import json
import pathlib

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen

GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def cube5_tet_boxes():
    P, T, _, _ = meshgen.cube5()
    X = P.T.astype(np.float32)
    pts = X[T.T]
    return pts.min(axis=1), pts.max(axis=1), X.min(axis=0), X.max(axis=0)


def test_cube_topology_known_answer():
    kat = json.loads((GOLD / "kat.json").read_text())["bvh_cube5"]
    lo, hi, wmin, wmax = cube5_tet_boxes()
    b = O.bvh_build(lo, hi, wmin, wmax)
    np.testing.assert_array_equal(b["child"], np.array(kat["child"]))
    np.testing.assert_array_equal(b["parent"], np.array(kat["parent"]))
    np.testing.assert_array_equal(b["rightmost"], np.array(kat["rightmost"]))


def test_morton_codes_match_reference_fixture():
    g = np.load(GOLD / "morton.npz")
    codes = O.morton(g["lo"], g["hi"], g["wmin"], g["wmax"])
    np.testing.assert_array_equal(codes, g["codes"])
    assert np.unique(codes).size < codes.size  # duplicates present


def check_tree(b, lo, hi):
    n = b["inds"].size
    child, parent, rm = b["child"], b["parent"], b["rightmost"]
    leafBegin = n - 1
    assert parent[0] == -1
    # Every node except the root has exactly one parent that lists it as a child.
    for node in range(1, 2 * n - 1):
        p = parent[node]
        assert child[p, 0] == node or child[p, 1] == node
    # Codes sorted, (code, index) strictly increasing (stable order).
    key = b["codes"].astype(np.uint64) << np.uint64(32) | b["inds"].astype(np.uint64)
    assert np.all(np.diff(key.astype(np.float64)) > 0) or np.all(key[1:] > key[:-1])
    # Subtree leaf ranges and rightmost leaves; boxes contain their leaves.
    def rng(node):
        if node >= leafBegin:
            return node - leafBegin, node - leafBegin
        a, _ = rng(child[node, 0])
        _, d = rng(child[node, 1])
        return a, d
    for i in range(0, n - 1, max(1, (n - 1) // 200)):
        a, d = rng(i)
        _, lend = rng(child[i, 0])
        assert rm[i, 0] == leafBegin + lend
        assert rm[i, 1] == leafBegin + d
        leaves = b["inds"][a: d + 1]
        assert np.all(b["ilo"][i] <= lo[leaves].min(axis=0))
        assert np.all(b["ihi"][i] >= hi[leaves].max(axis=0))
        np.testing.assert_array_equal(b["ilo"][i], lo[leaves].min(axis=0))
        np.testing.assert_array_equal(b["ihi"][i], hi[leaves].max(axis=0))


@pytest.mark.parametrize("n", [2, 3, 17, 1000])
def test_random_trees_are_well_formed(n):
    import sys
    sys.setrecursionlimit(10000)
    rng = np.random.default_rng(n)
    lo = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    hi = (lo + rng.uniform(0, 0.05, (n, 3))).astype(np.float32)
    lo[: n // 3] = lo[n // 3: 2 * (n // 3)]  # equal codes exercise the index tie-break
    hi[: n // 3] = hi[n // 3: 2 * (n // 3)]
    b = O.bvh_build(lo, hi, [0, 0, 0], [1.05, 1.05, 1.05])
    check_tree(b, lo, hi)


def test_brute_force_overlaps():
    lo = np.array([[0, 0, 0], [2, 2, 2]], np.float32)
    hi = np.array([[1, 1, 1], [3, 3, 3]], np.float32)
    qlo = np.array([[1, 1, 1], [1.5, 1.5, 1.5], [2.5, 0, 2.5]], np.float32)
    qhi = np.array([[2, 2, 2], [1.6, 1.6, 1.6], [2.6, 4, 2.6]], np.float32)
    pairs = O.overlaps(lo, hi, qlo, qhi)
    assert {tuple(p) for p in pairs} == {(0, 0), (0, 1), (2, 1)}
    np.testing.assert_array_equal(pairs, O.overlaps(lo, hi, qlo, qhi, all_pairs=True))


@pytest.mark.parametrize("case", ["random", "touching", "duplicates", "wide", "negative"])
def test_pruned_overlaps_equal_all_pairs(case):
    """The x-sorted candidate search returns exactly the pairs of the all-pairs test, in the same
    order (query, then box index)."""
    rng = np.random.default_rng(len(case))
    n, nq = 3000, 1500
    lo = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    hi = (lo + rng.uniform(0, 0.03, (n, 3))).astype(np.float32)
    qlo = rng.uniform(0, 1, (nq, 3)).astype(np.float32)
    qhi = (qlo + rng.uniform(0, 0.03, (nq, 3))).astype(np.float32)
    if case == "touching":  # queries whose lower x equals a box's upper x (closed boxes)
        qlo[:500, 0] = hi[:500, 0]
        qlo[:500, 1:] = lo[:500, 1:]
        qhi[:500] = np.maximum(qhi[:500], qlo[:500])
    elif case == "duplicates":
        lo[: n // 2] = lo[n // 2:]
        hi[: n // 2] = hi[n // 2:]
    elif case == "wide":  # one very wide box widens every candidate range
        lo[7], hi[7] = [-5, 0, 0], [5, 1, 1]
    elif case == "negative":
        lo, hi, qlo, qhi = lo - 2.0, hi - 2.0, qlo - 2.0, qhi - 2.0
    got = O.overlaps(lo, hi, qlo, qhi)
    exp = O.overlaps(lo, hi, qlo, qhi, all_pairs=True)
    assert exp.shape[0] > 0
    np.testing.assert_array_equal(got, exp)
