"""Contact term of the oracle and of the device arithmetic, pinned to the reference's
AccumulateVertexTriangleContact (fixture made from its FP64 instantiation)."""

import ctypes as C
import pathlib

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen

GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def test_oracle_contact_matches_reference_fixture():
    g = np.load(GOLD / "contact.npz")
    hit = 0
    for k in range(g["dt"].size):
        gg = g["g"][k, 0].copy()
        H = g["H"][k, 0].copy()
        O.lib().orc_vertex_triangle_contact(g["xtv"][k], g["xv"][k], g["xtf"][k], g["xf"][k], g["dt"][k], g["muC"][k],
                                           g["muF"][k], g["epsv"][k], float(np.finfo(np.float64).eps), gg, H)
        scale = max(1.0, np.abs(g["H"][k, 1]).max())
        np.testing.assert_allclose(H, g["H"][k, 1], rtol=1e-9, atol=1e-9 * scale)
        np.testing.assert_allclose(gg, g["g"][k, 1], rtol=1e-9, atol=1e-9 * max(1.0, np.abs(g["g"][k, 1]).max()))
        hit += int(not np.allclose(g["g"][k, 0], g["g"][k, 1]))
    assert hit > 20  # both contact and no-contact cases are covered


def test_device_contact_arithmetic_matches_reference_fixture():
    g = np.load(GOLD / "contact.npz")
    L = _capi.lib()
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    for k in range(g["dt"].size):
        gg = f(g["g"][k, 0])
        H = f(g["H"][k, 0])
        E = C.c_float()
        args = [f(g["xtv"][k]), f(g["xv"][k]), f(g["xtf"][k]), f(g["xf"][k])]  # kept alive for the call
        rc = L.pbgb_debug_vertex_triangle_contact(*[a.ctypes.data for a in args],
                                                  g["dt"][k], g["muC"][k], g["muF"][k], g["epsv"][k],
                                                  gg.ctypes.data, H.ctypes.data, C.byref(E))
        assert rc == 0
        ref_g, ref_H = g["g"][k, 1], g["H"][k, 1]
        np.testing.assert_allclose(H, ref_H, rtol=2e-3, atol=2e-4 * max(1.0, np.abs(ref_H).max()))
        np.testing.assert_allclose(gg, ref_g, rtol=2e-3, atol=2e-4 * max(1.0, np.abs(ref_g).max()))


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built")
def test_oracle_contact_matches_reference_directly():
    R = O.ref()
    rng = np.random.default_rng(11)
    for _ in range(200):
        xf = rng.uniform(-1, 1, (3, 3))
        p = rng.dirichlet([1, 1, 1]) @ xf
        n = np.cross(xf[1] - xf[0], xf[2] - xf[0])
        xv = p - 0.01 * n / np.linalg.norm(n)
        xtv = xv + rng.uniform(-0.02, 0.02, 3)
        xtf = (xf + rng.uniform(-0.02, 0.02, (3, 3))).ravel()
        g1, H1, g2, H2 = np.zeros(3), np.zeros(9), np.zeros(3), np.zeros(9)
        R.ref_vertex_triangle_contact_d(xtv, xv, xtf, np.ascontiguousarray(xf.ravel()), 1 / 60, 1e6, 0.3, 1e-2, g1, H1)
        O.lib().orc_vertex_triangle_contact(xtv, xv, xtf, np.ascontiguousarray(xf.ravel()), 1 / 60, 1e6, 0.3, 1e-2,
                                           float(np.finfo(np.float64).eps), g2, H2)
        np.testing.assert_allclose(g2, g1, rtol=1e-10, atol=1e-9)
        np.testing.assert_allclose(H2, H1, rtol=1e-10, atol=1e-9)


def small_scene(n_cubes=2, hexes=3, slab=(8, 8, 1)):
    return meshgen.contact_scene_workload(n_cubes_side=n_cubes, cube_hexes=hexes, slab_hexes=slab, gap=0.01)


def test_oracle_contact_step_keeps_cubes_above_slab():
    w = small_scene()
    O_ = O.OracleContactVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], w["V"], w["F"], w["B"],
                            muC=1e7, strategy=2)
    z0 = w["X"][w["B"] > 0, 2].min()
    zs = []
    for _ in range(20):
        O_.step(1 / 60, 20, 1, 1)
        zs.append(O_.x[w["B"] > 0, 2].min())
    assert np.isfinite(O_.x).all()
    assert zs[-1] < z0  # fell onto the slab (top face at z = 0)
    assert min(zs) > -0.02  # and was stopped by it
    assert abs(zs[-1] - zs[-2]) < 2e-3  # coming to rest
    assert O_.active.sum() > 0


def _point_in_tets(p, X, T):
    """Brute-force PointTetrahedron3D (geometry/OverlapQueries.h:562-587) of points p against every
    tet: inside unless strictly outside one of the faces (A,B,D), (B,C,D), (C,A,D), (A,C,B)."""
    A, B, Cc, D = (X[T[:, k]] for k in range(4))
    inside = np.ones((p.shape[0], T.shape[0]), bool)
    for a, b, c in ((A, B, D), (B, Cc, D), (Cc, A, D), (A, Cc, B)):
        nrm = np.cross(b - a, c - a)
        side = np.einsum("ptk,tk->pt", p[:, None, :] - a[None], nrm)
        inside &= side <= 0.0
    return inside


def test_multibody_dcd_oracle_matches_brute_force():
    """The CPU multibody detector's discrete half on a cube sunk 5 cm into a slab: penetrating
    vertices in both directions, and each one's nearest surface triangles of the body it
    penetrates, against brute force."""
    w = meshgen.contact_scene_workload(n_cubes_side=1, cube_hexes=4, slab_hexes=(8, 8, 1), cell=1.0)
    X, T, F, V, B = w["X"].copy(), w["T"], w["F"], w["V"], w["B"]
    X[B == 1, 2] -= 0.05 + 0.05  # the cube's bottom 5 cm below the slab's top
    body, nearest, d2 = O.dcd_contacts(X, T, F, V, B)
    p = X[V]
    for q_body in (0, 1):
        other = 1 - q_body
        qs = np.nonzero(B[V] == q_body)[0]
        inside = _point_in_tets(p[qs], X, T[B[T[:, 0]] == other]).any(axis=1)
        np.testing.assert_array_equal(body[qs] >= 0, inside)
        assert inside.sum() > 0
        assert (body[qs][inside] == other).all()
    # Nearest triangles of the penetrated body: squared distances against brute force.
    pen = np.nonzero(body >= 0)[0]
    for q in pen:
        tris = np.nonzero(B[F[:, 0]] == body[q])[0]
        a, b, c = (X[F[tris, k]] for k in range(3))
        dist = np.array([O_point_triangle(p[q], a[j], b[j], c[j]) for j in range(len(tris))])
        assert abs(d2[q] - dist.min()) <= 1e-12
        listed = nearest[q][nearest[q] >= 0]
        assert len(listed) >= 1 and set(listed) <= set(tris[np.abs(dist - dist.min()) <= 0.0])


def O_point_triangle(p, a, b, c):
    """Squared point-triangle distance by dense sampling-free projection (barycentric clamp over the
    face, then the three edges)."""
    ab, ac = b - a, c - a
    M = np.array([[ab @ ab, ab @ ac], [ab @ ac, ac @ ac]])
    rhs = np.array([ab @ (p - a), ac @ (p - a)])
    u, v = np.linalg.solve(M, rhs)
    if u >= 0 and v >= 0 and u + v <= 1:
        q = a + u * ab + v * ac
        return float((p - q) @ (p - q))

    def seg(p, s0, s1):
        d = s1 - s0
        t = np.clip((p - s0) @ d / (d @ d), 0.0, 1.0)
        r = p - (s0 + t * d)
        return float(r @ r)

    return min(seg(p, a, b), seg(p, b, c), seg(p, c, a))


def _toi_by_scan(p0, p1, tri0, tri1, n=20001):
    """Earliest time in [0, 1] at which the point lies in the triangle, by a dense scan of the
    coplanarity sign with barycentric checks at the crossings (reference-free check)."""
    t = np.linspace(0.0, 1.0, n)
    P = p0 + t[:, None] * (p1 - p0)
    A, Bv, Cc = (tri0[k] + t[:, None] * (tri1[k] - tri0[k]) for k in range(3))
    f = np.einsum("ij,ij->i", np.cross(Bv - A, Cc - A), P - A)
    for j in np.nonzero(np.sign(f[:-1]) * np.sign(f[1:]) <= 0)[0]:
        # linear interpolation of the crossing inside [t_j, t_j+1]
        tc = t[j] if f[j] == f[j + 1] else t[j] + (t[j + 1] - t[j]) * f[j] / (f[j] - f[j + 1])
        a, b, c = (tri0[k] + tc * (tri1[k] - tri0[k]) for k in range(3))
        x = p0 + tc * (p1 - p0)
        ab, ac, ap = b - a, c - a, x - a
        d00, d01, d11, d20, d21 = ab @ ab, ab @ ac, ac @ ac, ap @ ab, ap @ ac
        den = d00 * d11 - d01 * d01
        v, w = (d11 * d20 - d01 * d21) / den, (d00 * d21 - d01 * d20) / den
        if min(1 - v - w, v, w) >= -1e-6 and max(1 - v - w, v, w) <= 1 + 1e-6:
            return tc
    return -1.0


def test_vertex_triangle_ccd_oracle():
    """The vertex-triangle CCD of the multibody detector (geometry/PointTriangleCcd.h:125-160): a
    point falling through a fixed triangle hits it at the crossing time; one passing beside it
    does not; seeded random linear motions agree with a dense scan of the coplanarity sign."""
    tri = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    pts = np.array([[0.2, 0.2, 1.0], [0.2, 0.2, -1.0], [2.0, 2.0, 1.0], [2.0, 2.0, -1.0]])

    def one(p0, p1, t0, t1):
        xt = np.vstack([p0, t0])
        x = np.vstack([p1, t1])
        F = np.array([[1, 2, 3]])
        toi, f = O.ccd_vertex_triangle(xt, x, F, np.array([0]), np.array([0, 1, 1, 1]))
        return toi[0]

    assert abs(one(pts[0], pts[1], tri, tri) - 0.5) < 1e-12
    assert one(pts[2], pts[3], tri, tri) == -1.0
    rng = np.random.default_rng(7)
    hits = 0
    for _ in range(300):
        p0, p1 = rng.normal(size=3), rng.normal(size=3)
        t0 = rng.normal(size=(3, 3))
        t1 = t0 + 0.8 * rng.normal(size=(3, 3))
        got, want = one(p0, p1, t0, t1), _toi_by_scan(p0, p1, t0, t1)
        assert (got < 0) == (want < 0), (got, want)
        if got >= 0:
            hits += 1
            assert abs(got - want) < 1e-3
    assert hits > 10


# ---------------------------------------------------------------------------------------------
# Continuous half of the CPU multibody detector: point-triangle and edge-edge CCD.

def test_ccd_reference_doctest_cases():
    """Known answers of the reference's doctests (geometry/PointTriangleCcd.cpp:13-31,
    geometry/EdgeEdgeCcd.cpp:13-33): both crossings happen at t = 1/2, the edge-edge one at the
    middle of both edges."""
    pt_t = np.array([[0, 0.25, 0.25], [1, 0, 0], [1, 1, 0], [1, 0, 1]], float)
    pt_x = pt_t + np.array([[1, 0, 0], [-1, 0, 0], [-1, 0, 0], [-1, 0, 0]], float)
    assert O.point_triangle_ccd(pt_t, pt_x) == 0.5
    ee_t = np.array([[0, 0, 0], [0, 1, 1], [1, 0, 1], [1, 1, 0]], float)
    ee_x = ee_t + np.array([[1, 0, 0], [1, 0, 0], [-1, 0, 0], [-1, 0, 0]], float)
    np.testing.assert_array_equal(O.edge_edge_ccd(ee_t, ee_x), [0.5, 0.5, 0.5])


def _check_ccd_against(xts, xs, rs, pt):
    """Oracle CCD against the reference's results.  Point-triangle: hit or no hit everywhere, times
    of impact to 1e-9.  Edge-edge: both return the parameters of the last root visited, which agree
    to 1e-9 everywhere (the same roots are visited); hit or no hit agrees everywhere but on near
    misses (every fourth case, index % 4 == 3: one end point moved by 1e-9), where the hit test
    (closest distance exactly 0 in floating point) is decided by rounding: there the cubic is
    nearly degenerate and last-bit differences of its coefficients move the root by ~1e-12."""
    decided_by_rounding = 0
    for i, (xt, x, r) in enumerate(zip(xts, xs, rs)):
        if pt:
            t = O.point_triangle_ccd(xt, x)
            assert (t >= 0) == (r[0] >= 0), (i, t, r)
            if t >= 0:
                assert abs(t - r[0]) <= 1e-9
            continue
        got = O.edge_edge_ccd(xt, x)
        np.testing.assert_allclose(got[1:], r[1:], rtol=0, atol=1e-9)
        if (got[0] >= 0) != (r[0] >= 0):
            assert i % 4 == 3, (i, got, r)
            decided_by_rounding += 1
        elif got[0] >= 0:
            assert abs(got[0] - r[0]) <= 1e-9
    assert decided_by_rounding <= len(rs) // 8
    return decided_by_rounding


def test_ccd_oracle_matches_reference_fixture():
    """The oracle's CCD queries against the reference's own (fixture made from its FP64 build):
    generic motions, exact dyadic crossings, crossings whose second edge turns (which the
    reference's edge-edge cubic misses as written) and near misses (the agreement bar is in
    _check_ccd_against)."""
    g = np.load(GOLD / "ccd.npz")
    assert (g["ee_r"][:, 0] >= 0).sum() > 100 and (g["pt_r"][:, 0] >= 0).sum() > 300
    _check_ccd_against(g["pt_xt"], g["pt_x"], g["pt_r"], pt=True)
    _check_ccd_against(g["ee_xt"], g["ee_x"], g["ee_r"], pt=False)


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built")
def test_ccd_oracle_matches_reference_directly():
    import sys
    sys.path.insert(0, str(GOLD))
    import make_golden

    R = O.ref()
    fam = make_golden._ccd_families(np.random.default_rng(99), 2000)
    for key, fn, width in (("pt", R.ref_point_triangle_ccd, 4), ("ee", R.ref_edge_edge_ccd, 3)):
        rs = []
        for xt, x in fam[key]:
            o = np.zeros(width)
            fn(xt, x, o)
            rs.append(o)
        _check_ccd_against([a for a, _ in fam[key]], [b for _, b in fam[key]], rs, pt=key == "pt")


def _two_box_scene():
    """Two 2x2x2-hex boxes on dyadic coordinates: box 0 fixed on [0, 1]^3, box 1 above it, offset
    by (1/4, 3/8) in x and y, falling by 1/2 during the step; its bottom face reaches box 0's top
    face at t = 1/4, where axis-aligned edges cross exactly."""
    X0, T0 = meshgen.hex_grid(2, 2, 2, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    X1, T1 = meshgen.hex_grid(2, 2, 2, (0.25, 0.375, 1.125), (1.25, 1.375, 2.125))
    X = np.vstack([X0, X1]).astype(np.float64)
    T = np.vstack([T0, T1 + X0.shape[0]]).astype(np.int32)
    B = np.repeat([0, 1], [X0.shape[0], X1.shape[0]]).astype(np.int32)
    F = meshgen.boundary_faces(T).astype(np.int32)
    E = np.unique(np.sort(np.vstack([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1), axis=0).astype(np.int32)
    V = np.unique(F).astype(np.int32)
    Xe = X.copy()
    Xe[B == 1, 2] -= 0.5
    return X, Xe, T, F, E, V, B


def test_multibody_edge_edge_pairs_match_pairwise_queries():
    """orc_ccd_edge_edge over two boxes' surface edges: the box prefilter and the body rule lose no
    hit of the pairwise query run over every cross-body pair, the faces' exact crossings are found
    at t = 1/4, and edges with a penetrating end point drop out."""
    X, Xe, T, F, E, V, B = _two_box_scene()
    ei, ej, tuv = O.ccd_edge_edge(X, Xe, E, B)

    def brute(mask):
        out = {}
        for a in range(E.shape[0]):
            for b in range(E.shape[0]):
                if B[E[a, 0]] != 0 or B[E[b, 0]] != 1 or mask[E[a]].any() or mask[E[b]].any():
                    continue
                r = O.edge_edge_ccd(np.vstack([X[E[a]], X[E[b]]]), np.vstack([Xe[E[a]], Xe[E[b]]]))
                if r[0] >= 0:
                    out[(a, b)] = r
        return out

    want = brute(np.zeros(X.shape[0], bool))
    assert len(want) >= 4
    assert set(zip(ei.tolist(), ej.tolist())) == set(want)
    for a, b, r in zip(ei, ej, tuv):
        np.testing.assert_array_equal(r, want[(a, b)])
    assert (tuv[:, 0] == 0.25).sum() >= 4  # the two faces meet; later crossings lie inside box 0
    # Penetrating vertices: box 1's bottom layer.
    pen = np.zeros(X.shape[0], bool)
    pen[(B == 1) & (X[:, 2] == 1.125)] = True
    ei2, ej2, _ = O.ccd_edge_edge(X, Xe, E, B, pen)
    assert set(zip(ei2.tolist(), ej2.tolist())) == set(brute(pen))
    assert not pen[E[ei2]].any() and not pen[E[ej2]].any()
    assert len(ei2) < len(ei)


def test_multibody_all_pairs_composition():
    """The active-set update of the CPU multibody detector (UpdateActiveSet): the discrete half's
    vertices (box 1 moved at XK by 3/4 in x and sunk 1/16 into box 0's corner) report their nearest
    triangles and take no part in the continuous half; every continuous vertex-triangle pair is a
    hit of the pairwise query."""
    X, Xe, T, F, E, V, B = _two_box_scene()
    XK = X.copy()
    XK[B == 1] += [0.75, 0.0, -0.1875]
    VTv, VTf, EEei, EEej = O.multibody_all_pairs(X, Xe, XK, V, E, F, T, B)
    body, nearest, _ = O.dcd_contacts(XK, T, F, V, B)
    pen_vertices = set(V[body >= 0].tolist())
    assert len(pen_vertices) > 0
    n_dcd = sum(int((nearest[q] >= 0).sum()) for q in np.nonzero(body >= 0)[0])
    assert set(VTv[:n_dcd].tolist()) == pen_vertices
    for v, f in zip(VTv[n_dcd:], VTf[n_dcd:]):
        assert v not in pen_vertices and B[v] != B[F[f, 0]]
        assert O.point_triangle_ccd(np.vstack([X[v], X[F[f]]]), np.vstack([Xe[v], Xe[F[f]]])) >= 0
    mask = np.zeros(X.shape[0], bool)
    mask[list(pen_vertices)] = True
    ei, ej, _ = O.ccd_edge_edge(X, Xe, E, B, mask)
    assert set(zip(EEei.tolist(), EEej.tolist())) == set(zip(ei.tolist(), ej.tolist()))
    for a, b in zip(EEei, EEej):
        assert not set(E[a].tolist()) & pen_vertices and not set(E[b].tolist()) & pen_vertices
    assert len(VTv) > n_dcd
