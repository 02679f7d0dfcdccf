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
