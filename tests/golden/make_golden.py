"""Generates the golden fixtures of tests/golden/ from the reference's own code.

Run where the reference sources are available, with PBAT_REF_SRC naming the reference checkout's
``source/`` directory (``make -C oracle ref`` then builds ``oracle/_ref/libpbat_ref.so`` from them):

    PBAT_REF_SRC=/root/reference/source python tests/golden/make_golden.py      # every fixture
    PBAT_REF_SRC=/root/reference/source python tests/golden/make_golden.py ccd  # only ccd.npz

Every fixture is produced by calling the reference's header-only kernels through the harness
(oracle/ref_harness.cpp), on seeded inputs, so the oracle can be pinned on machines without the
reference.  Known-answer values transcribed from the reference's doctests are in kat.json.
"""

from __future__ import annotations

import ctypes as C
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

import oracle_lib as O  # noqa: E402
from physicsbasedanimationtoolkit_gb300 import meshgen  # noqa: E402


def random_F(rng, n):
    return np.eye(3)[None] + 0.35 * rng.standard_normal((n, 3, 3))


def snh(R, rng):
    n = 64
    F = random_F(rng, n)
    mu = rng.uniform(1e3, 1e6, n)
    lam = rng.uniform(1e3, 1e7, n)
    E = np.zeros(n)
    G = np.zeros((n, 9))
    H = np.zeros((n, 81))
    for k in range(n):
        f = np.ascontiguousarray(F[k].ravel(order="F"))
        E[k] = R.ref_snh_eval(f, mu[k], lam[k])
        g = np.zeros(9)
        h = np.zeros(81)
        R.ref_snh_grad_hessian(f, mu[k], lam[k], g, h)
        G[k], H[k] = g, h
    np.savez_compressed(HERE / "snh.npz", F=F, mu=mu, lam=lam, E=E, G=G, H=H)


def vertex_solves(R, rng):
    cases = []
    for c in range(48):
        n = int(rng.integers(1, 25))
        X = rng.standard_normal((n, 4, 3)) * 0.1
        # Build non-degenerate tets and their GP from rest shapes.
        GPs = np.zeros((n, 12))
        wgs = np.zeros(n)
        xe = np.zeros((n, 12))
        for q in range(n):
            while True:
                P = rng.standard_normal((4, 3)) * 0.1
                Dm = np.stack([P[1] - P[0], P[2] - P[0], P[3] - P[0]], axis=1)
                d = np.linalg.det(Dm)
                if d > 1e-4:
                    break
            Ji = np.linalg.inv(Dm)
            G = np.zeros((4, 3))
            G[1:] = Ji
            G[0] = -Ji.sum(axis=0)
            GPs[q] = G.ravel()
            wgs[q] = d / 6
            Xd = P + 0.02 * rng.standard_normal((4, 3))
            xe[q] = Xd.ravel()  # 3x4 column-major == 4 rows of xyz
        il = rng.integers(0, 4, n).astype(np.int32)
        mus = rng.uniform(1e4, 1e6, n)
        las = rng.uniform(1e5, 1e7, n)
        xt = rng.standard_normal(3) * 0.1
        xtl = xt + rng.standard_normal(3) * 0.01
        xi = xt + rng.standard_normal(3) * 0.01
        mi = rng.uniform(0.01, 2.0)
        kD = [0.0, 1e-3, 1e-2][c % 3]
        h = 1.0 / 60
        g = np.zeros(3)
        H = np.zeros(9)
        xo = xi.copy()
        R.ref_vertex_solve(n, np.ascontiguousarray(xe), np.ascontiguousarray(GPs), il, wgs, mus, las,
                           xt, xtl, mi, kD, h, h * h, 1e-7, xo, g, H)
        cases.append(dict(n=n, xe=xe, GPs=GPs, il=il, wg=wgs, mu=mus, lam=las, xt=xt, xtilde=xtl,
                          x=xi, m=mi, kD=kD, h=h, x_out=xo, g=g, H=H))
    flat = {}
    for k, cse in enumerate(cases):
        for name, val in cse.items():
            flat[f"c{k}_{name}"] = np.asarray(val)
    flat["count"] = np.array(len(cases))
    np.savez_compressed(HERE / "vertex_solve.npz", **flat)


def init_strategies(R, rng):
    n = 64
    xt = rng.standard_normal((n, 3))
    vtm1 = rng.standard_normal((n, 3))
    vt = rng.standard_normal((n, 3))
    a = rng.standard_normal((n, 3))
    a[::7] = 0.0
    out = np.zeros((5, n, 3))
    for s in range(5):
        for k in range(n):
            r = np.zeros(3)
            R.ref_initial_positions(xt[k].copy(), vtm1[k].copy(), vt[k].copy(), a[k].copy(), 1 / 60, 1 / 3600, s, r)
            out[s, k] = r
    np.savez_compressed(HERE / "init_strategies.npz", xt=xt, vtm1=vtm1, vt=vt, a=a, out=out)


def chebyshev(R):
    rhos = np.array([0.5, 0.9, 0.95, 0.99])
    om = np.zeros((rhos.size, 60))
    for r, rho in enumerate(rhos):
        w = 0.0
        for k in range(60):
            w = R.ref_chebyshev_omega(k, rho * rho, w)
            om[r, k] = w
    np.savez_compressed(HERE / "chebyshev.npz", rho=rhos, omega=om)


def coloring(R):
    out = {}
    meshes = {"cube5": meshgen.cube5()[1].T, "cube10": meshgen.hex_grid(10, 10, 10)[1],
              "beam": meshgen.hex_grid(12, 3, 3, hi=(4.0, 1.0, 1.0))[1]}
    for name, T in meshes.items():
        nV = int(T.max()) + 1
        ptr, adj = O.primal_graph(T, nV)
        out[f"{name}_T"] = T.astype(np.int32)
        for o in range(3):
            for s in range(2):
                c = np.zeros(nV, np.int32)
                R.ref_greedy_color(nV, ptr, adj, o, s, c)
                out[f"{name}_{o}_{s}"] = c
    np.savez_compressed(HERE / "coloring.npz", **out)


def trajectories(R):
    out = {}
    # The reference doctest's 5-tet cube, 1 step of 10 iterations at dt=1e-2.
    P, T, _, _ = meshgen.cube5()
    X, Tr = P.T.copy(), T.T.copy()
    for cheb in (None, 0.9):
        I = O.OracleVbd(X, Tr, np.full(5, 1000.0), *meshgen.lame(np.full(5, 1e6), np.full(5, 0.45)),
                        dbc=np.zeros(0, np.int32), rho_chebyshev=cheb)
        I.step(1e-2, 10, 1, 1, use_ref=True)
        out[f"cube5_{'cheb' if cheb else 'base'}_x"] = I.x.copy()
    # The unit-cube workload: 30 steps of 20 iterations at dt = 1/60 (CPU semantics).
    w = meshgen.unit_cube_workload()
    I = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"])
    I.step(1 / 60, 20, 1, 30, use_ref=True)
    out["cube10_x"] = I.x.copy()
    out["cube10_v"] = I.v.copy()
    # A small beam with Chebyshev (reference weights), damping and 2 substeps.
    X, T = meshgen.hex_grid(12, 3, 3, hi=(4.0, 1.0, 1.0))
    dbc = meshgen.face_vertices(X, 0, 0.0)
    rng = np.random.default_rng(5)
    v0 = rng.uniform(-0.1, 0.1, X.shape)
    mu, lam = meshgen.lame(np.full(T.shape[0], 5e5), np.full(T.shape[0], 0.48))
    I = O.OracleVbd(X, T, np.full(T.shape[0], 1000.0), mu, lam, dbc, v=v0, rho_chebyshev=0.95, kD=1e-3,
                    strategy=3)
    I.step(1 / 60, 15, 2, 6, use_ref=True)
    out["beam_x"] = I.x.copy()
    out["beam_v"] = I.v.copy()
    out["beam_v0"] = v0
    np.savez_compressed(HERE / "trajectories.npz", **out)


def morton_codes(R, rng):
    """Boxes in a scene box, their centres normalised in FP32 with the reference's operation order
    ((0.5*(b+e) - wmin)/(wmax - wmin), each step rounded), then the reference's Morton3D."""
    n = 4096
    wmin = np.array([-1.0, 0.5, -2.0], np.float32)
    wmax = np.array([3.0, 1.5, 6.0], np.float32)
    c = rng.uniform(-0.05, 1.05, (n, 3)).astype(np.float32)
    lo = (wmin + c * (wmax - wmin) - rng.uniform(0, 0.01, (n, 3))).astype(np.float32)
    hi = (lo + rng.uniform(0, 0.02, (n, 3))).astype(np.float32)
    lo[:64] = lo[64:128]  # duplicate boxes -> equal codes
    hi[:64] = hi[64:128]
    ext = (wmax - wmin).astype(np.float32)
    cn = ((np.float32(0.5) * (lo + hi)).astype(np.float32) - wmin).astype(np.float32) / ext
    codes = np.array([R.ref_morton3d(*map(float, p)) for p in cn.astype(np.float32)], np.uint32)
    np.savez_compressed(HERE / "morton.npz", lo=lo, hi=hi, wmin=wmin, wmax=wmax, codes=codes)


def contact_cases(R, rng):
    """The reference's vertex-triangle contact kernel in FP64 on seeded configurations: vertices
    slightly behind or in front of a triangle's plane, inside and outside its projection."""
    n = 96
    out = {k: [] for k in ("xtv", "xv", "xtf", "xf", "dt", "muC", "muF", "epsv", "g", "H", "E")}
    for c in range(n):
        xf = rng.uniform(-0.5, 0.5, (3, 3))
        xf[:, 2] = rng.uniform(-0.05, 0.05, 3)
        xtf = xf + rng.uniform(-0.01, 0.01, (3, 3))
        bary = rng.dirichlet([1, 1, 1]) if c % 4 else rng.uniform(-0.5, 1.5, 3)
        p = bary @ xf
        nrm = np.cross(xf[1] - xf[0], xf[2] - xf[0])
        nrm /= np.linalg.norm(nrm)
        xv = p + nrm * rng.uniform(-0.02, 0.01)
        xtv = xv + rng.uniform(-0.01, 0.01, 3)
        g = rng.standard_normal(3)
        H = rng.standard_normal((3, 3))
        H = H + H.T
        args = dict(xtv=xtv, xv=xv, xtf=np.ascontiguousarray(xtf.ravel()), xf=np.ascontiguousarray(xf.ravel()),
                    dt=1 / 60, muC=rng.uniform(1e4, 1e7), muF=rng.uniform(0.0, 0.6),
                    epsv=[1e-3, 1e-1, 10.0][c % 3])
        g_out = g.copy()
        H_out = np.ascontiguousarray(H.ravel(order="F"))
        E = R.ref_vertex_triangle_contact_d(args["xtv"], args["xv"], args["xtf"], args["xf"], args["dt"],
                                            args["muC"], args["muF"], args["epsv"], g_out, H_out)
        for k, v in args.items():
            out[k].append(v)
        out["g"].append(np.stack([g, g_out]))
        out["H"].append(np.stack([H.ravel(order="F"), H_out]))
        out["E"].append(E)
    np.savez_compressed(HERE / "contact.npz", **{k: np.array(v) for k, v in out.items()})


def _ccd_families(rng, n):
    """Seeded CCD inputs, four points at the start (xt) and the end (x) of the step, in four
    families: generic random motions; exact dyadic crossings (the reference doctests' configurations
    under random power-of-two scales, integer shifts and axis permutations, where the arithmetic is
    exact); the same crossings with the second edge also turning (exact at the crossing time, where
    the reference's edge-edge cubic misses them as written); near misses offset by 1e-9."""
    g_pt = np.array([[0, 0.25, 0.25], [1, 0, 0], [1, 1, 0], [1, 0, 1]], float)
    d_pt = np.array([[1, 0, 0], [-1, 0, 0], [-1, 0, 0], [-1, 0, 0]], float)
    g_ee = np.array([[0, 0, 0], [0, 1, 1], [1, 0, 1], [1, 1, 0]], float)
    d_ee = np.array([[1, 0, 0], [1, 0, 0], [-1, 0, 0], [-1, 0, 0]], float)
    fam = {"pt": [], "ee": []}
    for key, g0, d0 in (("pt", g_pt, d_pt), ("ee", g_ee, d_ee)):
        for k in range(n):
            kind = k % 4
            if kind == 0:
                xt = rng.uniform(-1, 1, (4, 3))
                x = xt + rng.uniform(-1, 1, (4, 3))
            else:
                perm = rng.permutation(3)
                s = 2.0 ** int(rng.integers(-3, 4))
                sh = rng.integers(-8, 8, 3).astype(float)
                xt = (g0 * s)[:, perm] + sh
                x = xt + (d0 * s)[:, perm]
                if kind == 2:
                    turn = (rng.integers(-2, 3, 3) * s)[perm].astype(float)
                    xt[3] -= 0.5 * turn  # the last point turns about the crossing time t = 1/2
                    x[3] += 0.5 * turn
                elif kind == 3:
                    x[0] += 1e-9 * rng.standard_normal(3)
            fam[key].append((np.ascontiguousarray(xt), np.ascontiguousarray(x)))
    return fam


def ccd_cases(R, rng):
    """The reference's own point-triangle and edge-edge CCD queries (geometry/PointTriangleCcd.h,
    geometry/EdgeEdgeCcd.h) in FP64 on the families of _ccd_families."""
    fam = _ccd_families(rng, 400)
    out = {}
    for key, fn, width in (("pt", R.ref_point_triangle_ccd, 4), ("ee", R.ref_edge_edge_ccd, 3)):
        xs, xe, r = [], [], []
        for xt, x in fam[key]:
            o = np.zeros(width)
            fn(xt, x, o)
            xs.append(xt)
            xe.append(x)
            r.append(o)
        out[key + "_xt"], out[key + "_x"], out[key + "_r"] = np.array(xs), np.array(xe), np.array(r)
    np.savez_compressed(HERE / "ccd.npz", **out)


def main(only=None):
    O.build_oracle(ref=True)
    R = O.ref()
    if R is None:
        raise SystemExit("the reference harness was not built")
    if only == "ccd":
        ccd_cases(R, np.random.default_rng(20261204))
        print("fixtures written to", HERE)
        return
    rng = np.random.default_rng(20261203)
    snh(R, rng)
    vertex_solves(R, rng)
    init_strategies(R, rng)
    chebyshev(R)
    coloring(R)
    trajectories(R)
    morton_codes(R, rng)
    contact_cases(R, rng)
    ccd_cases(R, np.random.default_rng(20261204))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
