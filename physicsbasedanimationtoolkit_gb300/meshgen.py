"""Seeded synthetic tetrahedral meshes for the VBD workloads.

The reference ships no mesh files for this path (its beam tool needs ``gpytoolbox``), so every
workload here is generated: a structured hex grid whose hexes are split into 6 tetrahedra along
the main diagonal (Kuhn / Freudenthal split, conforming across hexes), optional uniform vertex
jitter, pinned faces and per-tet materials.

Array conventions follow the reference's Python API (``pbat.sim.vbd.Data.with_volume_mesh``):
positions are ``3 x |#vertices|`` and tetrahedra ``4 x |#tets|`` (column per entity).  The
functions here return row-per-entity arrays (``|#vertices| x 3`` float64, ``|#tets| x 4`` int32),
callers transpose when they feed the reference-shaped API.
"""

from __future__ import annotations

import itertools

import numpy as np

# The 6 Kuhn tets of the unit cube: monotone lattice paths 000 -> 111, one per axis permutation.
_KUHN_PATHS = []
for _perm in itertools.permutations(range(3)):
    _c = [0, 0, 0]
    _path = [tuple(_c)]
    for _ax in _perm:
        _c[_ax] = 1
        _path.append(tuple(_c))
    _KUHN_PATHS.append(_path)


def _orient_local(path):
    """Reorder a 4-corner path so that the tet has positive volume."""
    p = np.array(path, dtype=np.float64)
    d = np.linalg.det(np.stack([p[1] - p[0], p[2] - p[0], p[3] - p[0]], axis=1))
    return path if d > 0 else [path[0], path[2], path[1], path[3]]


_KUHN = [_orient_local(p) for p in _KUHN_PATHS]


def hex_grid(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """Vertices and Kuhn tets of an ``nx x ny x nz`` hex grid spanning the box ``[lo, hi]``.

    Vertex ``(i, j, k)`` has index ``i + (nx+1)*(j + (ny+1)*k)`` (x fastest).  Hex ``(i, j, k)``
    contributes 6 consecutive tets, hexes ordered x fastest, so tets are spatially coherent.
    """
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    zs = np.linspace(lo[2], hi[2], nz + 1)
    Z, Y, Xc = np.meshgrid(zs, ys, xs, indexing="ij")
    X = np.stack([Xc.ravel(), Y.ravel(), Z.ravel()], axis=1)

    def vid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    T = np.empty((ii.size, 6, 4), dtype=np.int64)
    for t, path in enumerate(_KUHN):
        for a, (bx, by, bz) in enumerate(path):
            T[:, t, a] = vid(ii + bx, jj + by, kk + bz)
    return X, T.reshape(-1, 4).astype(np.int32)


def jitter(X, amount, seed):
    """Add ``U(-amount, amount)`` to every coordinate, from ``seed``."""
    rng = np.random.default_rng(seed)
    return X + rng.uniform(-amount, amount, size=X.shape)


def face_vertices(X, axis, value, tol=1e-9):
    """Indices of vertices whose ``axis`` coordinate equals ``value`` (the pinned face)."""
    return np.nonzero(np.abs(X[:, axis] - value) <= tol)[0].astype(np.int32)


def boundary_faces(T):
    """Outward-oriented boundary triangles of a tet mesh (faces used by exactly one tet)."""
    T = np.asarray(T, dtype=np.int64)
    # Faces opposite each local vertex, wound so that their normal points away from that vertex
    # for a positively oriented tet (a, b, c, d): opposite a -> (b, c, d), b -> (a, d, c),
    # c -> (a, b, d), d -> (a, c, b).
    loc = np.array([[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]])
    faces = T[:, loc].reshape(-1, 3)
    key = np.sort(faces, axis=1)
    _, inv, counts = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    inv = inv.ravel()
    keep = counts[inv] == 1
    return faces[keep].astype(np.int32)


def cube5():
    """The reference tests' 5-tet unit cube (positions 3x8, tets 4x5, surface 3x12).

    Values follow ``sim/vbd/Integrator.cpp:251-264`` of the reference (its doctest fixture).
    Returned in the reference's column-per-entity layout.
    """
    P = np.array(
        [
            [0.0, 1.0, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0],
            [0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0],
            [0.0, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 1.0],
        ]
    )
    T = np.array(
        [[0, 3, 5, 6, 0], [1, 2, 4, 7, 5], [3, 0, 6, 5, 3], [5, 6, 0, 3, 6]], dtype=np.int32
    )
    F = np.array(
        [
            [0, 1, 1, 3, 3, 2, 2, 0, 0, 0, 4, 5],
            [1, 5, 3, 7, 2, 6, 0, 4, 3, 2, 5, 7],
            [4, 4, 5, 5, 7, 7, 6, 6, 1, 3, 6, 6],
        ],
        dtype=np.int32,
    )
    V = np.arange(8, dtype=np.int32)
    return P, T, V, F


def lame(E, nu):
    """Lame coefficients (mu, lambda) from Young's modulus and Poisson ratio."""
    E = np.asarray(E, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    mu = E / (2.0 * (1.0 + nu))
    lam = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return mu, lam


# ---------------------------------------------------------------------------------------------
# Workloads.  Each returns a dict of row-per-entity arrays and scalar settings.
# ---------------------------------------------------------------------------------------------


def unit_cube_workload(n=10, seed=0, jitter_frac=0.01, E=1e6, nu=0.45, rho=1000.0):
    """Unit cube ``[0,1]^3`` as an ``n^3`` hex grid (6 tets/hex), jittered by ``U(+-0.01 h)``.

    Material: Stable Neo-Hookean, density 1000, E=1e6, nu=0.45.  The x=0 face is pinned and
    gravity is -9.81 along z.  With n=10: 1331 vertices, 6000 tets.
    """
    X, T = hex_grid(n, n, n)
    h = 1.0 / n
    Xj = jitter(X, jitter_frac * h, seed)
    # Keep the pinned face exactly on x = 0 for the pin selection (select before jitter).
    dbc = face_vertices(X, 0, 0.0)
    mu, lam = lame(np.full(T.shape[0], E), np.full(T.shape[0], nu))
    return dict(
        X=Xj,
        T=T,
        dbc=dbc,
        rho=np.full(T.shape[0], rho),
        mu=mu,
        lam=lam,
        v=np.zeros_like(Xj),
    )


def beam_workload(nx=160, ny=40, nz=40, seed=0, E=5e5, nu=0.48, rho=1000.0, vmax=0.1):
    """Beam ``[0,4]x[0,1]x[0,1]`` as an ``nx x ny x nz`` hex grid split into 6 tets per hex.

    The x=0 face is pinned; initial velocities are ``U(-vmax, vmax)`` per component from
    ``seed``.  With 160x40x40: 270,641 vertices and 1,536,000 tets.
    """
    X, T = hex_grid(nx, ny, nz, hi=(4.0, 1.0, 1.0))
    dbc = face_vertices(X, 0, 0.0)
    rng = np.random.default_rng(seed)
    v = rng.uniform(-vmax, vmax, size=X.shape)
    mu, lam = lame(np.full(T.shape[0], E), np.full(T.shape[0], nu))
    return dict(X=X, T=T, dbc=dbc, rho=np.full(T.shape[0], rho), mu=mu, lam=lam, v=v)


def batch_workload(n_meshes=256, nmin=6, nmax=32, seed=0, spacing=1.5):
    """Many cube grids of uneven size: side ``n ~ U{nmin..nmax}`` hexes per mesh, unit cubes
    laid out on a line (x offset ``spacing`` apart).  E log-uniform in [1e5, 1e7],
    nu ~ U(0.30, 0.48), density 1000, the x=0 face of each cube pinned, gravity on.

    Returns a list of per-mesh workload dicts.
    """
    rng = np.random.default_rng(seed)
    sides = rng.integers(nmin, nmax + 1, size=n_meshes)
    E = np.exp(rng.uniform(np.log(1e5), np.log(1e7), size=n_meshes))
    nu = rng.uniform(0.30, 0.48, size=n_meshes)
    meshes = []
    for b in range(n_meshes):
        n = int(sides[b])
        X, T = hex_grid(n, n, n)
        dbc = face_vertices(X, 0, 0.0)
        X = X + np.array([spacing * b, 0.0, 0.0])
        mu, lam = lame(np.full(T.shape[0], E[b]), np.full(T.shape[0], nu[b]))
        meshes.append(
            dict(
                X=X,
                T=T,
                dbc=dbc,
                rho=np.full(T.shape[0], 1000.0),
                mu=mu,
                lam=lam,
                v=np.zeros_like(X),
                side=n,
            )
        )
    return meshes


def adjoint_beam_workload(nx=40, ny=10, nz=10, seed=0, nu=0.45, rho=1000.0, offset=(0.0, 0.0, -0.3)):
    """Differentiation workload: beam ``[0,4]x[0,1]x[0,1]`` as an ``nx x ny x nz`` hex grid, per-tet
    log Young's modulus ~ N(log 1e6, 0.3^2) from ``seed``, the x=0 face pinned, starting at rest.
    The loss is the sum over the x=4 tip-face vertices of |x - (X + offset)|^2.  With 40x10x10:
    4,961 vertices, 24,000 tets, 121 tip vertices.
    """
    X, T = hex_grid(nx, ny, nz, hi=(4.0, 1.0, 1.0))
    rng = np.random.default_rng(seed)
    logE = rng.normal(np.log(1e6), 0.3, size=T.shape[0])
    tip = face_vertices(X, 0, 4.0)
    return dict(X=X, T=T, dbc=face_vertices(X, 0, 0.0), logE=logE, nu=nu, rho=np.full(T.shape[0], rho),
                tip=tip, target=X[tip] + np.asarray(offset, dtype=np.float64))


def contact_scene_workload(n_cubes_side=4, cube_hexes=16, slab_hexes=(64, 64, 2), cube_size=0.6,
                           cell=1.0, gap=0.05, seed=0, E=1e6, nu=0.45, rho=1000.0):
    """Cubes dropped on a fixed slab: an ``n x n`` arrangement of ``cube_hexes^3``-hex cubes (6 tets
    per hex) with a seeded random yaw in [0, 2 pi), each centred in a ``cell`` x ``cell`` square,
    their bottoms ``gap`` above a ``slab_hexes`` slab whose top face is z = 0 and whose vertices are
    all pinned.  Body 0 is the slab, bodies 1.. the cubes.  With the defaults: 91,283 vertices,
    442,368 tets and 66,560 surface triangles.

    Returns X (nV x 3), T (nT x 4), F (surface triangles, nF x 3, outward), V (surface vertices),
    B (body of each vertex), dbc (pinned vertices) and materials.
    """
    rng = np.random.default_rng(seed)
    sx, sy, sz = slab_hexes
    hxy = cell * n_cubes_side / sx
    Xs, Ts = hex_grid(sx, sy, sz, lo=(0.0, 0.0, -hxy * sz), hi=(cell * n_cubes_side, cell * n_cubes_side, 0.0))
    Xs = Xs.copy()
    Xs[:, 2] = np.linspace(-hxy * sz, 0.0, sz + 1)[np.arange(Xs.shape[0]) // ((sx + 1) * (sy + 1))]
    parts_X, parts_T, parts_B = [Xs], [Ts], [np.zeros(Xs.shape[0], np.int32)]
    offset = Xs.shape[0]
    yaws = rng.uniform(0.0, 2.0 * np.pi, n_cubes_side * n_cubes_side)
    Xc, Tc = hex_grid(cube_hexes, cube_hexes, cube_hexes, lo=(-0.5, -0.5, 0.0), hi=(0.5, 0.5, 1.0))
    Xc = Xc * cube_size
    for k in range(n_cubes_side * n_cubes_side):
        i, j = k % n_cubes_side, k // n_cubes_side
        c, s = np.cos(yaws[k]), np.sin(yaws[k])
        R = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
        Xk = Xc @ R.T + np.array([(i + 0.5) * cell, (j + 0.5) * cell, gap])
        parts_X.append(Xk)
        parts_T.append(Tc + offset)
        parts_B.append(np.full(Xk.shape[0], k + 1, np.int32))
        offset += Xk.shape[0]
    X = np.vstack(parts_X)
    T = np.vstack(parts_T).astype(np.int32)
    B = np.concatenate(parts_B)
    F = boundary_faces(T)
    V = np.unique(F).astype(np.int32)
    dbc = np.arange(Xs.shape[0], dtype=np.int32)
    mu, lam = lame(np.full(T.shape[0], E), np.full(T.shape[0], nu))
    return dict(X=X, T=T, F=F, V=V, B=B, dbc=dbc, rho=np.full(T.shape[0], rho), mu=mu, lam=lam,
                v=np.zeros_like(X), yaws=yaws)


def triangle_boxes(X, F, Xnext=None):
    """Axis-aligned boxes of triangles (swept between X and Xnext when given): lower, upper (n x 3)."""
    P = X[F]
    if Xnext is not None:
        P = np.concatenate([P, Xnext[F]], axis=1)
    return P.min(axis=1), P.max(axis=1)
