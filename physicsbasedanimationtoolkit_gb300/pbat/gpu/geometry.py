"""``pbat.gpu.geometry.Aabb`` and ``pbat.gpu.geometry.Bvh``: axis-aligned boxes and the linear BVH
over them (reference bindings: bindings/pypbat/gpu/geometry/Aabb.cpp, Bvh.cpp; implementation
gpu/geometry/Aabb.cu, Bvh.cu, gpu/impl/geometry/Bvh.cu/.cuh).

Boxes are passed either as an ``Aabb`` (as in the reference) or as lower / upper corner arrays of
shape ``3 x |#boxes|``.  The reference's ``Bvh.build`` sorts the ``Aabb`` it is given in place (by
Morton code); here the tree keeps its own sorted copy and the ``Aabb`` is left as constructed.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from ... import _capi


def _points(a, what):
    a = np.asarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[0] != 3:
        raise ValueError(f"expected {what} as a 3 x |#points| array")
    return np.ascontiguousarray(a.T)


class Aabb:
    """Axis-aligned boxes in 3 dimensions (reference: bindings/pypbat/gpu/geometry/Aabb.cpp).
    ``construct(min, max)`` takes the corners; ``construct(P, S)`` computes the boxes of the
    simplices S (K x |#simplices|, K = 1..4 vertices) over the points P (3 x |#points|) on the GPU."""

    def __init__(self, dims=3, n_aabb=0):
        if int(dims) != 3:
            raise ValueError("only 3-dimensional boxes are supported")
        self.resize(dims, n_aabb)

    def resize(self, dims, n_aabb):
        if int(dims) != 3:
            raise ValueError("only 3-dimensional boxes are supported")
        self._lo = np.zeros((3, int(n_aabb)), np.float32)
        self._hi = np.zeros((3, int(n_aabb)), np.float32)

    def construct(self, *args, **kwargs):
        if "P" in kwargs or "S" in kwargs or (len(args) == 2 and np.asarray(args[1]).dtype.kind in "iu"):
            P = kwargs.get("P", args[0] if args else None)
            S = kwargs.get("S", args[1] if len(args) > 1 else None)
            pts = _points(P, "P")
            simp = np.asarray(S)
            if simp.ndim != 2 or not 1 <= simp.shape[0] <= 4:
                raise ValueError("expected S as a K x |#simplices| array, K = 1..4")
            k, nS = simp.shape
            S_rows = np.ascontiguousarray(simp.T, dtype=np.int32)
            lo = np.zeros((nS, 3), np.float32)
            hi = np.zeros((nS, 3), np.float32)
            _capi.check_bvh(_capi.lib().pbgb_simplex_boxes(pts.shape[0], pts.ctypes.data, nS, S_rows.ctypes.data, k,
                                                           lo.ctypes.data, hi.ctypes.data))
            self._lo, self._hi = lo.T.copy(), hi.T.copy()
            return
        L = kwargs.get("min", args[0] if args else None)
        U = kwargs.get("max", args[1] if len(args) > 1 else None)
        self._lo = np.array(Bvh._rows(L).T)
        self._hi = np.array(Bvh._rows(U).T)

    @property
    def n_boxes(self):
        return self._lo.shape[1]

    @property
    def dims(self):
        return 3

    @property
    def min(self):
        return self._lo.copy()

    @property
    def max(self):
        return self._hi.copy()


def _corners(aabbs, upper=None):
    if isinstance(aabbs, Aabb):
        return aabbs._lo, aabbs._hi
    if upper is None:
        raise ValueError("expected an Aabb or lower and upper corner arrays")
    return aabbs, upper


class Bvh:
    def __init__(self, max_boxes, max_overlaps=0):
        h = C.c_void_p()
        _capi.check_bvh(_capi.lib().pbgb_bvh_create(int(max_boxes), C.byref(h)))
        self._h = h
        self.max_boxes = int(max_boxes)
        self.max_overlaps = int(max_overlaps)
        self.n = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _capi.lib().pbgb_bvh_destroy(h)
            except Exception:
                pass
            self._h = None

    @staticmethod
    def _rows(a):
        a = np.asarray(a, dtype=np.float32)
        if a.ndim != 2 or a.shape[0] != 3:
            raise ValueError("expected a 3 x |#boxes| array")
        return np.ascontiguousarray(a.T)

    def build(self, *args, **kwargs):
        """Morton-sort the boxes inside the scene box [min, max] and build the hierarchy:
        ``build(aabbs, min, max)`` as in the reference, or ``build(lower, upper, min, max)``."""
        if args and isinstance(args[0], Aabb) or isinstance(kwargs.get("aabbs"), Aabb):
            aabbs = kwargs.pop("aabbs", None) or args[0]
            rest = list(args[1:])
            lower, upper = aabbs._lo, aabbs._hi
        else:
            rest = list(args)
            lower = kwargs.pop("lower", None) if "lower" in kwargs else rest.pop(0)
            upper = kwargs.pop("upper", None) if "upper" in kwargs else rest.pop(0)
        min = kwargs.pop("min", None) if "min" in kwargs else rest.pop(0)  # noqa: A001 (reference names)
        max = kwargs.pop("max", None) if "max" in kwargs else rest.pop(0)  # noqa: A001
        lo, hi = self._rows(lower), self._rows(upper)
        wmin = np.ascontiguousarray(min, dtype=np.float32).ravel()
        wmax = np.ascontiguousarray(max, dtype=np.float32).ravel()
        _capi.check_bvh(_capi.lib().pbgb_bvh_build(self._h, lo.shape[0], lo.ctypes.data, hi.ctypes.data,
                                                   wmin.ctypes.data, wmax.ctypes.data), self._h)
        self.n = lo.shape[0]

    def refit(self, lower, upper):
        lo, hi = self._rows(lower), self._rows(upper)
        _capi.check_bvh(_capi.lib().pbgb_bvh_refit(self._h, lo.ctypes.data, hi.ctypes.data), self._h)

    def overlaps(self, lower, upper):
        """2 x |#overlaps| array of (query, box) pairs whose boxes overlap."""
        lo, hi = self._rows(lower), self._rows(upper)
        cap = max(self.max_overlaps, 1024)
        while True:
            pairs = np.zeros(2 * cap, np.int32)
            count = C.c_int64()
            _capi.check_bvh(_capi.lib().pbgb_bvh_overlaps(self._h, lo.shape[0], lo.ctypes.data, hi.ctypes.data,
                                                          pairs.ctypes.data, cap, C.byref(count)), self._h)
            if count.value <= cap:
                return pairs[: 2 * count.value].reshape(-1, 2).T.copy()
            cap = int(count.value)

    def detect_overlaps(self, aabbs, set=None, upper=None):  # noqa: A002 (reference argument names)
        """Self-overlaps of the built boxes as a 2 x |#overlaps| array (each unordered pair once,
        the box of the leaf earlier in Morton order first); with ``set`` (one int per box), only
        pairs from different sets.  ``aabbs`` must be the boxes of the last ``build`` (an ``Aabb``,
        or the lower corners with ``upper``)."""
        lo, hi = _corners(aabbs, upper)
        if np.asarray(lo).shape[-1] != self.n:
            raise ValueError("aabbs must be the boxes given to the last build()")
        sv = None
        if set is not None:
            sv = np.ascontiguousarray(np.asarray(set).ravel(), dtype=np.int32)
            if sv.size != self.n:
                raise ValueError("set must hold one entry per box")
        cap = max(self.max_overlaps, 1024)
        while True:
            pairs = np.zeros(2 * cap, np.int32)
            count = C.c_int64()
            _capi.check_bvh(_capi.lib().pbgb_bvh_self_overlaps(
                self._h, None if sv is None else sv.ctypes.data, pairs.ctypes.data, cap, C.byref(count)), self._h)
            if count.value <= cap:
                return pairs[: 2 * count.value].reshape(-1, 2).T.copy()
            cap = int(count.value)

    def _nearest(self, X, V, S, k):
        pts = _points(X, "X")
        verts = _points(V, "V")
        simp = np.asarray(S)
        if simp.ndim != 2 or simp.shape[0] != k:
            raise ValueError(f"expected a {k} x |#simplices| index array")
        rows = np.ascontiguousarray(simp.T, dtype=np.int32)
        nn = np.full(pts.shape[0], -1, np.int32)
        _capi.check_bvh(_capi.lib().pbgb_bvh_nearest_simplices(
            self._h, pts.shape[0], pts.ctypes.data, verts.shape[0], verts.ctypes.data, rows.shape[0],
            rows.ctypes.data, k, nn.ctypes.data), self._h)
        return nn

    def point_triangle_nearest_neighbours(self, aabbs, X, V, F):
        """Nearest triangle (column of F over the points V) to each column of X; the BVH must have
        been built over the triangles' boxes.  Among exact ties, the reference's pick."""
        return self._nearest(X, V, F, 3)

    def point_tetrahedron_nearest_neighbours(self, aabbs, X, V, T):
        """Nearest tetrahedron (0 distance inside) to each column of X; the BVH must have been
        built over the tetrahedra's boxes."""
        return self._nearest(X, V, T, 4)

    @property
    def visits(self):
        out = np.zeros(max(self.n - 1, 0), np.int32)
        if self.n > 1:
            _capi.check_bvh(_capi.lib().pbgb_bvh_visits(self._h, out.ctypes.data), self._h)
        return out

    def _topology(self):
        n = self.n
        out = dict(codes=np.zeros(n, np.uint32), inds=np.zeros(n, np.int32),
                   child=np.zeros(max(2 * (n - 1), 1), np.int32), parent=np.zeros(2 * n - 1, np.int32),
                   rightmost=np.zeros(max(2 * (n - 1), 1), np.int32),
                   ilo=np.zeros((max(n - 1, 1), 3), np.float32), ihi=np.zeros((max(n - 1, 1), 3), np.float32))
        _capi.check_bvh(_capi.lib().pbgb_bvh_topology(
            self._h, out["codes"].ctypes.data, out["inds"].ctypes.data, out["child"].ctypes.data,
            out["parent"].ctypes.data, out["rightmost"].ctypes.data, out["ilo"].ctypes.data,
            out["ihi"].ctypes.data), self._h)
        out["child"] = out["child"][: 2 * (n - 1)].reshape(-1, 2)
        out["rightmost"] = out["rightmost"][: 2 * (n - 1)].reshape(-1, 2)
        out["ilo"], out["ihi"] = out["ilo"][: n - 1], out["ihi"][: n - 1]
        return out

    # Reference property names (bindings/pypbat/gpu/geometry/Bvh.cpp:91-112).
    @property
    def morton(self):
        return self._topology()["codes"]

    @property
    def ordering(self):
        return self._topology()["inds"]

    @property
    def child(self):
        return self._topology()["child"].T.copy()

    @property
    def parent(self):
        return self._topology()["parent"]

    @property
    def rightmost(self):
        return self._topology()["rightmost"].T.copy()

    @property
    def min(self):
        return self._topology()["ilo"].T.copy()

    @property
    def max(self):
        return self._topology()["ihi"].T.copy()
