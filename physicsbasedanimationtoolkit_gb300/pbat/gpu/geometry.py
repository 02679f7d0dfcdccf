"""``pbat.gpu.geometry.Bvh``: linear BVH over axis-aligned boxes (reference binding:
bindings/pypbat/gpu/geometry/Bvh.cpp; implementation gpu/impl/geometry/Bvh.cu).

Boxes are given as lower / upper corner arrays of shape ``3 x |#boxes|`` (the reference passes a
``pbat.gpu.geometry.Aabb`` object holding the same two arrays).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from ... import _capi


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

    def build(self, lower, upper, min, max):  # noqa: A002 (reference argument names)
        """Morton-sort the boxes inside the scene box [min, max] and build the hierarchy."""
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
