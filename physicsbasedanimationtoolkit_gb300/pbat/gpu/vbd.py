"""``pbat.gpu.vbd``: the GPU VBD integrator (reference binding:
bindings/pypbat/gpu/vbd/Integrator.cpp:26-103; C++ API gpu/vbd/Integrator.h:33-148).

``Integrator(data)`` reproduces the reference GPU integrator's step semantics (AdaptiveVbd uses
the previous step's velocity).  ``BatchedIntegrator([data, ...])`` advances many independent meshes
with one launch sequence per step (an addition: the reference has one mesh per integrator).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from ... import _capi
from ..._integrator import IntegratorBase, SEMANTICS_GPU


class Integrator(IntegratorBase):
    def __init__(self, data):
        super().__init__(data, SEMANTICS_GPU)

    def step(self, dt=0.01, iterations=20, substeps=1):
        """Integrate 1 time step (dt, iterations per substep, substeps)."""
        self._step(dt, iterations, substeps)

    @property
    def x(self):
        """3 x |#vertices| vertex positions (float32)."""
        return self._get("x")

    @x.setter
    def x(self, value):
        self._set("x", value)

    @property
    def v(self):
        """3 x |#vertices| vertex velocities (float32)."""
        return self._get("v")

    @v.setter
    def v(self, value):
        self._set("v", value)

    def _no_get(self):
        raise AttributeError("write-only property (as in the reference binding)")

    a = property(lambda self: self._no_get(), lambda self, a: self._set("a", a),
                 doc="3 x |#vertices| external accelerations (set-only)")
    detH_residual = property(lambda self: self._no_get(), lambda self, z: self._set_detH(z),
                             doc="Numerical zero of the Hessian determinant check (set-only)")
    kD = property(lambda self: self._no_get(), lambda self, k: self._set_kD(k),
                  doc="Uniform Rayleigh damping coefficient (set-only)")
    strategy = property(lambda self: self._no_get(), lambda self, s: self._set_strategy(s),
                        doc="Initialization strategy (set-only)")

    @property
    def gpu_block_size(self):
        self._no_get()

    @gpu_block_size.setter
    def gpu_block_size(self, b):
        _capi.check(_capi.lib().pbgb_vbd_set_block_size(self._h, int(b)), self._h)

    @property
    def scene_bounding_box(self):
        self._no_get()

    @scene_bounding_box.setter
    def scene_bounding_box(self, box):
        lo = np.ascontiguousarray(box[0], dtype=np.float32).ravel()
        hi = np.ascontiguousarray(box[1], dtype=np.float32).ravel()
        _capi.check(_capi.lib().pbgb_vbd_set_scene_bounding_box(self._h, lo.ctypes.data, hi.ctypes.data), self._h)


class BatchedIntegrator(IntegratorBase):
    """Many meshes of uneven size advanced together: their arrays are concatenated, colour c of
    the batch is the union of every mesh's colour c, and one captured launch sequence steps all
    of them.  ``x``/``v`` address the concatenation (mesh b's vertices follow mesh b-1's)."""

    def __init__(self, datas, semantics=SEMANTICS_GPU):
        datas = list(datas)
        if not datas:
            raise ValueError("expected at least one mesh")
        super().__init__(datas[0], semantics, batch=datas)
        self.datas = datas
        self.vertex_offsets = np.cumsum([0] + [d.X.shape[1] for d in datas])

    def step(self, dt=0.01, iterations=20, substeps=1):
        self._step(dt, iterations, substeps)

    @property
    def x(self):
        return self._get("x")

    @x.setter
    def x(self, value):
        self._set("x", value)

    @property
    def v(self):
        return self._get("v")

    @v.setter
    def v(self, value):
        self._set("v", value)
