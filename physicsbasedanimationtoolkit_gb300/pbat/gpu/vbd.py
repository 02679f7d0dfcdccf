"""``pbat.gpu.vbd``: the GPU VBD integrator (reference binding:
bindings/pypbat/gpu/vbd/Integrator.cpp:26-103; C++ API gpu/vbd/Integrator.h:33-148).

``Integrator(data)`` reproduces the reference GPU integrator's step semantics (AdaptiveVbd uses
the previous step's velocity).  ``BatchedIntegrator([data, ...])`` advances many independent meshes
with one persistent kernel launch per step (an addition: the reference has one mesh per
integrator).
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

    def traced_step(self, dt=0.01, iterations=20, substeps=1, t=0, dir="."):
        """Integrate 1 time step and trace the result to disk as Matrix Market files named
        {variable}.t.{timestep}.s.{substep}[.k.{iteration}].mtx (plain VBD iterations)."""
        _capi.check(_capi.lib().pbgb_vbd_traced_step(self._h, float(dt), int(iterations), int(substeps), int(t),
                                                    str(dir).encode()), self._h)

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
    """Many meshes of uneven size advanced together: their arrays are concatenated, and one
    persistent kernel launch per step advances every mesh, each through its own colours (a mesh
    moves on as soon as its own previous colour is done).  With ``persistent = False``, or where
    the persistent step does not apply, colour c of the batch is the union of every mesh's colour c,
    one launch per colour.  ``x``/``v`` address the concatenation (mesh b's vertices follow mesh
    b-1's)."""

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
    def persistent(self):
        """Whether the next step runs as one persistent launch."""
        active = C.c_int32()
        _capi.check(_capi.lib().pbgb_vbd_persistent(self._h, C.byref(active)), self._h)
        return bool(active.value)

    @persistent.setter
    def persistent(self, enable):
        _capi.check(_capi.lib().pbgb_vbd_set_persistent(self._h, int(bool(enable))), self._h)

    @property
    def batch_tile(self):
        return getattr(self, "_batch_tile", 1)

    @batch_tile.setter
    def batch_tile(self, subtiles):
        """Sweep work items of ``subtiles`` x (block size / lanes per vertex) vertices."""
        _capi.check(_capi.lib().pbgb_vbd_set_batch_tile(self._h, int(subtiles)), self._h)
        self._batch_tile = int(subtiles)

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


class _Rollout:
    """torch.autograd.Function over ``steps`` GPU VBD steps (built on first use so that importing
    this module does not import torch)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        import torch

        class Rollout(torch.autograd.Function):
            @staticmethod
            def forward(ctx, mu, lam, x0, v0, integ, dt, iterations, substeps, steps, every):
                dev = x0.device
                nV = integ.n_vertices
                # The tape is reserved up front so that unsupported settings fail here.
                integ.adjoint_reserve(min(every, steps) * substeps, iterations)
                integ.set_material(mu.detach().cpu().numpy(), lam.detach().cpu().numpy())
                x = x0.detach().to(torch.float32).contiguous()
                v = v0.detach().to(torch.float32).contiguous()
                torch.cuda.synchronize(dev)
                integ._set_device("x", x.data_ptr())
                integ._set_device("v", v.data_ptr())
                checkpoints = []
                # The last segment is recorded on the way (a recorded step computes exactly what a
                # plain step does), so backward reverses it without running it again.
                last = ((steps - 1) // every) * every
                for t in range(steps):
                    if t % every == 0:
                        cx = torch.empty((nV, 3), dtype=torch.float32, device=dev)
                        cv = torch.empty_like(cx)
                        cp = torch.empty_like(cx)
                        integ._get_device("x", cx.data_ptr())
                        integ._get_device("v", cv.data_ptr())
                        integ._get_device("vprev", cp.data_ptr())
                        checkpoints.append((cx, cv, cp))
                    if t >= last:
                        integ.step_record(dt, iterations, substeps, (t - last) * substeps)
                    else:
                        integ.step(dt, iterations, substeps)
                xT = torch.empty((nV, 3), dtype=torch.float32, device=dev)
                vT = torch.empty_like(xT)
                pT = torch.empty_like(xT)
                integ._get_device("x", xT.data_ptr())
                integ._get_device("v", vT.data_ptr())
                integ._get_device("vprev", pT.data_ptr())
                integ.synchronize()
                ctx.integ = integ
                ctx.args = (dt, iterations, substeps, steps, every)
                ctx.checkpoints = checkpoints
                ctx.taped = True  # the tape holds the last segment until a backward reuses its slots
                ctx.final = (xT.clone(), vT.clone(), pT)
                ctx.save_for_backward(mu, lam)
                return xT, vT

            @staticmethod
            def backward(ctx, gx, gv):
                mu, lam = ctx.saved_tensors
                integ = ctx.integ
                dt, iterations, substeps, steps, every = ctx.args
                dev = ctx.final[0].device
                nV, nT = integ.n_vertices, integ.n_tets
                xbar = (torch.zeros((nV, 3), device=dev) if gx is None else gx.detach().to(dev, torch.float32)).contiguous().clone()
                vbar = (torch.zeros((nV, 3), device=dev) if gv is None else gv.detach().to(dev, torch.float32)).contiguous().clone()
                # The previous velocities (read by AdaptiveVbd under the GPU semantics) are state
                # too: their adjoint is carried from step to step; nothing depends on the last ones.
                pbar = torch.zeros((nV, 3), dtype=torch.float32, device=dev)
                dlogmu = torch.zeros(nT, dtype=torch.float64, device=dev)
                dloglambda = torch.zeros_like(dlogmu)
                integ.adjoint_reserve(min(every, steps) * substeps, iterations)
                torch.cuda.synchronize(dev)
                nseg = len(ctx.checkpoints)
                for seg in reversed(range(nseg)):
                    start = seg * every
                    end = min(start + every, steps)
                    cx, cv, cp = ctx.checkpoints[seg]
                    integ._set_device("x", cx.data_ptr())
                    integ._set_device("v", cv.data_ptr())
                    integ._set_device("vprev", cp.data_ptr())
                    if not (seg == nseg - 1 and ctx.taped):
                        for t in range(start, end):
                            integ.step_record(dt, iterations, substeps, (t - start) * substeps)
                    ctx.taped = False
                    for t in reversed(range(start, end)):
                        integ.step_adjoint((t - start) * substeps, substeps, xbar.data_ptr(), vbar.data_ptr(),
                                           dlogmu.data_ptr(), dloglambda.data_ptr(), pbar.data_ptr())
                # Leave the integrator at the end of the forward rollout.
                integ._set_device("x", ctx.final[0].data_ptr())
                integ._set_device("v", ctx.final[1].data_ptr())
                integ._set_device("vprev", ctx.final[2].data_ptr())
                integ.synchronize()
                dmu = dlogmu.to(mu.dtype).to(mu.device) / mu.detach()
                dlam = dloglambda.to(lam.dtype).to(lam.device) / lam.detach()
                return dmu, dlam, xbar, vbar, None, None, None, None, None, None

        cls.fn = Rollout
        return Rollout


def rollout(integrator, mu, lam, x0, v0, dt=0.01, iterations=20, steps=1, substeps=1, checkpoint_every=5):
    """Differentiable rollout of ``steps`` steps of ``integrator`` (an addition: the reference has
    no differentiation).

    mu, lam: per-tet Lame coefficients (|#tets|, torch tensors; set on the integrator);
    x0, v0: |#vertices| x 3 start positions and velocities (CUDA tensors).  Returns the positions
    and velocities after the last step.  Backward runs the adjoint kernels: the positions are
    checkpointed every ``checkpoint_every`` steps in the forward pass, the last segment is
    recorded on the way (the tape holds ``checkpoint_every`` steps), and every other segment is
    re-run with recording before it is reversed; with ``checkpoint_every >= steps`` the whole
    rollout is taped in the forward pass and backward re-runs nothing.  The gradient is the exact derivative of the
    computed iterations (FP32).  Supported: plain VBD or Chebyshev acceleration, any Rayleigh
    damping, every initial guess (the adaptive guesses' factor is differentiated on the branch the
    forward took), no contact.  The previous velocities the integrator holds at the start (read by
    AdaptiveVbd) are part of the start state but not differentiated.  Backward leaves the
    integrator at the rollout's end state.
    """
    if checkpoint_every < 1:
        raise ValueError("checkpoint_every must be >= 1")
    return _Rollout.get().apply(mu, lam, x0, v0, integrator, float(dt), int(iterations), int(substeps), int(steps),
                                int(checkpoint_every))
