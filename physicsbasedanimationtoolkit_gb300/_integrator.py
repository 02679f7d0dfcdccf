"""Handle management shared by ``pbat.sim.vbd.Integrator``, ``pbat.gpu.vbd.Integrator`` and the
batched integrator: builds ``pbgb_vbd_desc`` records from constructed ``Data`` and wraps the C ABI.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi

SEMANTICS_CPU = 0
SEMANTICS_GPU = 1

# Acceleration strategy each integrator runs, as the reference dispatches them: the CPU integrator
# (bindings/pypbat/sim/vbd/Integrator.cpp:31-45) builds Chebyshev, Anderson, Broyden and Nesterov
# integrators and the base integrator otherwise (trust region included); the GPU integrator
# (gpu/vbd/Integrator.cu:15-33) builds Anderson, Chebyshev and trust-region integrators and the base
# integrator otherwise (Nesterov and Broyden included).
_DISPATCH = {
    SEMANTICS_CPU: {0: 0, 1: 1, 2: 2, 3: 3, 4: 4, 5: 0},
    SEMANTICS_GPU: {0: 0, 1: 1, 2: 2, 3: 0, 4: 0, 5: 5},
}


def make_desc(data, semantics):
    """A ``pbgb_vbd_desc`` for a constructed ``Data`` plus the arrays it points into."""
    if not getattr(data, "_constructed", False):
        raise ValueError("Data must be constructed (call Data.construct()) before creating an integrator")
    accel = _DISPATCH[semantics].get(int(data.eAcceleration), 0)
    nV, nT = data.X.shape[1], data.E.shape[1]
    keep = dict(
        x=_capi.f64(np.asarray(data.x).T),
        X=_capi.f64(np.asarray(data.X).T),
        T=_capi.i32(np.asarray(data.E).T),
        v=_capi.f64(np.asarray(data.v).T),
        aext=_capi.f64(np.asarray(data.aext).T),
        m=_capi.f64(data.m),
        GP=_capi.f64(data._GP_rows),
        wg=_capi.f64(data.wg),
        mu=_capi.f64(data.lame[0]),
        lam=_capi.f64(data.lame[1]),
        Pptr=_capi.i32(data.Pptr),
        Padj=_capi.i32(data.Padj),
    )
    d = _capi.VbdDesc()
    d.n_vertices = nV
    d.n_tets = nT
    # The reference's CPU integrator has no contact terms (sim/vbd/Integrator.cpp:98-136): with its
    # semantics a surface mesh only describes the boundary; the GPU integrator adds contact.
    if semantics == SEMANTICS_GPU and getattr(data, "F", None) is not None and np.asarray(data.F).size > 0:
        keep.update(
            V=_capi.i32(data.V),
            F=_capi.i32(np.asarray(data.F).T),
            B=_capi.i32(data.B),
            XVA=_capi.f64(data.XVA),
            FA=_capi.f64(data.FA),
        )
        d.n_collision_vertices = int(np.asarray(data.V).size)
        d.n_collision_triangles = int(np.asarray(data.F).shape[1])
    d.muC = float(data.muC)
    d.muF = float(data.muF)
    d.epsv = float(data.epsv)
    d.active_set_update_frequency = int(data.active_set_update_frequency)
    for k, a in keep.items():
        setattr(d, k, a.ctypes.data)
    d.n_partitions = int(data.Pptr.size - 1)
    d.init_strategy = int(data.strategy)
    d.kD = float(data.kD)
    d.detHZero = float(data.detH_zero)
    d.acceleration = accel
    d.rho = float(data.rho)
    d.window_size = int(getattr(data, "window_size", 5))
    d.nesterov_lipschitz = float(getattr(data, "nesterov_L", 1.0))
    d.nesterov_start = int(getattr(data, "nesterov_start", 3))
    d.tr_eta = float(getattr(data, "eta", 0.2))
    d.tr_tau = float(getattr(data, "tau", 2.0))
    d.tr_curved = int(bool(getattr(data, "curved", True)))
    d.chebyshev_formula = int(getattr(data, "chebyshev_formula", 0))
    d.semantics = semantics
    return d, keep


class IntegratorBase:
    """Owns one ``pbgb_vbd`` handle."""

    def __init__(self, data, semantics, batch=None):
        L = _capi.lib()
        self.data = data
        self._semantics = semantics
        h = C.c_void_p()
        if batch is None:
            desc, self._keep = make_desc(data, semantics)
            rc = L.pbgb_vbd_create(C.byref(desc), C.byref(h))
        else:
            descs = (_capi.VbdDesc * len(batch))()
            self._keep = []
            for b, dat in enumerate(batch):
                dsc, keep = make_desc(dat, semantics)
                descs[b] = dsc
                self._keep.append(keep)
            rc = L.pbgb_vbd_create_batched(descs, len(batch), C.byref(h))
        _capi.check(rc)
        self._h = h
        self._keep = None  # the library copied everything during create
        nV, nT, nF, nC = (C.c_int32() for _ in range(4))
        _capi.check(L.pbgb_vbd_sizes(h, C.byref(nV), C.byref(nT), C.byref(nF), C.byref(nC)), h)
        self.n_vertices, self.n_tets, self.n_free, self.n_colors = nV.value, nT.value, nF.value, nC.value
        ref = data if batch is None else batch[0]
        self._strategy = ref.strategy
        self._kD = ref.kD
        self._detH = ref.detH_zero

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _capi.lib().pbgb_vbd_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def _step(self, dt, iterations, substeps):
        _capi.check(_capi.lib().pbgb_vbd_step(self._h, float(dt), int(iterations), int(substeps)), self._h)

    def synchronize(self):
        _capi.check(_capi.lib().pbgb_vbd_synchronize(self._h), self._h)

    def _get(self, which):
        out = np.empty((self.n_vertices, 3), dtype=np.float32)
        fn = {"x": "pbgb_vbd_get_positions", "v": "pbgb_vbd_get_velocities"}[which]
        _capi.check(getattr(_capi.lib(), fn)(self._h, out.ctypes.data), self._h)
        return out.T.copy()

    def _set(self, which, value):
        a = np.asarray(value, dtype=np.float32)
        if a.shape != (3, self.n_vertices):
            raise ValueError(f"expected an array of shape (3, {self.n_vertices})")
        buf = np.ascontiguousarray(a.T)
        fn = {
            "x": "pbgb_vbd_set_positions",
            "v": "pbgb_vbd_set_velocities",
            "a": "pbgb_vbd_set_external_acceleration",
        }[which]
        _capi.check(getattr(_capi.lib(), fn)(self._h, buf.ctypes.data), self._h)
        # set_* copies from pageable host memory on the handle's stream; wait so `buf` may die.
        self.synchronize()

    def _set_strategy(self, s):
        _capi.check(_capi.lib().pbgb_vbd_set_strategy(self._h, int(s)), self._h)
        self._strategy = s

    def _set_kD(self, kD):
        _capi.check(_capi.lib().pbgb_vbd_set_damping(self._h, float(kD)), self._h)
        self._kD = float(kD)

    def _set_detH(self, z):
        _capi.check(_capi.lib().pbgb_vbd_set_detH_zero(self._h, float(z)), self._h)
        self._detH = float(z)

    # -- extras beyond the reference API --------------------------------------------------------
    @property
    def lanes_per_vertex(self):
        return getattr(self, "_lanes", 0)

    @lanes_per_vertex.setter
    def lanes_per_vertex(self, lanes):
        _capi.check(_capi.lib().pbgb_vbd_set_lanes_per_vertex(self._h, int(lanes)), self._h)
        self._lanes = int(lanes)

    @property
    def staged_sweep(self):
        """(available, enabled) of the staged colour sweep (neighbours in shared memory)."""
        av, en = C.c_int32(), C.c_int32()
        _capi.check(_capi.lib().pbgb_vbd_staged_sweep(self._h, C.byref(av), C.byref(en)), self._h)
        return bool(av.value), bool(en.value)

    @staged_sweep.setter
    def staged_sweep(self, enable):
        _capi.check(_capi.lib().pbgb_vbd_set_staged_sweep(self._h, int(bool(enable))), self._h)

    def autotune(self, dt, iterations, substeps=1):
        """Pick lanes per vertex and block size by timing one step of each candidate (state is
        restored); returns (lanes, block_size, ms_per_step)."""
        lanes, block, ms = C.c_int32(), C.c_int32(), C.c_float()
        _capi.check(_capi.lib().pbgb_vbd_autotune(self._h, float(dt), int(iterations), int(substeps),
                                                 C.byref(lanes), C.byref(block), C.byref(ms)), self._h)
        self._lanes = lanes.value
        return lanes.value, block.value, ms.value

    def launches_per_step(self, iterations, substeps=1):
        n = C.c_int64()
        _capi.check(_capi.lib().pbgb_vbd_launches_per_step(self._h, int(iterations), int(substeps), C.byref(n)), self._h)
        return n.value

    def step_graph_kernels(self):
        """Kernel nodes of the CUDA graph the last step captured (-1 before the first step)."""
        n = C.c_int64()
        _capi.check(_capi.lib().pbgb_vbd_step_graph_kernels(self._h, C.byref(n)), self._h)
        return n.value

    def contacts(self):
        """(fc, active): contact triangles per vertex (|#vertices| x 8, -1 = none) and the active
        flags of the collision vertices after the last step."""
        nV = self.n_vertices
        fc = np.full((nV, 8), -1, np.int32)
        nS = int(np.asarray(getattr(self.data, "V", np.zeros(0))).size)
        active = np.zeros(max(nS, 1), np.uint8)
        _capi.check(_capi.lib().pbgb_vbd_get_contacts(self._h, fc.ctypes.data, active.ctypes.data), self._h)
        return fc, active[:nS]

    def contact_bvh(self):
        """The LBVH the last step built over the swept collision-triangle boxes: a dict of the
        sorted Morton codes, the sort order (inds), child / rightmost ((nF-1) x 2), parent, the
        full-step prediction xpred (|#vertices| x 3) the boxes were swept to from the positions at
        the step's start, and the scene box (min, max) the codes were normalised by."""
        nF = int(np.asarray(self.data.F).shape[1])
        nV = self.n_vertices
        out = dict(codes=np.zeros(nF, np.uint32), inds=np.zeros(nF, np.int32),
                   child=np.zeros(max(2 * (nF - 1), 1), np.int32), parent=np.zeros(max(2 * nF - 1, 1), np.int32),
                   rightmost=np.zeros(max(2 * (nF - 1), 1), np.int32), xpred=np.zeros((nV, 3), np.float32),
                   scene=np.zeros(6, np.float32))
        _capi.check(_capi.lib().pbgb_vbd_get_contact_bvh(
            self._h, out["codes"].ctypes.data, out["inds"].ctypes.data, out["child"].ctypes.data,
            out["parent"].ctypes.data, out["rightmost"].ctypes.data, out["xpred"].ctypes.data,
            out["scene"].ctypes.data), self._h)
        out["child"] = out["child"][: 2 * (nF - 1)].reshape(-1, 2)
        out["rightmost"] = out["rightmost"][: 2 * (nF - 1)].reshape(-1, 2)
        out["parent"] = out["parent"][: 2 * nF - 1]
        out["wmin"], out["wmax"] = out["scene"][:3].copy(), out["scene"][3:].copy()
        return out

    def save_state(self):
        """Checkpoint of the step state (positions, velocities, previous velocities, external
        accelerations, contact active set and lists) as bytes."""
        n = C.c_size_t()
        _capi.check(_capi.lib().pbgb_vbd_state_size(self._h, C.byref(n)), self._h)
        buf = (C.c_ubyte * n.value)()
        _capi.check(_capi.lib().pbgb_vbd_save_state(self._h, buf, n.value), self._h)
        return bytes(buf)

    def load_state(self, blob):
        """Resume from save_state's bytes (a handle built from the same data)."""
        buf = (C.c_ubyte * len(blob)).from_buffer_copy(blob)
        _capi.check(_capi.lib().pbgb_vbd_load_state(self._h, buf, len(blob)), self._h)

    def set_material(self, mu, lam):
        """Per-tet Lame coefficients (|#tets| each, system order); masses are kept."""
        mu = np.ascontiguousarray(mu, dtype=np.float64).ravel()
        lam = np.ascontiguousarray(lam, dtype=np.float64).ravel()
        if mu.size != self.n_tets or lam.size != self.n_tets:
            raise ValueError(f"expected {self.n_tets} Lame coefficients")
        _capi.check(_capi.lib().pbgb_vbd_set_material(self._h, mu.ctypes.data, lam.ctypes.data), self._h)

    # Device-pointer state access (|#vertices| x 3 float32 on the handle's device).  Stream-ordered
    # on the handle's stream: callers order their own work around them (synchronize()).
    def _get_device(self, which, ptr):
        fn = {"x": "pbgb_vbd_get_positions_device", "v": "pbgb_vbd_get_velocities_device",
              "vprev": "pbgb_vbd_get_previous_velocities_device"}[which]
        _capi.check(getattr(_capi.lib(), fn)(self._h, C.c_void_p(ptr)), self._h)

    def _set_device(self, which, ptr):
        fn = {"x": "pbgb_vbd_set_positions_device", "v": "pbgb_vbd_set_velocities_device",
              "vprev": "pbgb_vbd_set_previous_velocities_device"}[which]
        _capi.check(getattr(_capi.lib(), fn)(self._h, C.c_void_p(ptr)), self._h)

    def adjoint_reserve(self, slots, iterations):
        _capi.check(_capi.lib().pbgb_vbd_adjoint_reserve(self._h, int(slots), int(iterations)), self._h)

    def step_record(self, dt, iterations, substeps, slot):
        _capi.check(_capi.lib().pbgb_vbd_step_record(self._h, float(dt), int(iterations), int(substeps), int(slot)),
                    self._h)

    def step_adjoint(self, slot, substeps, xbar_ptr, vbar_ptr, dlogmu_ptr, dloglambda_ptr, vprevbar_ptr=None):
        """Reverses recorded substeps (device pointers); with ``vprevbar_ptr`` the adjoint of the
        previous velocities is carried too (pbgb_vbd_step_adjoint_state)."""
        L = _capi.lib()
        if vprevbar_ptr is None:
            rc = L.pbgb_vbd_step_adjoint(self._h, int(slot), int(substeps), C.c_void_p(xbar_ptr), C.c_void_p(vbar_ptr),
                                         C.c_void_p(dlogmu_ptr), C.c_void_p(dloglambda_ptr))
        else:
            rc = L.pbgb_vbd_step_adjoint_state(self._h, int(slot), int(substeps), C.c_void_p(xbar_ptr),
                                               C.c_void_p(vbar_ptr), C.c_void_p(vprevbar_ptr), C.c_void_p(dlogmu_ptr),
                                               C.c_void_p(dloglambda_ptr))
        _capi.check(rc, self._h)

    def trust_region_log(self):
        """Trust-region decisions of the last step: an (entries, 4) array, one row per (substep,
        iteration) -- t, rho (NaN when no stretched step was tried), squared radius after the
        iteration, flags (1 tried, 2 accepted)."""
        L, n = _capi.lib(), C.c_int32(0)
        _capi.check(L.pbgb_vbd_trust_region_log(self._h, None, 0, C.byref(n)), self._h)
        out = np.zeros((n.value, 4), dtype=np.float64)
        if n.value:
            _capi.check(L.pbgb_vbd_trust_region_log(self._h, out.ctypes.data, n.value, C.byref(n)), self._h)
        return out

    def objective(self, dt):
        """Backward-Euler objective at the current positions (FP64 device reduction)."""
        f = C.c_double()
        _capi.check(_capi.lib().pbgb_vbd_objective(self._h, float(dt), C.byref(f)), self._h)
        return f.value

    def gradient(self, dt):
        g = np.zeros((self.n_vertices, 3))
        _capi.check(_capi.lib().pbgb_vbd_gradient(self._h, float(dt), g.ctypes.data), self._h)
        return g.ravel()
