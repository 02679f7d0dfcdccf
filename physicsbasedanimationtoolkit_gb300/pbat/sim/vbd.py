"""``pbat.sim.vbd``: the VBD problem builder and the reference-CPU-semantics integrator.

Mirrors the reference bindings ``bindings/pypbat/sim/vbd/Data.cpp:16-274`` (``Data`` fluent
builder, enums) and ``bindings/pypbat/sim/vbd/Integrator.cpp:30-90`` (``Integrator``).  Arrays use
the reference's shapes: positions ``3 x |#vertices|``, tetrahedra ``4 x |#tets|``.
"""

from __future__ import annotations

import enum

import numpy as np

from ... import _capi
from ..._integrator import IntegratorBase, SEMANTICS_CPU
from ..graph import GreedyColorOrderingStrategy, GreedyColorSelectionStrategy


class InitializationStrategy(enum.IntEnum):
    """sim/vbd/Enums.h:9-15."""

    Position = 0
    Inertia = 1
    KineticEnergyMinimum = 2
    AdaptiveVbd = 3
    AdaptivePbat = 4


class AccelerationStrategy(enum.IntEnum):
    """sim/vbd/Enums.h:21-28 (``Base`` is the reference's ``None``)."""

    Base = 0
    Chebyshev = 1
    Anderson = 2
    Nesterov = 3
    Broyden = 4
    TrustRegion = 5


Position = InitializationStrategy.Position
Inertia = InitializationStrategy.Inertia
KineticEnergyMinimum = InitializationStrategy.KineticEnergyMinimum
AdaptiveVbd = InitializationStrategy.AdaptiveVbd
AdaptivePbat = InitializationStrategy.AdaptivePbat


def _lame(E, nu):
    mu = E / (2.0 * (1.0 + nu))
    lam = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return mu, lam


class Data:
    """VBD simulation configuration (sim/vbd/Data.h:14-247)."""

    def __init__(self):
        self.X = np.zeros((3, 0))
        self.E = np.zeros((4, 0), dtype=np.int64)
        self.B = np.zeros(0, dtype=np.int64)
        self.V = np.zeros(0, dtype=np.int64)
        self.F = np.zeros((3, 0), dtype=np.int64)
        self.XVA = np.zeros(0)
        self.FA = np.zeros(0)
        self.x = np.zeros((3, 0))
        self.v = np.zeros((3, 0))
        self.aext = np.zeros((3, 0))
        self.m = np.zeros(0)
        self.xt = np.zeros((3, 0))
        self.xtilde = np.zeros((3, 0))
        self.vt = np.zeros((3, 0))
        self.wg = np.zeros(0)
        self.GP = np.zeros((4, 0))
        self.rhoe = np.zeros(0)
        self.lame = np.zeros((2, 0))
        self.GVGp = np.zeros(0, dtype=np.int64)
        self.GVGe = np.zeros(0, dtype=np.int64)
        self.GVGilocal = np.zeros(0, dtype=np.int64)
        self.muD = 1.0
        self.dbc = np.zeros(0, dtype=np.int64)
        self.vertex_coloring_ordering = GreedyColorOrderingStrategy.LargestDegree
        self.vertex_coloring_selection = GreedyColorSelectionStrategy.LeastUsed
        self.colors = np.zeros(0, dtype=np.int64)
        self.Pptr = np.zeros(0, dtype=np.int64)
        self.Padj = np.zeros(0, dtype=np.int64)
        self.strategy = InitializationStrategy.AdaptivePbat
        self.kD = 0.0
        self.muC = 1e6
        self.muF = 0.3
        self.epsv = 1e-3
        self.active_set_update_frequency = 1
        self.detH_zero = 1e-7
        self.eAcceleration = AccelerationStrategy.Base
        self.rho = 1.0
        self.chebyshev_formula = 0
        self.window_size = 5
        self._constructed = False

    # -- builder -------------------------------------------------------------------------------
    def with_volume_mesh(self, X, T):
        """Sets the FEM mesh: ``X`` 3 x |#nodes| positions, ``T`` 4 x |#elements| tetrahedra."""
        self.X = np.array(X, dtype=np.float64, order="F", ndmin=2)
        self.E = np.array(T, dtype=np.int64, order="F", ndmin=2)
        if self.X.shape[0] != 3 or self.E.shape[0] != 4:
            raise ValueError("Expected X of shape 3 x |#nodes| and T of shape 4 x |#elements|")
        if self.B.size == 0:
            self.B = np.ones(self.X.shape[1], dtype=np.int64)
        return self

    def with_surface_mesh(self, V, F):
        """Sets the collision mesh: vertex indices ``V`` and 3 x |#triangles| ``F``."""
        self.V = np.asarray(V, dtype=np.int64).ravel()
        self.F = np.array(F, dtype=np.int64, ndmin=2)
        X = self.X
        AB = X[:, self.F[1]] - X[:, self.F[0]]
        AC = X[:, self.F[2]] - X[:, self.F[0]]
        dbl = np.linalg.norm(np.cross(AB.T, AC.T), axis=1)
        self.XVA = np.zeros(X.shape[1])
        for r in range(3):
            np.add.at(self.XVA, self.F[r], dbl / 6.0)
        self.FA = dbl / 2.0
        return self

    def with_bodies(self, B):
        self.B = np.asarray(B, dtype=np.int64).ravel()
        return self

    def with_velocity(self, v):
        self.v = np.array(v, dtype=np.float64, ndmin=2)
        return self

    def with_acceleration(self, a):
        self.aext = np.array(a, dtype=np.float64, ndmin=2)
        return self

    def with_material(self, rhoe, mue, lambdae):
        self.rhoe = np.asarray(rhoe, dtype=np.float64).ravel()
        self.lame = np.stack(
            [np.asarray(mue, dtype=np.float64).ravel(), np.asarray(lambdae, dtype=np.float64).ravel()]
        )
        return self

    def with_dirichlet_vertices(self, dbc, muD=1.0, input_sorted=True):
        dbc = np.asarray(dbc, dtype=np.int64).ravel()
        self.dbc = dbc if input_sorted else np.sort(dbc)
        self.muD = float(muD)
        return self

    def with_vertex_coloring_strategy(self, ordering, selection):
        self.vertex_coloring_ordering = GreedyColorOrderingStrategy(int(ordering))
        self.vertex_coloring_selection = GreedyColorSelectionStrategy(int(selection))
        return self

    def with_initialization_strategy(self, strategy):
        self.strategy = InitializationStrategy(int(strategy))
        return self

    def with_rayleigh_damping(self, kD):
        self.kD = float(kD)
        return self

    def with_contact_parameters(self, muC, muF, epsv):
        self.muC, self.muF, self.epsv = float(muC), float(muF), float(epsv)
        return self

    def with_active_set_update_frequency(self, frequency):
        self.active_set_update_frequency = int(frequency)
        return self

    def with_hessian_determinant_zero(self, zero):
        self.detH_zero = float(zero)
        return self

    def with_chebyshev_acceleration(self, rho, formula="reference"):
        """Chebyshev semi-iterative acceleration with spectral radius estimate ``rho``.

        ``formula="reference"`` reproduces the reference's weight recurrence as written
        (``4/4 - rho^2 omega``, sim/vbd/Kernels.h:96-102); ``"textbook"`` uses
        ``4/(4 - rho^2 omega)``.
        """
        self.rho = float(rho)
        self.eAcceleration = AccelerationStrategy.Chebyshev
        self.chebyshev_formula = {"reference": 0, "textbook": 1}[formula]
        return self

    def with_anderson_acceleration(self, window_size):
        self.window_size = int(window_size)
        self.eAcceleration = AccelerationStrategy.Anderson
        return self

    def with_broyden_acceleration(self, window_size):
        self.window_size = int(window_size)
        self.eAcceleration = AccelerationStrategy.Broyden
        return self

    def with_nesterov_acceleration(self, L, start=3):
        """Nesterov-accelerated VBD (sim/vbd/NesterovIntegrator.cpp) with Lipschitz constant L,
        accelerating the iterations after ``start``."""
        self.nesterov_L = float(L)
        self.nesterov_start = int(start)
        self.eAcceleration = AccelerationStrategy.Nesterov
        return self

    def with_trust_region_acceleration(self, eta, tau, curved):
        """Trust-region accelerated VBD (gpu/impl/vbd/TrustRegionIntegrator.cu): energy-reduction
        threshold ``eta``, radius growth factor ``tau`` and the curved or linear accelerated path."""
        self.eta = float(eta)
        self.tau = float(tau)
        self.curved = bool(curved)
        self.eAcceleration = AccelerationStrategy.TrustRegion
        return self

    def construct(self, validate=True):
        """Precompute masses, shape-function gradients, adjacency and the colouring on the host
        (sim/vbd/Data.cpp:179-308) through ``pbgb_vbd_data_construct``."""
        L = _capi.lib()
        nV, nT = self.X.shape[1], self.E.shape[1]
        self.x = self.X.copy(order="F")
        if self.xt.size == 0:
            self.xt = self.x.copy(order="F")
        if self.v.size == 0:
            self.v = np.zeros((3, nV), order="F")
        if self.aext.size == 0:
            self.aext = np.tile(np.array([[0.0], [0.0], [-9.81]]), (1, nV))
        self.xtilde = np.zeros((3, nV), order="F")
        self.vt = np.zeros((3, nV), order="F")
        if self.lame.size == 0:
            mu, lam = _lame(1e6, 0.45)
            self.lame = np.stack([np.full(nT, mu), np.full(nT, lam)])
        if self.rhoe.size == 0:
            self.rhoe = np.full(nT, 1e3)
        Xr = _capi.f64(self.X.T)
        Tr = _capi.i32(self.E.T)
        rho = _capi.f64(self.rhoe)
        dbc = _capi.i32(self.dbc)
        m = np.zeros(nV)
        GP = np.zeros(nT * 12)
        wg = np.zeros(nT)
        GVGp = np.zeros(nV + 1, np.int32)
        GVGe = np.zeros(4 * nT, np.int32)
        GVGi = np.zeros(4 * nT, np.int32)
        colors = np.zeros(nV, np.int32)
        Pptr = np.zeros(129, np.int32)
        Padj = np.zeros(max(nV, 1), np.int32)
        nP = _capi.C.c_int32()
        nA = _capi.C.c_int32()
        rc = L.pbgb_vbd_data_construct(
            nV, nT, _capi.ptr(Xr), _capi.ptr(Tr), _capi.ptr(rho), _capi.ptr(dbc), dbc.size,
            int(self.vertex_coloring_ordering), int(self.vertex_coloring_selection),
            _capi.ptr(m), _capi.ptr(GP), _capi.ptr(wg), _capi.ptr(GVGp), _capi.ptr(GVGe),
            _capi.ptr(GVGi), _capi.ptr(colors), _capi.ptr(Pptr), _capi.C.byref(nP), _capi.ptr(Padj),
            _capi.C.byref(nA),
        )
        _capi.check(rc)
        self.m = m
        # Reference layout: GP is 4 x (3 |#elements|), column 3e+d holds d/dX_d of the 4 shape
        # functions of element e.
        self._GP_rows = GP  # nT x 4 x 3 row-major, what the C ABI consumes
        self.GP = GP.reshape(nT, 4, 3).transpose(1, 0, 2).reshape(4, 3 * nT)
        self.wg = wg
        self.GVGp, self.GVGe, self.GVGilocal = GVGp.astype(np.int64), GVGe.astype(np.int64), GVGi.astype(np.int64)
        self.colors = colors.astype(np.int64)
        self.Pptr = Pptr[: nP.value + 1].astype(np.int64)
        self.Padj = Padj[: nA.value].astype(np.int64)
        # Dirichlet vertices carry no velocity or external force (Data.cpp:236-243).
        self.v = np.array(self.v, dtype=np.float64)
        self.aext = np.array(self.aext, dtype=np.float64)
        self.v[:, self.dbc] = 0.0
        self.aext[:, self.dbc] = 0.0
        if validate:
            ok = (
                self.x.shape == self.xt.shape == self.v.shape == self.aext.shape == (3, nV)
                and self.m.size == nV
                and self.B.size == nV
            )
            if not ok:
                raise ValueError(
                    f"x, v, aext, m and B must have same #columns={nV} as x, and 3 rows (except m and B)"
                )
            if self.eAcceleration == AccelerationStrategy.Chebyshev and not (0.0 < self.rho < 1.0):
                raise ValueError("Expected 0 < rho < 1")
            if self.eAcceleration in (AccelerationStrategy.Anderson, AccelerationStrategy.Broyden) and self.window_size < 1:
                raise ValueError("Expected m > 0")
            if self.eAcceleration == AccelerationStrategy.Nesterov:
                if not getattr(self, "nesterov_L", 1.0) > 0.0:
                    raise ValueError("Expected L > 0")
                if getattr(self, "nesterov_start", 3) < 0:
                    raise ValueError("Expected start >= 0")
            if self.eAcceleration == AccelerationStrategy.TrustRegion:
                if getattr(self, "eta", 0.2) < 0:
                    raise ValueError("Expected eta >= 0")
                if getattr(self, "tau", 2.0) <= 1:
                    raise ValueError("Expected tau > 1")
        self._constructed = True
        return self


class Integrator(IntegratorBase):
    """``pbat.sim.vbd.Integrator`` (sim/vbd/Integrator.h:15-63): the reference CPU integrator's
    step semantics, computed on the GPU in FP32.  ``x`` and ``v`` are FP64 3 x |#nodes| arrays
    like the reference's ``data.x``/``data.v``."""

    def __init__(self, data):
        super().__init__(data, SEMANTICS_CPU)

    def step(self, dt, iterations, substeps=1):
        self._step(dt, iterations, substeps)

    def trace_next_step(self, path=".", t=-1):
        """Trace the next step: per substep, {path}/{t}.{s}.f.mtx, .grad.mtx and .x.mtx hold the
        objective, its gradient and the positions at every iterate (Matrix Market)."""
        _capi.check(_capi.lib().pbgb_vbd_trace_next_step(self._h, str(path).encode(), int(t)), self._h)

    @property
    def x(self):
        return self._get("x").astype(np.float64)

    @x.setter
    def x(self, value):
        self._set("x", value)

    @property
    def v(self):
        return self._get("v").astype(np.float64)

    @v.setter
    def v(self, value):
        self._set("v", value)

    @property
    def strategy(self):
        return self._strategy

    @strategy.setter
    def strategy(self, s):
        self._set_strategy(s)

    @property
    def kD(self):
        return self._kD

    @kD.setter
    def kD(self, kD):
        self._set_kD(kD)

    @property
    def detH_residual(self):
        return self._detH

    @detH_residual.setter
    def detH_residual(self, z):
        self._set_detH(z)
