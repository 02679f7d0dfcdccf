"""ctypes access to the FP64 oracle (``oracle/_build/liboracle_vbd.so``) and, where it was built,
to the reference harness (``oracle/_ref/libpbat_ref.so``).

Test infrastructure: imported by the tests, the smoke check and the benchmark's CPU-baseline leg
only.  ``build_oracle()`` compiles the oracle on first use (g++ -fopenmp, a few seconds).
"""

from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_SO = ORACLE_DIR / "_build" / "liboracle_vbd.so"
REF_SO = ORACLE_DIR / "_ref" / "libpbat_ref.so"

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class OrcProblem(C.Structure):
    """Mirror of ``orc_problem`` (oracle/orc_problem.h)."""

    _fields_ = [
        ("nV", C.c_int32),
        ("nT", C.c_int32),
        ("X", C.c_void_p),
        ("T", C.c_void_p),
        ("m", C.c_void_p),
        ("GP", C.c_void_p),
        ("wg", C.c_void_p),
        ("mu", C.c_void_p),
        ("lam", C.c_void_p),
        ("GVGp", C.c_void_p),
        ("GVGe", C.c_void_p),
        ("GVGilocal", C.c_void_p),
        ("nPartitions", C.c_int32),
        ("Pptr", C.c_void_p),
        ("Padj", C.c_void_p),
        ("aext", C.c_void_p),
        ("strategy", C.c_int32),
        ("kD", C.c_double),
        ("detHZero", C.c_double),
        ("acceleration", C.c_int32),
        ("rho", C.c_double),
        ("chebyshev_formula", C.c_int32),
        ("semantics", C.c_int32),
        ("nthreads", C.c_int32), ("window", C.c_int32), ("nesterov_L", C.c_double),
        ("nesterov_start", C.c_int32), ("tr_eta", C.c_double), ("tr_tau", C.c_double), ("tr_curved", C.c_int32),
        ("tr_forced", C.c_void_p), ("tr_log", C.c_void_p),
    ]


def build_oracle(ref: bool = False) -> None:
    """Compile the oracle (and the reference harness when ``ref`` and the reference exist)."""
    targets = ["all"]
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), *targets], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_SO.exists():
            build_oracle()
        L = C.CDLL(str(ORACLE_SO))
        L.orc_construct.restype = C.c_int
        L.orc_construct.argtypes = [
            C.c_int32, C.c_int32, _f64p, _i32p, _f64p, _i32p, C.c_int32, C.c_int32, C.c_int32,
            _f64p, _f64p, _f64p, _i32p, _i32p, _i32p, _i32p, _i32p,
            C.POINTER(C.c_int32), _i32p, C.POINTER(C.c_int32),
        ]
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = [
            C.POINTER(OrcProblem), _f64p, _f64p, C.c_void_p, C.c_double, C.c_int32, C.c_int32,
            C.c_int32,
        ]
        L.orc_objective.restype = C.c_double
        L.orc_adjoint.restype = C.c_int
        L.orc_adjoint.argtypes = [C.POINTER(OrcProblem), _f64p, _f64p, _f64p, C.c_double, C.c_int32, C.c_int32,
                                  C.c_int32, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.orc_objective.argtypes = [C.POINTER(OrcProblem), _f64p, _f64p, C.c_double]
        L.orc_gradient.restype = None
        L.orc_gradient.argtypes = [C.POINTER(OrcProblem), _f64p, _f64p, C.c_double, _f64p]
        L.orc_snh_eval.restype = C.c_double
        L.orc_snh_eval.argtypes = [_f64p, C.c_double, C.c_double]
        L.orc_snh_grad.argtypes = [_f64p, C.c_double, C.c_double, _f64p]
        L.orc_snh_grad_hessian.argtypes = [_f64p, C.c_double, C.c_double, _f64p, _f64p]
        L.orc_chebyshev_omega.restype = C.c_double
        L.orc_chebyshev_omega.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_int32]
        L.orc_initial_positions.argtypes = [
            _f64p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_int32, _f64p,
        ]
        L.orc_vertex_solve.argtypes = [
            C.c_int32, _f64p, _f64p, _i32p, _f64p, _f64p, _f64p, _f64p, _f64p, C.c_double,
            C.c_double, C.c_double, C.c_double, C.c_double, _f64p, _f64p, _f64p,
        ]
        L.orc_num_threads.restype = C.c_int32
        _f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        _u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
        L.orc_morton.argtypes = [C.c_int32, _f32p, _f32p, _f32p, _f32p, _u32p]
        L.orc_bvh_build.argtypes = [C.c_int32, _f32p, _f32p, _f32p, _f32p, _u32p, _i32p, _i32p, _i32p,
                                    _i32p, _f32p, _f32p]
        L.orc_bvh_boxes.argtypes = [C.c_int32, _i32p, _i32p, _f32p, _f32p, _f32p, _f32p]
        L.orc_vertex_triangle_contact.argtypes = [_f64p] * 4 + [C.c_double] * 5 + [_f64p, _f64p]
        L.orc_run_contact.restype = C.c_int
        L.orc_run_contact.argtypes = [C.POINTER(OrcProblem), C.c_void_p, _f64p, _f64p, _f64p, C.c_double,
                                      C.c_int32, C.c_int32, C.c_int32]
        L.orc_overlaps.restype = C.c_int64
        L.orc_overlaps.argtypes = [C.c_int32, _f32p, _f32p, C.c_int32, _f32p, _f32p, _i32p, C.c_int64]
        L.orc_overlaps_all_pairs.restype = C.c_int64
        L.orc_overlaps_all_pairs.argtypes = [C.c_int32, _f32p, _f32p, C.c_int32, _f32p, _f32p, _i32p, C.c_int64]
        L.orc_ccd_vertex_triangle.restype = C.c_int
        L.orc_ccd_vertex_triangle.argtypes = [C.c_int32, _f64p, _f64p, C.c_int32, _i32p, C.c_int32, _i32p, _i32p,
                                              _f64p, _i32p]
        _u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
        L.orc_ccd_vertex_triangle_pairs.restype = C.c_int64
        L.orc_ccd_vertex_triangle_pairs.argtypes = [C.c_int32, _f64p, _f64p, C.c_int32, _i32p, C.c_int32, _i32p,
                                                    _i32p, _u8p, C.c_int64, _i32p, _i32p, _f64p]
        L.orc_ccd_edge_edge.restype = C.c_int64
        L.orc_ccd_edge_edge.argtypes = [C.c_int32, _f64p, _f64p, C.c_int32, _i32p, _i32p, _u8p, C.c_int64,
                                        _i32p, _i32p, _f64p]
        L.orc_edge_edge_ccd.argtypes = [_f64p, _f64p, _f64p]
        L.orc_point_triangle_ccd.restype = C.c_double
        L.orc_point_triangle_ccd.argtypes = [_f64p, _f64p]
        L.orc_dcd_contacts.restype = C.c_int
        L.orc_dcd_contacts.argtypes = [C.c_int32, _f64p, C.c_int32, _i32p, C.c_int32, _i32p, C.c_int32, _i32p,
                                       _i32p, _i32p, _i32p, _f64p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return REF_SO.exists()


def ref():
    """The reference harness, or None where it was not built (e.g. without the reference)."""
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            return None
        L = C.CDLL(str(REF_SO))
        L.ref_snh_eval.restype = C.c_double
        L.ref_snh_eval.argtypes = [_f64p, C.c_double, C.c_double]
        L.ref_snh_grad.argtypes = [_f64p, C.c_double, C.c_double, _f64p]
        L.ref_snh_grad_hessian.argtypes = [_f64p, C.c_double, C.c_double, _f64p, _f64p]
        L.ref_chebyshev_omega.restype = C.c_double
        L.ref_chebyshev_omega.argtypes = [C.c_int32, C.c_double, C.c_double]
        L.ref_initial_positions.argtypes = [
            _f64p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_int32, _f64p,
        ]
        L.ref_vertex_solve.argtypes = lib().orc_vertex_solve.argtypes
        L.ref_greedy_color.argtypes = [C.c_int32, _i32p, _i32p, C.c_int32, C.c_int32, _i32p]
        L.ref_morton3d.restype = C.c_uint32
        L.ref_morton3d.argtypes = [C.c_float, C.c_float, C.c_float]
        L.ref_run.restype = C.c_int
        L.ref_run.argtypes = lib().orc_run.argtypes
        fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.ref_vertex_triangle_contact_d.restype = C.c_double
        L.ref_vertex_triangle_contact_d.argtypes = [_f64p] * 4 + [C.c_double] * 4 + [_f64p, _f64p]
        L.ref_point_triangle_ccd.argtypes = [_f64p, _f64p, _f64p]
        L.ref_edge_edge_ccd.argtypes = [_f64p, _f64p, _f64p]
        L.ref_vertex_triangle_contact.restype = C.c_float
        L.ref_vertex_triangle_contact.argtypes = [
            fp, fp, fp, fp, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp,
        ]
        _ref = L
    return _ref


def construct(X, T, rho, dbc, ordering=2, selection=0):
    """Oracle ``Data::Construct`` precompute.  X: nV x 3, T: nT x 4 (row per entity)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.int32)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    dbc = np.ascontiguousarray(dbc, dtype=np.int32)
    nV, nT = X.shape[0], T.shape[0]
    out = dict(
        m=np.zeros(nV),
        GP=np.zeros(nT * 12),
        wg=np.zeros(nT),
        GVGp=np.zeros(nV + 1, np.int32),
        GVGe=np.zeros(4 * nT, np.int32),
        GVGilocal=np.zeros(4 * nT, np.int32),
        colors=np.zeros(nV, np.int32),
        Pptr=np.zeros(130, np.int32),
        Padj=np.zeros(max(nV, 1), np.int32),
    )
    nP = C.c_int32()
    nA = C.c_int32()
    rc = lib().orc_construct(
        nV, nT, X, T, rho, dbc, dbc.size, ordering, selection,
        out["m"], out["GP"], out["wg"], out["GVGp"], out["GVGe"], out["GVGilocal"],
        out["colors"], out["Pptr"], C.byref(nP), out["Padj"], C.byref(nA),
    )
    if rc != 0:
        raise ValueError(f"orc_construct failed with status {rc}")
    out["Pptr"] = out["Pptr"][: nP.value + 1].copy()
    out["Padj"] = out["Padj"][: nA.value].copy()
    out["GP"] = out["GP"].reshape(nT, 4, 3)
    return out


class OracleVbd:
    """FP64 CPU VBD integrator on a constructed problem (reference CPU semantics by default)."""

    def __init__(self, X, T, rho, mu, lam, dbc, v=None, aext=None, strategy=4, kD=0.0,
                 detHZero=1e-7, rho_chebyshev=None, chebyshev_formula=0, semantics=0,
                 nthreads=0, ordering=2, selection=0, data=None, anderson_window=None, nesterov=None,
                 trust_region=None, broyden_window=None):
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.T = np.ascontiguousarray(T, dtype=np.int32)
        nV = self.X.shape[0]
        self.data = data if data is not None else construct(self.X, self.T, rho, dbc, ordering, selection)
        self.mu = np.ascontiguousarray(mu, dtype=np.float64)
        self.lam = np.ascontiguousarray(lam, dtype=np.float64)
        dbc = np.asarray(dbc, dtype=np.int64)
        self.x = self.X.copy()
        self.v = np.zeros((nV, 3)) if v is None else np.array(v, dtype=np.float64)
        self.aext = np.tile([0.0, 0.0, -9.81], (nV, 1)) if aext is None else np.array(aext, dtype=np.float64)
        # Data::Construct zeroes velocity and external acceleration on Dirichlet vertices.
        self.v[dbc] = 0.0
        self.aext[dbc] = 0.0
        self.aext = np.ascontiguousarray(self.aext)
        self.vprev = np.zeros_like(self.v)
        self.GP = np.ascontiguousarray(self.data["GP"].reshape(-1))
        P = OrcProblem()
        P.nV, P.nT = nV, self.T.shape[0]
        keep = [self.X, self.T, self.data["m"], self.GP, self.data["wg"], self.mu, self.lam,
                self.data["GVGp"], self.data["GVGe"], self.data["GVGilocal"], self.data["Pptr"],
                self.data["Padj"], self.aext]
        self._keep = keep
        (P.X, P.T, P.m, P.GP, P.wg, P.mu, P.lam, P.GVGp, P.GVGe, P.GVGilocal, P.Pptr, P.Padj,
         P.aext) = [a.ctypes.data for a in keep]
        P.nPartitions = self.data["Pptr"].size - 1
        P.strategy = strategy
        P.kD = kD
        P.detHZero = detHZero
        P.acceleration = 0 if rho_chebyshev is None else 1
        P.rho = 1.0 if rho_chebyshev is None else rho_chebyshev
        if anderson_window is not None:
            if not 1 <= anderson_window <= 16:
                raise ValueError("Anderson window must be in [1, 16]")
            P.acceleration = 2
            P.window = int(anderson_window)
        if broyden_window is not None:
            if not 1 <= broyden_window <= 16:
                raise ValueError("Broyden window must be in [1, 16]")
            P.acceleration = 4
            P.window = int(broyden_window)
        if nesterov is not None:
            P.acceleration = 3
            P.nesterov_L, P.nesterov_start = float(nesterov[0]), int(nesterov[1])
        if trust_region is not None:
            P.acceleration = 5
            P.tr_eta, P.tr_tau, P.tr_curved = float(trust_region[0]), float(trust_region[1]), int(bool(trust_region[2]))
        P.chebyshev_formula = chebyshev_formula
        P.semantics = semantics
        P.nthreads = nthreads
        self.P = P

    def step(self, dt, iterations, substeps=1, nsteps=1, use_ref=False, trust_region_log=None):
        """Advance ``nsteps`` steps.  trust_region_log: a logged run's trust-region decisions
        (nsteps x substeps x iterations rows of t, rho, R^2, flags) to replay instead of the
        oracle's own.  With the trust-region strategy the oracle's own decisions are kept in
        ``self.trust_region_log`` afterwards (same layout)."""
        L = ref() if use_ref else lib()
        own = np.zeros((nsteps * substeps * iterations, 4))
        self.P.tr_log = own.ctypes.data
        self.trust_region_log = own
        forced = None
        if trust_region_log is not None:
            forced = np.ascontiguousarray(trust_region_log, dtype=np.float64)
            if forced.shape != (nsteps * substeps * iterations, 4):
                raise ValueError("trust_region_log must hold nsteps x substeps x iterations rows of 4")
            self.P.tr_forced = forced.ctypes.data
        try:
            rc = L.ref_run(C.byref(self.P), self.x, self.v, self.vprev.ctypes.data, dt, iterations,
                           substeps, nsteps) if use_ref else L.orc_run(
                C.byref(self.P), self.x, self.v, self.vprev.ctypes.data, dt, iterations, substeps,
                nsteps)
        finally:
            self.P.tr_forced = None
            self.P.tr_log = None
        if rc != 0:
            raise RuntimeError(f"oracle run failed: {rc}")

    def adjoint(self, dt, iterations, substeps, nsteps, xbar, vbar, vprevbar=None, with_vprev=False):
        """Reverse-mode derivative of ``nsteps`` steps from the current state (not advanced).
        xbar, vbar (nV x 3): dL/dx, dL/dv of the final state (vprevbar: dL/d of the final previous
        velocity, zero by default).  Returns dL/dx0, dL/dv0, dL/dlog(mu), dL/dlog(lambda) per tet
        (and dL/dvprev0 with ``with_vprev``)."""
        xb = np.array(xbar, dtype=np.float64, order="C")
        vb = np.array(vbar, dtype=np.float64, order="C")
        pb = np.zeros_like(xb) if vprevbar is None else np.array(vprevbar, dtype=np.float64, order="C")
        dmu = np.zeros(self.T.shape[0])
        dla = np.zeros(self.T.shape[0])
        rc = lib().orc_adjoint(C.byref(self.P), np.ascontiguousarray(self.x), np.ascontiguousarray(self.v),
                               np.ascontiguousarray(self.vprev), dt, iterations, substeps, nsteps, xb, vb, pb, dmu, dla)
        if rc != 0:
            raise RuntimeError(f"oracle adjoint failed: {rc}")
        return (xb, vb, dmu, dla, pb) if with_vprev else (xb, vb, dmu, dla)

    def objective(self, x, xtilde, dt):
        return lib().orc_objective(C.byref(self.P), np.ascontiguousarray(x), np.ascontiguousarray(xtilde), dt)

    def gradient(self, x, xtilde, dt):
        g = np.zeros(self.X.shape[0] * 3)
        lib().orc_gradient(C.byref(self.P), np.ascontiguousarray(x), np.ascontiguousarray(xtilde), dt, g)
        return g


class OrcContact(C.Structure):
    """Mirror of ``orc_contact`` (oracle/contact_oracle.cpp)."""

    _fields_ = [
        ("nSurfV", C.c_int32), ("V", C.c_void_p), ("nF", C.c_int32), ("F", C.c_void_p), ("B", C.c_void_p),
        ("XVA", C.c_void_p), ("FA", C.c_void_p), ("muC", C.c_double), ("muF", C.c_double),
        ("epsv", C.c_double), ("freq", C.c_int32), ("wmin", C.c_float * 3), ("wmax", C.c_float * 3),
        ("active", C.c_void_p), ("dupper", C.c_void_p), ("fc", C.c_void_p), ("forced_fc", C.c_void_p),
    ]


class OracleContactVbd(OracleVbd):
    """FP64 oracle of the contact-enabled step (GPU integrator semantics)."""

    def __init__(self, X, T, rho, mu, lam, dbc, V, F, B, muC=1e6, muF=0.3, epsv=1e-3, freq=1, **kw):
        kw.setdefault("semantics", 1)
        super().__init__(X, T, rho, mu, lam, dbc, **kw)
        X = self.X
        Fv = np.ascontiguousarray(F, dtype=np.int32)
        dbl = np.linalg.norm(np.cross(X[Fv[:, 1]] - X[Fv[:, 0]], X[Fv[:, 2]] - X[Fv[:, 0]]), axis=1)
        XVA = np.zeros(X.shape[0])
        for r in range(3):
            np.add.at(XVA, Fv[:, r], dbl / 6.0)
        self.cV = np.ascontiguousarray(V, dtype=np.int32)
        self.cF = Fv
        self.cB = np.ascontiguousarray(B, dtype=np.int32)
        self.XVA = XVA
        self.FA = dbl / 2.0
        self.active = np.zeros(self.cV.size, np.uint8)
        self.dupper = np.full(self.cV.size, float(np.finfo(np.float32).max))
        self.fc = np.full(X.shape[0] * 8, -1, np.int32)
        Cc = OrcContact()
        Cc.nSurfV, Cc.nF = self.cV.size, Fv.shape[0]
        Cc.V, Cc.F, Cc.B = self.cV.ctypes.data, Fv.ctypes.data, self.cB.ctypes.data
        Cc.XVA, Cc.FA = self.XVA.ctypes.data, self.FA.ctypes.data
        Cc.muC, Cc.muF, Cc.epsv, Cc.freq = muC, muF, epsv, freq
        Cc.active, Cc.dupper, Cc.fc = self.active.ctypes.data, self.dupper.ctypes.data, self.fc.ctypes.data
        # Scene box of the Morton codes: the rest-state bounding box, as on the device by default.
        Cc.wmin[:] = [float(c) for c in X.min(axis=0).astype(np.float32)]
        Cc.wmax[:] = [float(c) for c in X.max(axis=0).astype(np.float32)]
        self.C = Cc

    def step(self, dt, iterations, substeps=1, nsteps=1, use_ref=False, trust_region_log=None, contact_lists=None):
        """contact_lists (replay): the lists (|#vertices| x 8 per list update, e.g. the device's) to
        use instead of the oracle's own nearest-triangle queries."""
        own = np.zeros((nsteps * substeps * iterations, 4))
        self.P.tr_log = own.ctypes.data
        self.trust_region_log = own
        lists = None
        if contact_lists is not None:
            updates = (nsteps * substeps + self.C.freq - 1) // self.C.freq
            lists = np.ascontiguousarray(contact_lists, dtype=np.int32).reshape(-1)
            if lists.size != updates * 8 * self.X.shape[0]:
                raise ValueError("contact_lists must hold |#vertices| x 8 entries per list update")
            self.C.forced_fc = lists.ctypes.data
        forced = None
        if trust_region_log is not None:
            forced = np.ascontiguousarray(trust_region_log, dtype=np.float64)
            if forced.shape != (nsteps * substeps * iterations, 4):
                raise ValueError("trust_region_log must hold nsteps x substeps x iterations rows of 4")
            self.P.tr_forced = forced.ctypes.data
        try:
            rc = lib().orc_run_contact(C.byref(self.P), C.addressof(self.C), self.x, self.v, self.vprev, dt,
                                       iterations, substeps, nsteps)
        finally:
            self.P.tr_forced = None
            self.P.tr_log = None
            self.C.forced_fc = None
        if rc != 0:
            raise RuntimeError(f"oracle run failed: {rc}")


def bvh_build(lo, hi, wmin, wmax):
    """Oracle LBVH build; lo, hi: n x 3 float32.  Returns a dict of the sorted codes, leaf order,
    child (n-1 x 2), parent (2n-1), rightmost (n-1 x 2) and internal boxes."""
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    hi = np.ascontiguousarray(hi, dtype=np.float32)
    n = lo.shape[0]
    out = dict(codes=np.zeros(n, np.uint32), inds=np.zeros(n, np.int32),
               child=np.zeros(max(2 * (n - 1), 1), np.int32), parent=np.zeros(2 * n - 1, np.int32),
               rightmost=np.zeros(max(2 * (n - 1), 1), np.int32), ilo=np.zeros((max(n - 1, 1), 3), np.float32),
               ihi=np.zeros((max(n - 1, 1), 3), np.float32))
    lib().orc_bvh_build(n, lo, hi, np.asarray(wmin, np.float32), np.asarray(wmax, np.float32), out["codes"],
                        out["inds"], out["child"], out["parent"], out["rightmost"], out["ilo"], out["ihi"])
    out["child"] = out["child"][: 2 * (n - 1)].reshape(-1, 2)
    out["rightmost"] = out["rightmost"][: 2 * (n - 1)].reshape(-1, 2)
    out["ilo"], out["ihi"] = out["ilo"][: n - 1], out["ihi"][: n - 1]
    return out


def bvh_boxes(child, inds, lo, hi):
    n = inds.size
    ilo = np.zeros((max(n - 1, 1), 3), np.float32)
    ihi = np.zeros((max(n - 1, 1), 3), np.float32)
    lib().orc_bvh_boxes(n, np.ascontiguousarray(child, np.int32).ravel(), np.ascontiguousarray(inds, np.int32),
                        np.ascontiguousarray(lo, np.float32), np.ascontiguousarray(hi, np.float32), ilo, ihi)
    return ilo[: n - 1], ihi[: n - 1]


def morton(lo, hi, wmin, wmax):
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    codes = np.zeros(lo.shape[0], np.uint32)
    lib().orc_morton(lo.shape[0], lo, np.ascontiguousarray(hi, np.float32), np.asarray(wmin, np.float32),
                     np.asarray(wmax, np.float32), codes)
    return codes


def overlaps(lo, hi, qlo, qhi, all_pairs=False):
    """Overlapping (query, box) pairs (n x 2, ordered by query then box), every candidate decided
    by the closed-box test; ``all_pairs`` tests every pair instead of the x-sorted candidates."""
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    qlo = np.ascontiguousarray(qlo, np.float32)
    qhi = np.ascontiguousarray(qhi, np.float32)
    fn = lib().orc_overlaps_all_pairs if all_pairs else lib().orc_overlaps
    cap = 1 << 20
    while True:
        pairs = np.zeros(2 * cap, np.int32)
        c = fn(lo.shape[0], lo, hi, qlo.shape[0], qlo, qhi, pairs, cap)
        if c <= cap:
            return pairs[: 2 * c].reshape(-1, 2)
        cap = int(c)


def primal_graph(T, nV):
    """CSR vertex graph (neighbours including self, ascending) of a tet mesh."""
    T = np.asarray(T, dtype=np.int64)
    rows = np.repeat(T, 4, axis=1).ravel()
    cols = np.tile(T, (1, 4)).ravel()
    key = np.unique(rows * nV + cols)
    r, c = key // nV, key % nV
    ptr = np.zeros(nV + 1, np.int32)
    np.add.at(ptr, r + 1, 1)
    return np.cumsum(ptr).astype(np.int32), c.astype(np.int32)


def dcd_contacts(x, T, F, V, B):
    """Discrete half of the CPU multibody mesh detector (oracle/contact_oracle.cpp
    orc_dcd_contacts): for each collision vertex V[q], the body it penetrates (-1: none), its
    nearest surface triangles of that body (exact ties, -1 padded, 8 per vertex) and their squared
    distance.  x (nV x 3), T (nT x 4), F (nF x 3), V (collision vertices), B (body per vertex)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.int32)
    F = np.ascontiguousarray(F, dtype=np.int32)
    V = np.ascontiguousarray(V, dtype=np.int32)
    B = np.ascontiguousarray(B, dtype=np.int32)
    n = V.size
    body = np.empty(n, np.int32)
    nearest = np.empty((n, 8), np.int32)
    d2 = np.empty(n, np.float64)
    rc = lib().orc_dcd_contacts(x.shape[0], x, T.shape[0], T, F.shape[0], F, n, V, B, body, nearest, d2)
    if rc != 0:
        raise RuntimeError("orc_dcd_contacts failed")
    return body, nearest, d2


def edge_edge_ccd(xt, x):
    """One edge-edge CCD query of the oracle (oracle/contact_oracle.cpp edge_edge_ccd): xt, x are
    4 x 3 (p1, q1, p2, q2 at the start and the end of the step); returns (t, u, v), t = -1 for no
    crossing."""
    out = np.zeros(3)
    lib().orc_edge_edge_ccd(np.ascontiguousarray(xt, dtype=np.float64), np.ascontiguousarray(x, dtype=np.float64), out)
    return out


def point_triangle_ccd(xt, x):
    """One point-triangle CCD query of the oracle: xt, x are 4 x 3 (x, a, b, c); returns t or -1."""
    return lib().orc_point_triangle_ccd(np.ascontiguousarray(xt, dtype=np.float64),
                                        np.ascontiguousarray(x, dtype=np.float64))


def _grow(call):
    """Runs a capacity-bounded pair query twice when the first capacity was short."""
    cap = 1024
    while True:
        n, out = call(cap)
        if n <= cap:
            return n, out
        cap = int(n)


def ccd_vertex_triangle_pairs(xt, x, F, V, B, penetrating=None):
    """Every vertex-triangle CCD hit of the CPU multibody detector (oracle/contact_oracle.cpp
    orc_ccd_vertex_triangle_pairs): (vertex, triangle, time of impact) arrays, ordered by
    (vertex, triangle).  penetrating: optional bool per vertex (skipped vertices)."""
    xt = np.ascontiguousarray(xt, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    V = np.ascontiguousarray(V, dtype=np.int32)
    B = np.ascontiguousarray(B, dtype=np.int32)
    mask = np.ascontiguousarray(np.zeros(x.shape[0], bool) if penetrating is None else penetrating, dtype=np.uint8)

    def call(cap):
        v, f, t = np.empty(cap, np.int32), np.empty(cap, np.int32), np.empty(cap, np.float64)
        n = lib().orc_ccd_vertex_triangle_pairs(x.shape[0], xt, x, F.shape[0], F, V.size, V, B, mask, cap, v, f, t)
        return n, (v, f, t)

    n, (v, f, t) = _grow(call)
    return v[:n].copy(), f[:n].copy(), t[:n].copy()


def ccd_edge_edge(xt, x, E, B, penetrating=None):
    """Every edge-edge CCD hit of the CPU multibody detector (oracle/contact_oracle.cpp
    orc_ccd_edge_edge): (first edge, second edge, (t, u, v)) with the first edge on the lower
    body, ordered by (first, second).  E: nE x 2 collision edges; penetrating as above."""
    xt = np.ascontiguousarray(xt, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    E = np.ascontiguousarray(E, dtype=np.int32)
    B = np.ascontiguousarray(B, dtype=np.int32)
    mask = np.ascontiguousarray(np.zeros(x.shape[0], bool) if penetrating is None else penetrating, dtype=np.uint8)

    def call(cap):
        a, b, r = np.empty(cap, np.int32), np.empty(cap, np.int32), np.empty((cap, 3), np.float64)
        n = lib().orc_ccd_edge_edge(x.shape[0], xt, x, E.shape[0], E, B, mask, cap, a, b, r)
        return n, (a, b, r)

    n, (a, b, r) = _grow(call)
    return a[:n].copy(), b[:n].copy(), r[:n].copy()


def multibody_all_pairs(XT, X, XK, V, E, F, T, B):
    """The CPU multibody detector's active-set update (sim/contact/MultibodyMeshMixedCcdDcd.h
    UpdateActiveSet 561-583; the Python binding's all_pairs): the discrete half at XK marks
    penetrating vertices and reports each with its nearest triangles of the body it penetrates;
    the continuous half on XT -> X reports every vertex-triangle hit of the other collision
    vertices and every edge-edge hit of edges without a penetrating end point.  Returns
    (VTv, VTf, EEei, EEej) like the binding; the order is the oracle's (sets match the
    reference's)."""
    body, nearest, _ = dcd_contacts(XK, T, F, V, B)
    pen = np.zeros(np.asarray(XK).shape[0], bool)
    pen[np.asarray(V)[body >= 0]] = True
    vt_v, vt_f = [], []
    for q in np.nonzero(body >= 0)[0]:
        for f in nearest[q][nearest[q] >= 0]:
            vt_v.append(int(V[q]))
            vt_f.append(int(f))
    cv, cf, _ = ccd_vertex_triangle_pairs(XT, X, F, V, B, pen)
    ei, ej, _ = ccd_edge_edge(XT, X, E, B, pen)
    return (np.array(vt_v + cv.tolist(), np.int64), np.array(vt_f + cf.tolist(), np.int64),
            ei.astype(np.int64), ej.astype(np.int64))


def ccd_vertex_triangle(xt, x, F, V, B):
    """Vertex-triangle CCD of the CPU multibody detector (oracle/contact_oracle.cpp
    orc_ccd_vertex_triangle): for each collision vertex V[q], the earliest time of impact in [0, 1]
    of its linear trajectory xt -> x with a linearly moving triangle of another body (-1: none) and
    that triangle."""
    xt = np.ascontiguousarray(xt, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    V = np.ascontiguousarray(V, dtype=np.int32)
    B = np.ascontiguousarray(B, dtype=np.int32)
    toi = np.empty(V.size, np.float64)
    tri = np.empty(V.size, np.int32)
    rc = lib().orc_ccd_vertex_triangle(x.shape[0], xt, x, F.shape[0], F, V.size, V, B, toi, tri)
    if rc != 0:
        raise RuntimeError("orc_ccd_vertex_triangle failed")
    return toi, tri
