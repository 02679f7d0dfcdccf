"""Vertex-triangle contact on the device: the reference doctest's active-set scenario, and
contact-enabled steps against the FP64 oracle."""

import ctypes as C

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import _capi, meshgen, pbat

pytestmark = pytest.mark.gpu


class Ccd:
    def __init__(self, nV, V, F, B):
        self.V = np.ascontiguousarray(V, np.int32)
        self.F = np.ascontiguousarray(F, np.int32)
        self.B = np.ascontiguousarray(B, np.int32)
        h = C.c_void_p()
        _capi.check_ccd(_capi.lib().pbgb_ccd_create(nV, self.V.size, self.V.ctypes.data, self.F.shape[0],
                                                    self.F.ctypes.data, self.B.ctypes.data, C.byref(h)))
        self.h = h

    def __del__(self):
        _capi.lib().pbgb_ccd_destroy(self.h)

    def call(self, name, *arrays):
        arrays = [np.ascontiguousarray(a, np.float32) for a in arrays]
        _capi.check_ccd(getattr(_capi.lib(), name)(self.h, *[a.ctypes.data for a in arrays]), self.h)

    def get(self):
        n = self.V.size
        active = np.zeros(n, np.uint8)
        nn = np.zeros(8 * n, np.int32)
        dup = np.zeros(n, np.float32)
        na = C.c_int32()
        _capi.check_ccd(_capi.lib().pbgb_ccd_get(self.h, active.ctypes.data, nn.ctypes.data, dup.ctypes.data,
                                                 C.byref(na)), self.h)
        return active, nn.reshape(n, 8), dup, na.value


def test_two_tets_active_set_reference_scenario():
    """gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:232-328: the bottom tet's top vertex passes
    through the top tet's bottom face."""
    XT = np.array([[0, 1, 0, 0.1, 0, 1, 0, 0.1],
                   [0, 0, 1, 0.1, 0, 0, 1, 0.1],
                   [0, 0, 0, 1, 1.01, 1.01, 1.01, 2.01]], np.float32)
    F = np.array([[0, 1, 2, 0, 4, 5, 6, 4], [1, 2, 0, 2, 5, 6, 4, 6], [3, 3, 3, 1, 7, 7, 7, 5]]).T
    V = np.arange(8)
    B = np.array([0, 0, 0, 0, 1, 1, 1, 1])
    X = XT.copy()
    X[2, :4] += 0.01
    X[2, 4:] -= 0.01
    c = Ccd(8, V, F, B)
    c.call("pbgb_ccd_initialize", XT.T, X.T, np.array([0, 0, 0]), np.array([1, 1, 2.01]))
    active, nn, dup, na = c.get()
    assert na == 4
    assert active.sum() == 4
    assert active[3] == 1
    c.call("pbgb_ccd_update", X.T)
    active, nn, dup, na = c.get()
    for v in range(8):
        assert (nn[v] >= 0).any() == bool(active[v])
    c.call("pbgb_ccd_finalize", X.T)


def small_scene():
    return meshgen.contact_scene_workload(n_cubes_side=2, cube_hexes=3, slab_hexes=(8, 8, 1), gap=0.01)


def contact_data(w, muC=1e7, strategy=2):
    return (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
            .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
            .with_contact_parameters(muC, 0.3, 1e-3).with_initialization_strategy(strategy).construct())


def plane_distances(x, F, fc, verts):
    """Signed distance of each collision vertex to the plane of every triangle listed for it
    (+inf where none is listed); the minimum |distance| per vertex is returned."""
    out = np.full(len(verts), np.inf)
    for q, i in enumerate(verts):
        for f in fc[i][fc[i] >= 0]:
            a, b, c = x[F[f]]
            n = np.cross(b - a, c - a)
            out[q] = min(out[q], abs((x[i] - a) @ n) / np.linalg.norm(n))
    return out


def test_contact_steps_match_oracle():
    """20 contact-enabled steps against the FP64 oracle.  Positions agree to 1e-4 of the scene
    diagonal.  The active flags agree exactly at the first step with contacts; afterwards a flag may
    differ only for a vertex that at some step lay within 1e-3 of the diagonal of a listed
    triangle's plane (finalize decides on the side of that plane, and FP32 and FP64 iterates may
    fall on opposite sides of it; a flag persists once the vertex leaves the search radius, as in
    gpu/impl/contact/VertexTriangleMixedCcdDcd.cu:186-223)."""
    w = small_scene()
    I = pbat.gpu.vbd.Integrator(contact_data(w))
    R = O.OracleContactVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], w["V"], w["F"], w["B"],
                           muC=1e7, strategy=2)
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    verts = np.asarray(w["V"])
    F = np.asarray(w["F"])
    near = np.full(verts.size, np.inf)
    errs = []
    first_checked = False
    for _ in range(20):
        I.step(1 / 60, 20, 1)
        R.step(1 / 60, 20, 1, 1)
        x = I.x.T.astype(np.float64)
        errs.append(np.abs(x - R.x).max() / diag)
        fc, active = I.contacts()
        rfc = R.fc.reshape(-1, 8)
        if not first_checked and (active.any() or R.active.any()):
            np.testing.assert_array_equal(active.astype(bool), R.active.astype(bool))
            first_checked = True
        for xs in (x, R.x):
            for lists in (fc, rfc):
                near = np.minimum(near, plane_distances(xs, F, lists, verts))
    assert first_checked and active.sum() > 0
    assert max(errs) <= 1e-4, errs
    differ = np.nonzero(active.astype(bool) != R.active.astype(bool))[0]
    assert differ.size <= 0.05 * verts.size, differ
    assert (near[differ] <= 1e-3 * diag).all(), (differ, near[differ] / diag)


def test_contact_scene_of_sixteen_cubes_runs():
    """16 cubes of 16^3 hexes on a 64x64x2 slab (91,283 vertices, 66,560 surface triangles)."""
    w = meshgen.contact_scene_workload()
    I = pbat.gpu.vbd.Integrator(contact_data(w))
    z0 = w["X"][w["B"] > 0, 2].min()
    for _ in range(8):
        I.step(1 / 60, 30, 1)
    x = I.x.T
    assert np.isfinite(x).all()
    zc = x[w["B"] > 0, 2]
    # The penalty (muC = 1e7) lets the cubes sink a few centimetres into the slab at most.
    assert zc.min() < z0 and zc.min() > -0.05
    fc, active = I.contacts()
    assert active.sum() > 100
    assert (fc >= 0).any()


def test_staged_sweep_equals_gathering_sweep_with_contact():
    w = small_scene()
    A = pbat.gpu.vbd.Integrator(contact_data(w))
    B = pbat.gpu.vbd.Integrator(contact_data(w))
    B.staged_sweep = False
    for _ in range(6):
        A.step(1 / 60, 15, 1)
        B.step(1 / 60, 15, 1)
    np.testing.assert_array_equal(A.x, B.x)
    fa, aa = A.contacts()
    fb, ab = B.contacts()
    np.testing.assert_array_equal(fa, fb)
    np.testing.assert_array_equal(aa, ab)


def test_active_set_agrees_with_cpu_multibody_detector():
    """The GPU path's active set against the discrete half of the CPU multibody mesh detector
    (sim/contact/MultibodyMeshMixedCcdDcd.h, restated in oracle/contact_oracle.cpp), an independent
    algorithm: a 4x4x4-hex cube moved from 5 cm above a slab to 5 cm inside it.  After initialize,
    update and finalize, a collision vertex is active on the device exactly when the CPU detector
    finds it inside a tetrahedron of the other body, and the device's nearest listed triangle is at
    the CPU's nearest squared distance (FP32 tolerance)."""
    w = meshgen.contact_scene_workload(n_cubes_side=1, cube_hexes=4, slab_hexes=(8, 8, 1), cell=1.0)
    XT, T, F, V, B = w["X"].copy(), w["T"], w["F"], w["V"], w["B"]
    X = XT.copy()
    X[B == 1, 2] -= 0.1  # the cube's bottom from 5 cm above the slab's top to 5 cm below it
    body, nearest, d2 = O.dcd_contacts(X, T, F, V, B)
    c = Ccd(X.shape[0], V, F, B)
    lo, hi = np.minimum(XT.min(0), X.min(0)), np.maximum(XT.max(0), X.max(0))
    c.call("pbgb_ccd_initialize", XT, X, lo, hi)
    c.call("pbgb_ccd_update", X)
    c.call("pbgb_ccd_finalize", X)
    active, nn, dup, na = c.get()
    pen = body >= 0
    assert pen.sum() > 20
    np.testing.assert_array_equal(active.astype(bool), pen)
    Xf = X.astype(np.float32).astype(np.float64)
    for q in np.nonzero(pen)[0]:
        f = nn[q][nn[q] >= 0]
        assert len(f) >= 1
        assert (B[F[f, 0]] == body[q]).all()
        p = Xf[V[q]]
        d = min(_sqdist(p, *Xf[F[g]]) for g in f)
        assert abs(d - d2[q]) <= 1e-6 * max(1.0, d2[q]) + 1e-9


def _sqdist(p, a, b, c):
    ab, ac = b - a, c - a
    M = np.array([[ab @ ab, ab @ ac], [ab @ ac, ac @ ac]])
    u, v = np.linalg.solve(M, np.array([ab @ (p - a), ac @ (p - a)]))
    if u >= 0 and v >= 0 and u + v <= 1:
        r = p - (a + u * ab + v * ac)
        return float(r @ r)

    def seg(s0, s1):
        d = s1 - s0
        t = np.clip((p - s0) @ d / (d @ d), 0.0, 1.0)
        r = p - (s0 + t * d)
        return float(r @ r)

    return min(seg(a, b), seg(b, c), seg(c, a))


def test_anderson_with_contact_matches_oracle():
    """gpu/vbd/Integrator.cu:15-33 builds the Anderson integrator for contact scenes too: window 5
    on the two-buffer contact sweep (the iterate updated in both position buffers), 12 steps
    against the FP64 contact oracle running the same Anderson loop."""
    w = small_scene()
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
         .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
         .with_contact_parameters(1e7, 0.3, 1e-3).with_initialization_strategy(2)
         .with_anderson_acceleration(5).construct())
    I = pbat.gpu.vbd.Integrator(d)
    R = O.OracleContactVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], w["V"], w["F"], w["B"],
                           muC=1e7, strategy=2, anderson_window=5)
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    errs = []
    for _ in range(12):
        I.x, I.v = R.x.T.copy(), R.v.T.copy()
        I.step(1 / 60, 15, 1)
        R.step(1 / 60, 15, 1, 1)
        errs.append(np.abs(I.x.T - R.x).max() / diag)
    fc, active = I.contacts()
    assert R.active.sum() > 0
    assert max(errs) <= 1e-4, errs


def test_trust_region_with_contact_matches_oracle_on_the_device_decisions():
    """The trust region with contact (the objective adds the active vertices' contact energy,
    gpu/impl/vbd/TrustRegionIntegrator.cu:265-360): the oracle replays the device's logged decisions
    step by step; positions within 1e-4 of the diagonal over the first 10 steps (measured up to
    6e-6).  A stretched step multiplies the FP32/FP64 difference of the VBD step by t (up to ~16),
    and the penalty switching on below a triangle's plane amplifies it further: at step 11 of this
    scene, where the active set drops from 99 to 78 vertices, the replayed oracle lands 6.7e-3 of
    the diagonal away (FP64 trust-region and plain VBD differ by 2.6e-3 there), so the check stops
    before it."""
    w = small_scene()
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
         .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
         .with_contact_parameters(1e7, 0.3, 1e-3).with_initialization_strategy(2)
         .with_trust_region_acceleration(0.2, 2.0, False).construct())
    I = pbat.gpu.vbd.Integrator(d)
    R = O.OracleContactVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], w["V"], w["F"], w["B"],
                           muC=1e7, strategy=2, trust_region=(0.2, 2.0, False))
    diag = np.linalg.norm(w["X"].max(0) - w["X"].min(0))
    tried = 0
    for _ in range(10):
        I.x, I.v = R.x.T.copy(), R.v.T.copy()
        I.step(1 / 60, 15, 1)
        log = I.trust_region_log()
        tried += int((log[:, 3] > 0).sum())
        R.step(1 / 60, 15, 1, 1, trust_region_log=log)
        err = np.abs(I.x.T - R.x).max() / diag
        assert err <= 1e-4, err
    assert tried > 0 and R.active.sum() > 0


def test_active_set_covers_cpu_ccd_hits():
    """The swept-box broad phase of the GPU active set against the vertex-triangle CCD of the CPU
    multibody detector: a cube moved in one step from 5 cm above a slab to 25 cm into it (its
    bottom vertices pass through the slab's top face, the slab's top vertices through its bottom
    face).  Every collision vertex whose trajectory meets a triangle of another body during the step
    (exact CCD, oracle/contact_oracle.cpp) is active after the GPU initialization."""
    w = meshgen.contact_scene_workload(n_cubes_side=1, cube_hexes=4, slab_hexes=(8, 8, 1), cell=1.0)
    XT, F, V, B = w["X"].copy(), w["F"], w["V"], w["B"]
    X = XT.copy()
    X[B == 1, 2] -= 0.3
    toi, tri = O.ccd_vertex_triangle(XT, X, F, V, B)
    hits = toi >= 0
    assert hits.sum() > 20
    assert (B[F[tri[hits], 0]] != B[V[hits]]).all()
    c = Ccd(X.shape[0], V, F, B)
    lo, hi = np.minimum(XT.min(0), X.min(0)), np.maximum(XT.max(0), X.max(0))
    c.call("pbgb_ccd_initialize", XT, X, lo, hi)
    active, nn, dup, na = c.get()
    missed = np.nonzero(hits & ~active.astype(bool))[0]
    assert missed.size == 0, missed
