"""Parity at the benchmark configurations, full size, against the FP64 oracle.

These are the workloads every throughput figure of bench.py is measured on:

* the beam: [0,4]x[0,1]^2 as 160x40x40 hexes x 6 tets (270,641 vertices), E 5e5, nu 0.48, the
  x=0 face pinned, initial velocities U(-0.1, 0.1), Chebyshev rho 0.95 (the reference's weight
  recurrence), 50 iterations, 60 steps of 1/60 s, on the GPU integrator;
* the batch: 256 cube grids with side U{6..32} hexes, E log-uniform in [1e5, 1e7], nu U(0.30,
  0.48), one face pinned, gravity, 20 iterations, stepped together by one batched integrator;
* the contact scene: 16 cubes of 16^3 hexes above a pinned 64x64x2 slab, vertex-triangle
  contact (muC 1e7, muF 0.3, epsv 1e-3), 30 iterations, 120 steps, the LBVH over the swept
  collision triangles rebuilt every step.

Tolerance: positions within 1e-4 of the bounding-box diagonal (FP32 device arithmetic against
the FP64 oracle on the same mesh, colouring and iteration count); the LBVH's Morton codes, sort
order, topology and overlap pairs bit for bit.
"""

import numpy as np
import pytest

import oracle_lib as O
from physicsbasedanimationtoolkit_gb300 import meshgen, pbat

pytestmark = pytest.mark.gpu

TOL = 1e-4  # of the bounding-box diagonal


def diag(X):
    return float(np.linalg.norm(X.max(0) - X.min(0)))


def test_beam_160x40x40_chebyshev_60_steps_matches_oracle():
    w = meshgen.beam_workload(nx=160, ny=40, nz=40, seed=0)
    data = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
            .with_dirichlet_vertices(w["dbc"]).with_velocity(w["v"].T).with_chebyshev_acceleration(0.95)
            .construct())
    I = pbat.gpu.vbd.Integrator(data)
    R = O.OracleVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], v=w["v"], strategy=4,
                    rho_chebyshev=0.95, chebyshev_formula=0, semantics=1)
    d = diag(w["X"])
    errs = []
    for _ in range(6):
        for _ in range(10):
            I.step(1 / 60, 50, 1)
        R.step(1 / 60, 50, 1, 10)
        errs.append(float(np.abs(I.x.T.astype(np.float64) - R.x).max() / d))
    assert max(errs) <= TOL, errs
    # The beam moved: its free end swings by centimetres under gravity and the initial velocities.
    assert np.abs(R.x - w["X"]).max() > 1e-2


def test_batch_of_256_meshes_matches_oracle_per_mesh():
    """The whole 256-mesh batch is stepped by one batched integrator; a seeded subset of meshes
    that includes the smallest and the largest is checked against its own oracle after every
    step."""
    meshes = meshgen.batch_workload(n_meshes=256, nmin=6, nmax=32, seed=0)
    datas = [pbat.sim.vbd.Data().with_volume_mesh(m["X"].T, m["T"].T).with_material(m["rho"], m["mu"], m["lam"])
             .with_dirichlet_vertices(m["dbc"]).construct() for m in meshes]
    B = pbat.gpu.vbd.BatchedIntegrator(datas)
    sides = np.array([m["side"] for m in meshes])
    rng = np.random.default_rng(5)
    pick = {int(np.argmin(sides)), int(np.argmax(sides))}
    pick |= set(int(b) for b in rng.choice(len(meshes), 6, replace=False))
    pick = sorted(pick)
    assert sides[pick].min() == 6 and sides[pick].max() == 32
    oracles = {b: O.OracleVbd(meshes[b]["X"], meshes[b]["T"], meshes[b]["rho"], meshes[b]["mu"], meshes[b]["lam"],
                              meshes[b]["dbc"], v=meshes[b]["v"], strategy=4, semantics=1) for b in pick}
    off = B.vertex_offsets
    worst = 0.0
    for _ in range(3):
        B.step(1 / 60, 20, 1)
        x = B.x
        for b in pick:
            oracles[b].step(1 / 60, 20, 1, 1)
            xb = x[:, off[b]: off[b + 1]].T.astype(np.float64)
            worst = max(worst, float(np.abs(xb - oracles[b].x).max() / diag(meshes[b]["X"])))
    assert worst <= TOL, worst
    # Every mesh of the batch moved and stayed finite.
    x = B.x
    assert np.isfinite(x).all()
    for b in range(len(meshes)):
        assert np.abs(x[:, off[b]: off[b + 1]].T - meshes[b]["X"]).max() > 1e-4


def contact_scene_integrator():
    w = meshgen.contact_scene_workload()
    data = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
            .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
            .with_contact_parameters(1e7, 0.3, 1e-3).with_initialization_strategy(2).construct())
    return w, pbat.gpu.vbd.Integrator(data)


def sorted_pairs(p):
    p = np.asarray(p).reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def test_contact_scene_lbvh_bit_exact_at_every_step_of_120():
    """At every one of the 120 steps, the hierarchy the step built over its swept triangle boxes
    (from the positions at the step's start and the full-step prediction) has the oracle's Morton
    codes, stable sort order, child / parent / rightmost topology, and the overlap pairs of the
    swept vertex boxes against those triangle boxes are the all-pairs set, bit for bit."""
    w, I = contact_scene_integrator()
    F = np.asarray(w["F"])
    V = np.asarray(w["V"])
    nF = F.shape[0]
    bvh = pbat.gpu.geometry.Bvh(nF, 0)
    q_total = 0
    for step in range(120):
        x0 = I.x.T.copy()  # float32 positions at the step's start
        I.step(1 / 60, 30, 1)
        bv = I.contact_bvh()
        xp = bv["xpred"]
        lo, hi = meshgen.triangle_boxes(x0, F, xp)
        lo, hi = lo.astype(np.float32), hi.astype(np.float32)
        o = O.bvh_build(lo, hi, bv["wmin"], bv["wmax"])
        np.testing.assert_array_equal(bv["codes"], o["codes"], err_msg=f"step {step}: Morton codes")
        np.testing.assert_array_equal(bv["inds"], o["inds"], err_msg=f"step {step}: sort order")
        np.testing.assert_array_equal(bv["child"], o["child"], err_msg=f"step {step}: children")
        np.testing.assert_array_equal(bv["parent"], o["parent"], err_msg=f"step {step}: parents")
        np.testing.assert_array_equal(bv["rightmost"], o["rightmost"], err_msg=f"step {step}: rightmost")
        # Overlap pairs of the swept collision-vertex boxes on the same boxes: the public Bvh (the
        # same build and query kernels) against all pairs.
        qlo = np.minimum(x0[V], xp[V]).astype(np.float32)
        qhi = np.maximum(x0[V], xp[V]).astype(np.float32)
        bvh.build(lo.T, hi.T, bv["wmin"], bv["wmax"])
        t = bvh._topology()
        np.testing.assert_array_equal(t["inds"], bv["inds"])
        np.testing.assert_array_equal(t["child"], bv["child"])
        got = sorted_pairs(bvh.overlaps(qlo.T, qhi.T).T)
        exp = O.overlaps(lo, hi, qlo, qhi)
        np.testing.assert_array_equal(got, exp, err_msg=f"step {step}: overlap pairs")
        q_total += exp.shape[0]
    assert q_total > 120 * V.size  # every vertex box overlaps at least its own triangles' boxes
    x = I.x.T
    assert np.isfinite(x).all()
    fc, active = I.contacts()
    assert active.sum() > 100  # the cubes rest on the slab


def device_contact_state(I, nV, nS):
    """(x, v, vprev, active, dupper, fc) of the device integrator, from its checkpoint blob
    (header of 6 int32; x, v, vprev, aext as nV float4; active flags padded to 4 bytes; search
    radii as nS float32; contact lists as 8 nV int32)."""
    blob = I.save_state()
    off = 24
    arrays = []
    for _ in range(4):
        arrays.append(np.frombuffer(blob, np.float32, 4 * nV, off).reshape(nV, 4)[:, :3].astype(np.float64))
        off += 16 * nV
    active = np.frombuffer(blob, np.uint8, nS, off).copy()
    off += (nS + 3) & ~3
    dupper = np.frombuffer(blob, np.float32, nS, off).astype(np.float64)
    off += 4 * nS
    fc = np.frombuffer(blob, np.int32, 8 * nV, off).copy()
    return arrays[0], arrays[1], arrays[2], active, dupper, fc


def point_triangle_distance(p, a, b, c):
    """Distance from p to triangle abc (closest point by Voronoi regions of the triangle)."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = ab @ ap, ac @ ap
    if d1 <= 0 and d2 <= 0:
        return np.linalg.norm(p - a)
    bp = p - b
    d3, d4 = ab @ bp, ac @ bp
    if d3 >= 0 and d4 <= d3:
        return np.linalg.norm(p - b)
    vc = d1 * d4 - d3 * d2
    if vc <= 0 and d1 >= 0 and d3 <= 0:
        return np.linalg.norm(p - (a + d1 / (d1 - d3) * ab))
    cp = p - c
    d5, d6 = ab @ cp, ac @ cp
    if d6 >= 0 and d5 <= d6:
        return np.linalg.norm(p - c)
    vb = d5 * d2 - d1 * d6
    if vb <= 0 and d2 >= 0 and d6 <= 0:
        return np.linalg.norm(p - (a + d2 / (d2 - d6) * ac))
    va = d3 * d6 - d5 * d4
    if va <= 0 and (d4 - d3) >= 0 and (d5 - d6) >= 0:
        return np.linalg.norm(p - (b + (d4 - d3) / ((d4 - d3) + (d5 - d6)) * (c - b)))
    den = 1.0 / (va + vb + vc)
    return np.linalg.norm(p - (a + ab * vb * den + ac * vc * den))


def test_contact_scene_matches_contact_oracle_through_contact():
    """30 steps (the cubes start 5 cm above the slab and touch it at about step 6).

    * Until the first contact, free-running positions agree within 1e-4 of the diagonal.
    * Once contact starts, the step is compared one step at a time from the device's state
      (positions, velocities, active set, search radii and lists, read from the checkpoint blob):
      the FP32 device and the FP64 oracle take discrete decisions that near-ties can tip either
      way (a triangle within FLT_EPSILON of the nearest joins a list or not; a vertex projects
      inside a triangle or just outside it), each decision changes a contact force by a finite
      amount, and free-running trajectories of this stiff scene then drift apart.
      * The contact lists the device chose equal the lists the oracle chooses from the same state,
        except where the two differ only by triangles tied within 1e-5 of the diagonal with the
        nearest one, on at most 1 % of the vertices with contacts.
      * With the device's lists, the oracle's step from the same state lands within 1e-4 of the
        diagonal of the device's on all but 0.5 % of the vertices, and within 5e-3 everywhere.
        The step is discontinuous in its state: a listed triangle's penalty applies only while
        the vertex projects inside it, so a penetrating vertex over a shared edge gets one, two or
        no penalties as rounding falls.  The FP64 oracle itself, stepped from the same state
        perturbed by 1e-7 (relative, the size of FP32 rounding) with the same lists, moves up to
        4 of the 91,283 vertices by more than 1e-4 of the diagonal (at most 8.9e-4) in one step
        of this scene, while its 99.9th percentile stays near 1e-6.  On the device the largest
        such step moved 108 vertices (0.12 %) by more than 1e-4, at most 1.7e-3."""
    w, I = contact_scene_integrator()
    kw = dict(muC=1e7, muF=0.3, epsv=1e-3, strategy=2)
    R = O.OracleContactVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], w["V"], w["F"], w["B"], **kw)
    D = O.OracleContactVbd(w["X"], w["T"], w["rho"], w["mu"], w["lam"], w["dbc"], w["V"], w["F"], w["B"], **kw)
    nV, V, F = w["X"].shape[0], np.asarray(w["V"]), np.asarray(w["F"])
    d = diag(w["X"])
    free, step_errs, first_contact, mismatched, listed = [], [], None, 0, 0
    for step in range(30):
        state = device_contact_state(I, nV, V.size)
        x0, v0, vp0, act0, dup0, fc0 = state
        I.step(1 / 60, 30, 1)
        x = I.x.T.astype(np.float64)
        fc_dev = I.contacts()[0].reshape(-1)
        if first_contact is None and (fc_dev >= 0).any():
            first_contact = step
        if first_contact is None:
            # Free-running until contact.
            R.step(1 / 60, 30, 1, 1)
            free.append(float(np.abs(x - R.x).max() / d))
            continue
        # The oracle's own decisions from the device's state.
        D.x[:], D.v[:], D.vprev[:] = x0, v0, vp0
        D.active[:], D.dupper[:], D.fc[:] = act0, dup0, fc0
        D.step(1 / 60, 30, 1, 1)
        dev, orc = fc_dev.reshape(nV, 8), D.fc.reshape(nV, 8)
        xs = x0 + (1 / 60) * v0 + (1 / 60) ** 2 * D.aext  # the initial guess the lists were taken at
        for i in np.nonzero((dev != orc).any(axis=1))[0]:
            a, b = set(dev[i][dev[i] >= 0]), set(orc[i][orc[i] >= 0])
            dist = {f: point_triangle_distance(xs[i], *xs[F[f]]) for f in a | b}
            best = min(dist.values())
            assert all(dist[f] - best <= 1e-5 * d for f in a ^ b), (step, i, dist)
            mismatched += 1
        listed += int((dev >= 0).any(axis=1).sum())
        # The oracle's step from the same state with the device's lists.
        R.x[:], R.v[:], R.vprev[:] = x0, v0, vp0
        R.active[:], R.dupper[:], R.fc[:] = act0, dup0, fc0
        R.step(1 / 60, 30, 1, 1, contact_lists=fc_dev)
        e = np.abs(x - R.x).max(axis=1) / d
        step_errs.append((step, float(e.max()), int((e > TOL).sum()), int((e > 10 * TOL).sum())))
    assert first_contact is not None and 0 < first_contact < 15, first_contact
    assert max(free) <= TOL, free
    bad = [r for r in step_errs if r[1] > 5e-3 or r[2] > 0.005 * nV]
    assert not bad, (bad, step_errs)
    assert listed > 1000 and mismatched <= 0.01 * listed, (mismatched, listed)
