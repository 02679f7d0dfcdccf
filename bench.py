#!/usr/bin/env python3
"""Benchmark of the VBD step on one GB300 (replicas on N GPUs under torchrun).

Headline workload (the metric's configuration): 256 cube grids with side n ~ U{6..32} hexes split
into 6 tets per hex (3,252,189 vertices, 17,350,662 tets), E log-uniform in [1e5, 1e7], nu
U(0.30, 0.48), density 1000, one face pinned, gravity, 20 VBD iterations per step, dt = 1/60, all
meshes stepped together by the batched integrator (one persistent launch per step); beside it the
same meshes stepped by one integrator per mesh (one launch per colour, each on its own stream).
A "step" is one time step of the whole batch.  Metric: vertex-updates/s = free vertices x
iterations x substeps x steps / time.

Secondary legs: the [0,4]x[0,1]^2 beam at 160x40x40 hexes (270,641 vertices, Chebyshev rho 0.95, 50
iterations), the adjoint on the 40x10x10 differentiation beam, the 16-cube contact scene, a
4.19M-box LBVH build and the Anderson / trust-region / Broyden accelerations on the beam.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference algorithm's CPU implementation (the FP64 oracle port, all
host threads) on the same batched workload and prints the same JSON line with "impl": "reference".
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "VBD vertex-updates/s, batched vs single-launch at ≤1e-4 rel err; bwd/fwd time"
UNIT = "vertex-updates/s"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 512 << 20


def workload_beam(args):
    from physicsbasedanimationtoolkit_gb300 import meshgen

    w = meshgen.beam_workload(nx=args.nx, ny=args.ny, nz=args.nz, seed=0)
    return w


def make_data(pbat, w, rho=0.95):
    return (
        pbat.sim.vbd.Data()
        .with_volume_mesh(w["X"].T, w["T"].T)
        .with_material(w["rho"], w["mu"], w["lam"])
        .with_dirichlet_vertices(w["dbc"])
        .with_velocity(w["v"].T)
        .with_chebyshev_acceleration(rho)
        .construct()
    )


def algorithmic_bytes(data):
    """Sum over free vertices of (60 + 120 deg(i)) bytes: one vertex-update's FP32/int32 inputs and
    output (CSR pair 8, mass 4, xt 12, xtilde 12, x read 12 and written 12; per incident tet:
    (e, ilocal) 8, 4 indices 16, GP 48, (mu, lambda) 8, wg 4, three other positions 36)."""
    deg = np.diff(data.GVGp)[data.Padj]
    return int(60 * deg.size + 120 * int(deg.sum()))


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    FIELDS = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # nvidia-smi takes a moment to start: wait for its first sample so that the timed
            # region is sampled from its beginning.
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def peak_hbm():
    try:
        p = json.loads(PEAKS_FILE.read_text())
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


KERNEL_SOURCES = {
    "batched_step_cfg3.md": ["batched.cu", "batched.cuh", "sweep_device.cuh", "vbd_math.cuh", "vbd_kernels.cuh"],
    "vbd_sweep_beam160x40x40.md": ["vbd_kernels.cu", "sweep_device.cuh", "vbd_math.cuh", "vbd_kernels.cuh"],
}


def kernel_source_sha(name):
    """sha256 (first 16 hex digits) of the sources the kernel of a profile summary is built from."""
    import hashlib

    h = hashlib.sha256()
    for f in KERNEL_SOURCES[name]:
        h.update((ROOT / "physicsbasedanimationtoolkit_gb300" / "csrc" / f).read_bytes())
    return h.hexdigest()[:16]


def traffic_from_profiles(name):
    """DRAM bytes per launch from the committed ncu summary profiles/<name>, when the summary was
    captured from the current kernel sources (its `source_sha` line equals their hash); otherwise
    (None, reason)."""
    f = ROOT / "profiles" / name
    try:
        lines = f.read_text().splitlines()
    except OSError:
        return None, "no profile summary"
    traffic, sha = None, None
    for line in lines:
        if line.startswith("traffic_bytes_per_launch:"):
            traffic = float(line.split(":", 1)[1].strip())
        elif line.startswith("source_sha:"):
            sha = line.split(":", 1)[1].strip()
    if traffic is None:
        return None, "the profile summary has no traffic figure"
    if sha != kernel_source_sha(name):
        return None, "the profile summary was captured from other kernel sources"
    return traffic, f"ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/{name}"


def dram_rate(traffic, avg_launch_ms, peak):
    """The ncu-measured DRAM bytes of one launch over the live launch duration, and its fraction of
    the HBM peak (the algorithmic figure counts bytes that L2 serves as well)."""
    if traffic is None or not avg_launch_ms:
        return {"dram_gbs": None, "dram_frac": None}
    gbs = traffic / (avg_launch_ms * 1e-3) / 1e9
    return {"dram_gbs": gbs, "dram_frac": gbs / peak}


def batch_oracles(meshes):
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O

    O.build_oracle()
    threads = O.lib().orc_num_threads()
    oracles = [O.OracleVbd(m["X"], m["T"], m["rho"], m["mu"], m["lam"], m["dbc"], v=m["v"], strategy=4, semantics=1)
               for m in meshes]
    return oracles, int(threads)


def cpu_batch_step(oracles, iterations):
    """One time step of every mesh with the FP64 oracle, one mesh after the other (the reference
    steps one mesh per integrator), each mesh's colour sweeps on all host threads."""
    for R in oracles:
        R.step(1 / 60, iterations, 1, 1)


def cpu_baseline(meshes, iterations, seconds_budget=20.0):
    """The FP64 oracle (port of the reference's CPU integrator) on all host threads, on a bounded
    sample of the batched workload: one time step of all meshes with as many of the iterations as
    fit the budget."""
    oracles, threads = batch_oracles(meshes)
    n_free = sum(int(R.data["Padj"].size) for R in oracles)
    t0 = time.perf_counter()
    cpu_batch_step(oracles, 1)
    t_iter = time.perf_counter() - t0
    iters = max(1, min(iterations, int(seconds_budget / max(t_iter, 1e-9))))
    t0 = time.perf_counter()
    cpu_batch_step(oracles, iters)
    dt = time.perf_counter() - t0
    sample = (f"1 time step x {iters} of {iterations} iterations of all {len(meshes)} meshes (one after the "
              f"other), FP64, {threads} OpenMP threads")
    return {"value": n_free * iters / dt, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            "seconds": dt}


def run_reference(args):
    """--impl reference: the CPU implementation of the path (oracle port) on the batched workload,
    rank 0 only.  Each step is a bounded sample: one time step of all meshes with as many of the
    iterations as keep warmup + steps within a few minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from physicsbasedanimationtoolkit_gb300 import meshgen

    meshes = meshgen.batch_workload(n_meshes=args.batch_meshes, nmin=6, nmax=32, seed=0)
    oracles, threads = batch_oracles(meshes)
    n_free = sum(int(R.data["Padj"].size) for R in oracles)
    t0 = time.perf_counter()
    cpu_batch_step(oracles, 1)
    t_iter = time.perf_counter() - t0
    budget = 150.0 / max(1, args.steps + args.warmup)
    iters = max(1, min(args.batch_iterations, int(budget / max(t_iter, 1e-9))))
    for _ in range(args.warmup):
        cpu_batch_step(oracles, iters)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_batch_step(oracles, iters)
    el = time.perf_counter() - t0
    value = n_free * iters * args.steps / el
    sample = (f"each step: 1 time step x {iters} of {args.batch_iterations} iterations of all {len(meshes)} "
              f"meshes (one after the other), FP64, {threads} OpenMP threads")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": config_of(args, meshes),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def batch_workload(args, pbat):
    """The batched workload: 256 cube grids with side n ~ U{6..32} hexes (6 tets per hex), E
    log-uniform in [1e5, 1e7], nu ~ U(0.30, 0.48), density 1000, one face pinned, gravity, 20
    iterations per step, dt = 1/60."""
    from physicsbasedanimationtoolkit_gb300 import meshgen

    meshes = meshgen.batch_workload(n_meshes=args.batch_meshes, nmin=6, nmax=32, seed=0)
    datas = [
        pbat.sim.vbd.Data().with_volume_mesh(m["X"].T, m["T"].T).with_material(m["rho"], m["mu"], m["lam"])
        .with_dirichlet_vertices(m["dbc"]).construct()
        for m in meshes
    ]
    return meshes, datas


def batch_algorithmic_bytes(datas, iterations):
    """Algorithmic bytes of one batched step: per iteration the sum over every mesh's free vertices
    of (60 + 120 deg(i)) bytes (the vertex-update formula of the sweep), plus per substep the
    inertial target and initial guess (48 B read, 64 B written per vertex) and the velocity update
    (48 B read, 32 B written per vertex)."""
    per_iter = sum(algorithmic_bytes(d) for d in datas)
    nV = sum(int(d.X.shape[1]) for d in datas)
    return iterations * per_iter + (112 + 80) * nV


def time_single_launch(singles, dt, iters, steps, torch):
    """One integrator per mesh, each on its own stream: all steps of all meshes are launched, then
    waited for.  Timed with CUDA events: a start event on a master stream that every integrator's
    stream waits on, an end event on every integrator's stream that the master waits on."""
    from physicsbasedanimationtoolkit_gb300 import _capi

    master = torch.cuda.Stream()
    streams = []
    for s in singles:
        sp = C.c_void_p()
        _capi.check(_capi.lib().pbgb_vbd_stream(s.handle, C.byref(sp)), s.handle)
        streams.append(torch.cuda.ExternalStream(sp.value))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(master)
    for st in streams:
        st.wait_event(e0)
    for _ in range(steps):
        for s in singles:
            s.step(dt, iters, 1)
    for st in streams:
        ev = torch.cuda.Event()
        ev.record(st)
        master.wait_event(ev)
    e1.record(master)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3


def run_batch(args, pbat, _capi, torch, with_single=True):
    """Batched uneven meshes (batch_workload): one persistent launch per step advances the whole
    batch; the comparison steps one integrator per mesh, one launch per colour, each on its own
    stream (all launched before one wait).  Both arms are timed with CUDA events on their streams.
    Returns the batch figures and the agreement between the two (bit for bit: same lanes, block
    size and per-vertex arithmetic)."""
    meshes, datas = batch_workload(args, pbat)
    dt, iters = 1 / 60, args.batch_iterations
    B = pbat.gpu.vbd.BatchedIntegrator(datas)
    if args.lanes:
        # A fixed launch (profiling runs launch exactly what a timed run launched, without the
        # autotuner's candidates).
        B.lanes_per_vertex = args.lanes
        block = args.block or 256
        _capi.check(_capi.lib().pbgb_vbd_set_block_size(B.handle, block), B.handle)
        lanes, tuned_ms = args.lanes, None
    else:
        lanes, block, tuned_ms = B.autotune(dt, iters, 1)
    n_free = B.n_free
    sp = C.c_void_p()
    _capi.check(_capi.lib().pbgb_vbd_stream(B.handle, C.byref(sp)), B.handle)
    stream = torch.cuda.ExternalStream(sp.value)
    for _ in range(args.warmup):
        B.step(dt, iters, 1)
    B.synchronize()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_batched = 0.0
    torch.cuda.nvtx.range_push("timed_batch")  # lets ncu --nvtx-include select the timed steps
    for _ in range(args.steps):
        flush.add_(1.0)
        torch.cuda.synchronize()
        e0.record(stream)
        B.step(dt, iters, 1)
        e1.record(stream)
        B.synchronize()
        t_batched += e0.elapsed_time(e1) * 1e-3
    torch.cuda.nvtx.range_pop()
    out = {
        "workload": f"{len(meshes)} cube grids, side U{{6..32}} hexes x 6 tets, {iters} iterations, no acceleration",
        "n_meshes": len(meshes),
        "n_vertices": int(B.n_vertices),
        "n_tets": int(B.n_tets),
        "n_free_vertices": int(n_free),
        "persistent": bool(B.persistent),
        "batched_value": n_free * iters * args.steps / t_batched,
        "batched_ms_per_step": 1e3 * t_batched / args.steps,
        "autotuned": {"lanes": lanes, "block": block, "ms_per_step": tuned_ms},
        "batched_launches_per_step": int(B.launches_per_step(iters, 1)),
        "algorithmic_bytes_per_step": batch_algorithmic_bytes(datas, iters),
        "timing": "CUDA events on each arm's streams; L2 flushed before every batched step",
        "unit": UNIT,
    }
    if with_single:
        singles = []
        for d in datas:
            s = pbat.gpu.vbd.Integrator(d)
            s.lanes_per_vertex = lanes
            _capi.check(_capi.lib().pbgb_vbd_set_block_size(s.handle, block), s.handle)
            singles.append(s)
        for _ in range(args.warmup):
            for s in singles:
                s.step(dt, iters, 1)
        for s in singles:
            s.synchronize()
        # Agreement from the same number of steps: a fresh batch against the single integrators.
        off = B.vertex_offsets
        B2 = pbat.gpu.vbd.BatchedIntegrator(datas)
        B2.lanes_per_vertex = lanes
        _capi.check(_capi.lib().pbgb_vbd_set_block_size(B2.handle, block), B2.handle)
        for _ in range(args.warmup):
            B2.step(dt, iters, 1)
        xb = B2.x
        worst = 0.0
        for b, s in enumerate(singles):
            X = meshes[b]["X"]
            diag = np.linalg.norm(X.max(0) - X.min(0))
            worst = max(worst, float(np.abs(xb[:, off[b]: off[b + 1]] - s.x).max() / diag))
        del B2
        t_single = time_single_launch(singles, dt, iters, args.steps, torch)
        out.update({
            "single_launch_value": n_free * iters * args.steps / t_single,
            "single_launch_ms_per_step": 1e3 * t_single / args.steps,
            "speedup": t_single / t_batched,
            "single_launches_per_step": int(sum(s.launches_per_step(iters, 1) for s in singles)),
            "max_rel_diff_batched_vs_single": worst,
        })
    return out


def run_adjoint(args, pbat, torch):
    """Differentiation workload: beam [0,4]x[0,1]^2 at 40x10x10 hexes (4,961 vertices, 24,000
    tets), per-tet log E ~ N(log 1e6, 0.3^2), nu 0.45, 30 steps of 20 iterations at dt = 1/60, the
    reference Data's default initial guess (AdaptivePbat), loss on the 121 tip vertices;
    checkpoints every 5 steps.  Forward = the rollout (graph-replayed steps plus checkpoint
    copies, the last segment recorded), backward = re-recording every other segment and reversing
    all of them.  `taped`: the same with the whole rollout recorded in the forward pass
    (checkpoint_every = 30; 153 MB of tape), so backward only reverses.  Both are timed with CUDA
    events on the integrator's stream, where all of their device work runs (the host's launch gaps
    included); the host clock around a synchronize is reported beside them."""
    from physicsbasedanimationtoolkit_gb300 import _capi, meshgen

    w = meshgen.adjoint_beam_workload()
    nT = w["T"].shape[0]
    nu = w["nu"]
    mu0, lam0 = meshgen.lame(np.exp(w["logE"]), np.full(nT, nu))
    data = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], mu0, lam0)
            .with_dirichlet_vertices(w["dbc"]).construct())
    I = pbat.gpu.vbd.Integrator(data)
    sp = C.c_void_p()
    _capi.check(_capi.lib().pbgb_vbd_stream(I.handle, C.byref(sp)), I.handle)
    stream = torch.cuda.ExternalStream(sp.value)
    dt, iters, steps, every = 1 / 60, 20, 30, 5
    logE = torch.tensor(w["logE"], dtype=torch.float64, requires_grad=True)
    x0 = torch.tensor(w["X"], dtype=torch.float32, device="cuda", requires_grad=True)
    v0 = torch.zeros_like(x0, requires_grad=True)
    tip = torch.tensor(w["tip"], device="cuda")
    target = torch.tensor(w["target"], dtype=torch.float32, device="cuda")
    def timed(every):
        fwd, bwd, fwd_host, bwd_host = [], [], [], []
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        for k in range(args.warmup + args.steps):
            logE.grad = None
            x0.grad = None
            v0.grad = None
            E = torch.exp(logE)
            mu = E / (2 * (1 + nu))
            lam = E * nu / ((1 + nu) * (1 - 2 * nu))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ev[0].record(stream)
            xT, _ = pbat.gpu.vbd.rollout(I, mu, lam, x0, v0, dt=dt, iterations=iters, steps=steps, checkpoint_every=every)
            ev[1].record(stream)
            loss = ((xT[tip] - target) ** 2).sum()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            ev[2].record(stream)
            loss.backward()
            ev[3].record(stream)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            if k >= args.warmup:
                fwd.append(ev[0].elapsed_time(ev[1]))
                bwd.append(ev[2].elapsed_time(ev[3]))
                fwd_host.append(1e3 * (t1 - t0))
                bwd_host.append(1e3 * (t2 - t1))
        f, b = float(np.median(fwd)), float(np.median(bwd))
        return {"checkpoint_every": every, "fwd_ms": f, "bwd_ms": b, "bwd_over_fwd": b / f,
                "host_fwd_ms": float(np.median(fwd_host)), "host_bwd_ms": float(np.median(bwd_host)),
                "loss": float(loss.detach()),
                "grad_norms": {"log_E": float(logE.grad.norm()), "v0": float(v0.grad.norm()),
                               "x0": float(x0.grad.norm())}}

    out = timed(every)
    out["taped"] = timed(steps)
    out["workload"] = ("beam [0,4]x[0,1]^2 40x10x10 hexes x 6 tets, log E ~ N(log 1e6, 0.3^2), nu 0.45, "
                       "30 steps x 20 iterations, dt 1/60, AdaptivePbat initial guess, tip-face loss, checkpoints every 5 steps")
    out["timing"] = ("CUDA events on the integrator's stream around the rollout and around backward, median of the "
                     "timed repetitions")
    return out


def run_accelerated(args, pbat, torch, kind):
    """An accelerated solve on the benchmark beam [0,4]x[0,1]^2 at 160x40x40 hexes (270,641
    vertices, 1,536,000 tets), 50 iterations per step, dt = 1/60, against plain VBD with the same
    iterations from the same state: step time (CUDA events on the integrator's stream) and the norm
    of the FP64 objective gradient over the free vertices after one step.  kind: "anderson"
    (window 5), "broyden" (window 5) or "trust_region" (linear path, eta 0.2, tau 2)."""
    import ctypes as C

    from physicsbasedanimationtoolkit_gb300 import _capi

    w = workload_beam(args)
    dt, iters = 1 / 60, 50

    def measure(accel):
        d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_material(w["rho"], w["mu"], w["lam"])
             .with_dirichlet_vertices(w["dbc"]).with_velocity(w["v"].T).with_initialization_strategy(2))
        if accel == "anderson":
            d = d.with_anderson_acceleration(5)
        elif accel == "trust_region":
            d = d.with_trust_region_acceleration(0.2, 2.0, False)
        elif accel == "broyden":
            d = d.with_broyden_acceleration(5)
        # Broyden is a CPU-integrator strategy in the reference (the GPU integrator runs plain VBD).
        cls = pbat.sim.vbd.Integrator if accel == "broyden" else pbat.gpu.vbd.Integrator
        I = cls(d.construct())
        I.autotune(dt, iters, 1)  # lanes and block size per strategy; the state is restored
        x0, v0 = I.x.copy(), I.v.copy()
        I.step(dt, iters, 1)
        g = I.gradient(dt).reshape(-1, 3)
        g[w["dbc"]] = 0.0
        gnorm = float(np.linalg.norm(g))
        for _ in range(args.warmup):
            I.step(dt, iters, 1)
        I.x, I.v = x0, v0
        sp = C.c_void_p()
        _capi.check(_capi.lib().pbgb_vbd_stream(I.handle, C.byref(sp)), I.handle)
        stream = torch.cuda.ExternalStream(sp.value)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        I.synchronize()
        torch.cuda.nvtx.range_push(f"timed_{accel or 'plain'}")  # lets ncu --nvtx-include select these steps
        e0.record(stream)
        for _ in range(args.steps):
            I.step(dt, iters, 1)
        e1.record(stream)
        I.synchronize()
        torch.cuda.nvtx.range_pop()
        return e0.elapsed_time(e1) / args.steps, gnorm, I.n_free

    ms_a, g_a, n_free = measure(kind)
    ms_p, g_p, _ = measure(None)
    out = {
        "workload": "beam 160x40x40 hexes x 6 tets, 50 iterations, dt 1/60, KineticEnergyMinimum initial guess",
        "ms_per_step": ms_a,
        "value": n_free * iters / (ms_a * 1e-3),
        "unit": UNIT,
        "grad_norm_after_one_step": g_a,
        "plain_ms_per_step": ms_p,
        "plain_grad_norm_after_one_step": g_p,
    }
    out.update({"path": "linear", "eta": 0.2, "tau": 2.0} if kind == "trust_region" else {"window": 5})
    return out


def run_contact(args, pbat, torch):
    """Contact scene: 16 cubes (16^3 hexes, 0.6 m) above a pinned 64x64x2 slab, 91,283 vertices,
    442,368 tets, 66,560 collision triangles; 30 iterations per step, dt = 1/60, muC = 1e7.  Each
    step rebuilds the active set (LBVH over swept triangle boxes), refreshes the contact lists and
    runs the contact-aware colour sweeps; timed with CUDA events on the integrator's stream.
    The cubes are first let fall for 60 untimed steps (they rest on the slab, in contact, from
    about step 40 on); then min(steps, 30) steps are timed, so the figure describes the
    contact-rich phase whatever --steps is."""
    from physicsbasedanimationtoolkit_gb300 import meshgen

    w = meshgen.contact_scene_workload()
    d = (pbat.sim.vbd.Data().with_volume_mesh(w["X"].T, w["T"].T).with_surface_mesh(w["V"], w["F"].T)
         .with_bodies(w["B"]).with_material(w["rho"], w["mu"], w["lam"]).with_dirichlet_vertices(w["dbc"])
         .with_contact_parameters(1e7, 0.3, 1e-3).with_initialization_strategy(2).construct())
    I = pbat.gpu.vbd.Integrator(d)
    dt, iters = 1 / 60, 30
    settle, timed = 60, min(args.steps, 30)
    for _ in range(max(settle, args.warmup)):
        I.step(dt, iters, 1)
    if args.contact_launch:
        lanes, block = args.contact_launch
        I.lanes_per_vertex, I.gpu_block_size = lanes, block
    else:
        lanes, block, _ = I.autotune(dt, iters, 1)  # restores the state after each candidate
    for _ in range(args.warmup):
        I.step(dt, iters, 1)
    I.synchronize()
    sp = C.c_void_p()
    from physicsbasedanimationtoolkit_gb300 import _capi
    _capi.check(_capi.lib().pbgb_vbd_stream(I.handle, C.byref(sp)), I.handle)
    stream = torch.cuda.ExternalStream(sp.value)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed_contact")  # lets ncu --nvtx-include select the timed steps
    e0.record(stream)
    for _ in range(timed):
        I.step(dt, iters, 1)
    e1.record(stream)
    I.synchronize()
    torch.cuda.nvtx.range_pop()
    t = e0.elapsed_time(e1) * 1e-3
    fc, active = I.contacts()
    return {
        "workload": "16 cubes of 16^3 hexes on a pinned 64x64x2 slab, vertex-triangle contact, 30 iterations",
        "n_vertices": int(I.n_vertices),
        "n_tets": int(I.n_tets),
        "settle_steps": max(settle, args.warmup) + args.warmup,
        "timed_steps": timed,
        "autotuned": {"lanes": lanes, "block": block},
        "value": I.n_free * iters * timed / t,
        "unit": UNIT,
        "ms_per_step": 1e3 * t / timed,
        "launches_per_step": int(I.launches_per_step(iters, 1)),
        "active_vertices": int(active.sum()),
        "vertices_with_contacts": int((fc >= 0).any(axis=1).sum()),
    }


LBVH_BYTES_PER_BOX = 312  # Morton 40, 4 radix passes 84, Karras 36, leaf 68, internal node 84


def run_lbvh(args, _capi, torch):
    """LBVH build over 4,194,304 seeded boxes (centres U[0,1)^3, half-extents U[0, 1e-3)) from
    device arrays: Morton codes, the stable 4-pass radix sort, the Karras hierarchy and the bottom-up
    boxes (leaf gather fused in); CUDA events on the BVH's stream.  Algorithmic bytes per box:
    Morton 40 (two boxes read, code and index written); radix 4 x (key read by the count, key and
    index read and written by the scatter) = 80, plus ~4 of digit counters; Karras 36 (codes read,
    children, parents and rightmost leaves written); leaf 68 (index, gathered box, leaf box
    written); internal node 84 (visit counter cleared and added 8, children 8, sibling box 32, box
    written 32, parent 4)."""
    n = 1 << 22
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    c = torch.rand((n, 3), device="cuda", generator=g)
    e = torch.rand((n, 3), device="cuda", generator=g) * 1e-3
    lo = torch.zeros((n, 4), device="cuda")
    hi = torch.zeros((n, 4), device="cuda")
    lo[:, :3] = c - e
    hi[:, :3] = c + e
    wmin = np.zeros(3, np.float32)
    wmax = np.ones(3, np.float32)
    L = _capi.lib()
    b = C.c_void_p()
    _capi.check_bvh(L.pbgb_bvh_create(n, C.byref(b)), b)
    try:
        sp = C.c_void_p()
        _capi.check_bvh(L.pbgb_bvh_stream(b, C.byref(sp)), b)
        stream = torch.cuda.ExternalStream(sp.value)
        torch.cuda.synchronize()

        def build():
            _capi.check_bvh(L.pbgb_bvh_build_device(b, n, C.c_void_p(lo.data_ptr()), C.c_void_p(hi.data_ptr()),
                                                     wmin.ctypes.data, wmax.ctypes.data), b)

        for _ in range(args.warmup):
            build()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            build()
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        # A host-buffer call surfaces the device-side error flags of the builds.
        nq = 1
        cnt = C.c_int64()
        q = np.array([[0.5, 0.5, 0.5]], np.float32)
        _capi.check_bvh(L.pbgb_bvh_overlaps(b, nq, q.ctypes.data, q.ctypes.data, None, 0, C.byref(cnt)), b)
    finally:
        L.pbgb_bvh_destroy(b)
    peak, peak_kind = peak_hbm()
    achieved = n * LBVH_BYTES_PER_BOX / (ms * 1e-3) / 1e9
    return {
        "workload": "LBVH build of 4,194,304 seeded boxes from device arrays (Morton, 4-pass radix sort, "
                    "Karras, leaf gather, bottom-up boxes)",
        "n_boxes": n,
        "ms_per_build": ms,
        "boxes_per_s": n / (ms * 1e-3),
        "algorithmic_bytes_per_box": LBVH_BYTES_PER_BOX,
        "achieved_GBs": achieved,
        "frac_of_hbm_peak": achieved / peak,
        "peak_kind": peak_kind,
    }


def run_single_launch(args, pbat, _capi, torch, meshes, datas, launch_config):
    """The comparison arm of the headline: one single-mesh integrator per mesh (one launch per
    colour), each on its own stream, with the headline's lanes and block size; CUDA events on the
    streams (time_single_launch).  Also the agreement with a fresh batch after the same steps."""
    dt, iters = 1 / 60, args.batch_iterations
    lanes, block = launch_config["lanes"], launch_config["block"]
    singles = []
    for d in datas:
        s = pbat.gpu.vbd.Integrator(d)
        s.lanes_per_vertex = lanes
        _capi.check(_capi.lib().pbgb_vbd_set_block_size(s.handle, block), s.handle)
        singles.append(s)
    for _ in range(args.warmup):
        for s in singles:
            s.step(dt, iters, 1)
    for s in singles:
        s.synchronize()
    B = pbat.gpu.vbd.BatchedIntegrator(datas)
    B.lanes_per_vertex = lanes
    _capi.check(_capi.lib().pbgb_vbd_set_block_size(B.handle, block), B.handle)
    for _ in range(args.warmup):
        B.step(dt, iters, 1)
    xb, off = B.x, B.vertex_offsets
    worst = 0.0
    for b, s in enumerate(singles):
        X = meshes[b]["X"]
        diag = np.linalg.norm(X.max(0) - X.min(0))
        worst = max(worst, float(np.abs(xb[:, off[b]: off[b + 1]] - s.x).max() / diag))
    del B
    n_free = sum(s.n_free for s in singles)
    t = time_single_launch(singles, dt, iters, args.steps, torch)
    out = {
        "value": n_free * iters * args.steps / t,
        "ms_per_step": 1e3 * t / args.steps,
        "launches_per_step": int(sum(s.launches_per_step(iters, 1) for s in singles)),
        "max_rel_diff_batched_vs_single": worst,
        "timing": "CUDA events: a start event all 256 streams wait on, an end event on every stream",
        "unit": UNIT,
    }
    del singles
    torch.cuda.empty_cache()
    return out


def run_beam(args, pbat, _capi, torch):
    """The single large beam: [0,4]x[0,1]^2 at 160x40x40 hexes (270,641 vertices, 1,536,000 tets),
    E 5e5, nu 0.48, x=0 face pinned, initial velocities U(-0.1, 0.1), Chebyshev rho 0.95, 50
    iterations per step, dt 1/60; the single-mesh integrator, launch autotuned.  Device-resident
    rate (CUDA events, L2 flushed between steps), the colour-sweep roofline, and the rate through
    the C ABI with host buffers."""
    w = workload_beam(args)
    data = make_data(pbat, w)
    vbd = pbat.gpu.vbd.Integrator(data)
    L = _capi.lib()
    h = vbd.handle
    dt, iters = 1 / 60, args.iterations
    if args.beam_launch:
        t_lanes, t_block = args.beam_launch
        vbd.lanes_per_vertex = t_lanes
        _capi.check(L.pbgb_vbd_set_block_size(h, t_block), h)
        t_ms = None
    else:
        t_lanes, t_block, t_ms = vbd.autotune(dt, iters, 1)
    n_free = vbd.n_free
    sp = C.c_void_p()
    _capi.check(L.pbgb_vbd_stream(h, C.byref(sp)), h)
    stream = torch.cuda.ExternalStream(sp.value)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        vbd.step(dt, iters, 1)
    vbd.synchronize()
    steps = args.steps
    t_total = 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_beam")
    for _ in range(steps):
        flush.add_(1.0)
        torch.cuda.synchronize()
        e0.record(stream)
        vbd.step(dt, iters, 1)
        e1.record(stream)
        vbd.synchronize()
        t_total += e0.elapsed_time(e1)
    torch.cuda.nvtx.range_pop()
    ms_per_step = t_total / steps
    launches_per_step = vbd.launches_per_step(iters, 1)
    sweeps_per_step = iters * vbd.n_colors
    nV = vbd.n_vertices
    xh = torch.empty((nV, 3), dtype=torch.float32, pin_memory=True)
    vh = torch.empty((nV, 3), dtype=torch.float32, pin_memory=True)
    _capi.check(L.pbgb_vbd_get_positions(h, xh.data_ptr()), h)
    _capi.check(L.pbgb_vbd_get_velocities(h, vh.data_ptr()), h)
    e2e_steps = max(3, steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        _capi.check(L.pbgb_vbd_set_positions(h, xh.data_ptr()), h)
        _capi.check(L.pbgb_vbd_set_velocities(h, vh.data_ptr()), h)
        _capi.check(L.pbgb_vbd_step(h, dt, iters, 1), h)
        _capi.check(L.pbgb_vbd_get_positions(h, xh.data_ptr()), h)
        _capi.check(L.pbgb_vbd_get_velocities(h, vh.data_ptr()), h)
    e2e_s = time.perf_counter() - t0
    peak, peak_kind = peak_hbm()
    bytes_per_launch = algorithmic_bytes(data) / vbd.n_colors
    # Launch duration: the event-timed step over its colour launches (an upper bound: the substep
    # kernels, ~2 % of the step, are counted against the sweeps).
    avg_launch_ms = ms_per_step / sweeps_per_step
    achieved = bytes_per_launch / (avg_launch_ms * 1e-3) / 1e9
    traffic, traffic_basis = traffic_from_profiles("vbd_sweep_beam160x40x40.md")
    out = {
        "config": beam_config(args, w),
        "value": n_free * iters / (ms_per_step * 1e-3),
        "unit": UNIT,
        "ms_per_step": ms_per_step,
        "steps": steps,
        "e2e": {"value": n_free * iters * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nV * 24,
                "d2h_bytes_per_step": nV * 24},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_basis": traffic_basis, "peak_kind": peak_kind,
                     "kernel": "staged_sweep_kernel (per-colour vertex Newton sweep)",
                     "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_us": avg_launch_ms * 1e3,
                     **dram_rate(traffic, avg_launch_ms, peak)},
        "launch_config": {"lanes": t_lanes, "block": t_block, "tuned_ms_per_step": t_ms},
        "launches_per_step": int(launches_per_step),
    }
    del vbd, flush
    torch.cuda.empty_cache()
    return out


def config_of(args, meshes):
    nV = sum(int(m["X"].shape[0]) for m in meshes)
    nT = sum(int(m["T"].shape[0]) for m in meshes)
    return {
        "workload": f"batch of {len(meshes)} cube grids, side U{{6..32}} hexes x 6 tets (seed 0), "
                    f"{args.batch_iterations} iterations, no acceleration, one persistent launch per step",
        "n_meshes": len(meshes),
        "n_vertices": nV,
        "n_tets": nT,
        "iterations": args.batch_iterations,
        "substeps": 1,
        "dt": 1 / 60,
        "material": "SNH, E log-uniform [1e5, 1e7], nu U(0.30, 0.48), rho 1000",
        "parallelism": f"replicas x{args.gpus}",
        "l2": "working set (~3 GB) > L2 (129 MB); L2 flushed (512 MB write) before every timed step",
    }


def beam_config(args, w):
    return {
        "workload": f"beam [0,4]x[0,1]^2 {args.nx}x{args.ny}x{args.nz} hexes x 6 tets, Chebyshev rho=0.95",
        "n_vertices": int(w["X"].shape[0]),
        "n_tets": int(w["T"].shape[0]),
        "iterations": args.iterations,
        "substeps": 1,
        "dt": 1 / 60,
        "material": "SNH E=5e5 nu=0.48 rho=1000",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--iterations", type=int, default=50)
    ap.add_argument("--nx", type=int, default=160)
    ap.add_argument("--ny", type=int, default=40)
    ap.add_argument("--nz", type=int, default=40)
    ap.add_argument("--lanes", type=int, default=0, help="headline and --only batch: lanes per vertex instead of autotuning")
    ap.add_argument("--block", type=int, default=0, help="headline with --lanes: block size (default 256)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-beam", dest="beam", action="store_false", default=True,
                    help="skip the single large beam (Chebyshev, 50 iterations) leg")
    ap.add_argument("--batch-meshes", type=int, default=256)
    ap.add_argument("--no-single", action="store_true",
                    help="--only batch: skip the one-integrator-per-mesh comparison (profiling runs)")
    ap.add_argument("--batch-iterations", type=int, default=20)
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false", default=True,
                    help="skip the adjoint (bwd/fwd) measurement on the differentiation beam")
    ap.add_argument("--no-contact", dest="contact", action="store_false", default=True,
                    help="skip the contact-scene step measurement")
    ap.add_argument("--no-lbvh", dest="lbvh", action="store_false", default=True,
                    help="skip the LBVH build measurement")
    ap.add_argument("--no-anderson", dest="anderson", action="store_false", default=True,
                    help="skip the Anderson-acceleration measurement")
    ap.add_argument("--no-trust-region", dest="trust_region", action="store_false", default=True,
                    help="skip the trust-region-acceleration measurement")
    ap.add_argument("--contact-launch", type=lambda t: tuple(int(v) for v in t.split(",")), default=None,
                    metavar="LANES,BLOCK", help="contact leg: use these lanes per vertex and block size instead "
                    "of autotuning (for profiling runs that must launch what a timed run launched)")
    ap.add_argument("--beam-launch", type=lambda t: tuple(int(v) for v in t.split(",")), default=None,
                    metavar="LANES,BLOCK", help="beam leg: use these lanes per vertex and block size instead of "
                    "autotuning (profiling runs)")
    ap.add_argument("--no-broyden", dest="broyden", action="store_false", default=True,
                    help="skip the Broyden-acceleration measurement")
    ap.add_argument("--only", choices=["batch", "beam", "adjoint", "contact", "lbvh", "anderson", "broyden", "trust_region"],
                    default=None,
                    help="run only this secondary measurement and print its figures (no benchmark line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch

    from physicsbasedanimationtoolkit_gb300 import _capi, pbat
    from physicsbasedanimationtoolkit_gb300.replicas import Replicas

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    group = Replicas("nccl", device=torch.device("cuda", local))
    rank, world = group.rank, group.world

    if args.only:
        legs = {
            "batch": lambda: run_batch(args, pbat, _capi, torch, with_single=not args.no_single),
            "beam": lambda: run_beam(args, pbat, _capi, torch),
            "adjoint": lambda: run_adjoint(args, pbat, torch),
            "contact": lambda: run_contact(args, pbat, torch),
            "lbvh": lambda: run_lbvh(args, _capi, torch),
            "anderson": lambda: run_accelerated(args, pbat, torch, "anderson"),
            "trust_region": lambda: run_accelerated(args, pbat, torch, "trust_region"),
            "broyden": lambda: run_accelerated(args, pbat, torch, "broyden"),
        }
        if rank == 0:
            print(json.dumps({"only": args.only, args.only: legs[args.only]()}))
        group.close()
        return 0

    meshes, datas = batch_workload(args, pbat)
    L = _capi.lib()
    dt, iters = 1 / 60, args.batch_iterations
    B = pbat.gpu.vbd.BatchedIntegrator(datas)
    h = B.handle
    if args.lanes:
        B.lanes_per_vertex = args.lanes
        if args.block:
            _capi.check(L.pbgb_vbd_set_block_size(h, args.block), h)
        tuned = None
    else:
        # The integrator's own autotuner (public API; restores the state after each candidate).
        t_lanes, t_block, t_ms = B.autotune(dt, iters, 1)
        tuned = {"lanes": t_lanes, "block": t_block, "ms_per_step": t_ms}
    n_free = B.n_free
    sp = C.c_void_p()
    _capi.check(L.pbgb_vbd_stream(h, C.byref(sp)), h)
    stream = torch.cuda.ExternalStream(sp.value)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        B.step(dt, iters, 1)
    B.synchronize()

    # ---- device-resident throughput (CUDA events on the integrator's stream) --------------------
    t_total = 0.0
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    group.barrier()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed_headline")  # lets ncu --nvtx-include select the timed steps
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.add_(1.0)  # L2 flush outside the timed interval
            torch.cuda.synchronize()
            ev0[k].record(stream)
            B.step(dt, iters, 1)
            ev1[k].record(stream)
            B.synchronize()
            t_total += ev0[k].elapsed_time(ev1[k])
        torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    group.barrier()
    t_total = group.max(t_total)
    ms_per_step = t_total / args.steps
    updates_per_step = n_free * iters
    value = group.sum(updates_per_step * args.steps) / (t_total * 1e-3)
    launches_per_step = B.launches_per_step(iters, 1)

    # ---- end to end through the C ABI with host buffers -----------------------------------------
    nV = B.n_vertices
    xh = torch.empty((nV, 3), dtype=torch.float32, pin_memory=True)
    vh = torch.empty((nV, 3), dtype=torch.float32, pin_memory=True)
    _capi.check(L.pbgb_vbd_get_positions(h, xh.data_ptr()), h)
    _capi.check(L.pbgb_vbd_get_velocities(h, vh.data_ptr()), h)
    e2e_steps = max(3, args.steps // 2)
    group.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        _capi.check(L.pbgb_vbd_set_positions(h, xh.data_ptr()), h)
        _capi.check(L.pbgb_vbd_set_velocities(h, vh.data_ptr()), h)
        _capi.check(L.pbgb_vbd_step(h, dt, iters, 1), h)
        _capi.check(L.pbgb_vbd_get_positions(h, xh.data_ptr()), h)
        _capi.check(L.pbgb_vbd_get_velocities(h, vh.data_ptr()), h)
    e2e_s = group.max(time.perf_counter() - t0)
    e2e_value = group.sum(updates_per_step * e2e_steps) / e2e_s
    io_bytes = nV * 3 * 4 * 2
    persistent = B.persistent
    lanes_used = B.lanes_per_vertex
    del B, flush
    torch.cuda.empty_cache()

    if rank == 0:
        peak, peak_kind = peak_hbm()
        bytes_per_step = batch_algorithmic_bytes(datas, iters)
        # One persistent launch per step: the launch duration is the event-timed step (the
        # counters' memset node before it, ~2 us, is counted against it).
        avg_launch_ms = ms_per_step / max(launches_per_step, 1)
        achieved = bytes_per_step / max(launches_per_step, 1) / (avg_launch_ms * 1e-3) / 1e9
        traffic, traffic_basis = traffic_from_profiles("batched_step_cfg3.md")
        launch_config = {"autotuned": tuned is not None, "lanes": lanes_used,
                         "block": tuned["block"] if tuned else (args.block or 256), "persistent": persistent}
        single = run_single_launch(args, pbat, _capi, torch, meshes, datas, launch_config)
        cpu = None if args.no_cpu_baseline else cpu_baseline(meshes, iters)
        beam = run_beam(args, pbat, _capi, torch) if args.beam else None
        adjoint = run_adjoint(args, pbat, torch) if args.adjoint else None
        contact = run_contact(args, pbat, torch) if args.contact else None
        lbvh = run_lbvh(args, _capi, torch) if args.lbvh else None
        anderson = run_accelerated(args, pbat, torch, "anderson") if args.anderson else None
        trust_region = run_accelerated(args, pbat, torch, "trust_region") if args.trust_region else None
        broyden = run_accelerated(args, pbat, torch, "broyden") if args.broyden else None
        launches = launches_per_step * args.steps
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": config_of(args, meshes),
            "single_launch_value": single["value"],
            "speedup_vs_single_launch": single["value"] and value / single["value"],
            "single_launch": single,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": io_bytes,
                    "d2h_bytes_per_step": io_bytes,
                    "path": "C ABI pbgb_vbd_set_positions/velocities + step + get_positions/velocities, pinned host buffers"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_basis": traffic_basis,
                         "peak_kind": peak_kind,
                         "kernel": "batched_step_kernel (persistent step of the whole batch)",
                         "algorithmic_bytes_per_launch": bytes_per_step / max(launches_per_step, 1),
                         "avg_launch_us": avg_launch_ms * 1e3,
                         "avg_launch_us_basis": "timed steps (CUDA events on the integrator's stream) / launches per step",
                         **dram_rate(traffic, avg_launch_ms, peak)},
            "launch_config": launch_config,
            "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "clocks": clocks.summary(),
            "n_free_vertices": n_free,
            "beam": beam,
            "adjoint": adjoint,
            "contact": contact,
            "lbvh": lbvh,
            "anderson": anderson,
            "trust_region": trust_region,
            "broyden": broyden,
        }
        print(json.dumps(line))
    group.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
