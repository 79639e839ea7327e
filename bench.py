#!/usr/bin/env python3
"""Benchmark of the pyCudaPolygon hot path on GB300.

Workload (one "step"): one FIRE step of the plain method at scale -- 4096
polygons of 32 vertices (131,072 vertices), 50:50 bidisperse radii 1.4,
packing fraction 0.88, seeded synthetic system -- with the reference's full
step: Verlet update, edge-midpoint cells, contact search (broad phase, narrow
phase, exit matching), SHAKE (5 iterations, retry x10), overlap energy and
force, constraint projection, energy-rollback test and FIRE velocity update.

metric  pair evals/s: polygon pairs (a < b) taken through the narrow phase,
        exit matching and force per second (the pairs whose bounding circles
        and crossing-margin boxes meet).  `value` is measured with the system resident in HBM, L2 flushed
        (256 MiB write) before every timed step, CUDA events around each step.
e2e     the same metric through the C ABI with host buffers: positions copied
        from pinned host memory in, the step, positions copied back, per step.

--impl reference times the CPU restatement of the reference (oracle/, C with
OpenMP on all host cores) on the same workload; the reference itself is CUDA
code that does not build as shipped and has no CPU implementation.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair evals/s"
UNIT = "pair evals/s"
N_POLY, N_VERT, PHI = 4096, 32, 0.88
WORKLOAD = ("plain FIRE step at scale: 4096 polygons x 32 vertices (131072 vertices), "
            "phi 0.88, cell list + narrow phase + outersections + overlap force + "
            "constraint projection + SHAKE (5, retry 50)")
FIRE_ARGS = dict(dtMax=0.1, alphaStart=0.1, fAlpha=0.99, fInc=1.1, fDec=0.5, nMin=5, shakeIter=5)
# the workload as both arms report it
CONFIG = {"workload": WORKLOAD, "polygons": N_POLY, "vertices_per_polygon": N_VERT, "phi": PHI,
          "l2": "flushed before every timed step (256 MiB write)",
          "fire": "dt0 1e-3, dtMax 0.1, alpha0 0.1, fAlpha 0.99, fInc 1.1, fDec 0.5, "
                  "nMin 5, shakeIter 5"}
PAIR_RULE = ("a pair eval is a polygon pair a < b handed to the narrow phase (bounding "
             "circles meet and boxes padded by the crossing margin meet), counted on the "
             "device over the timed steps, rollback searches included; the CPU arms count "
             "the same rule in numpy at both ends of their runs; circle_pairs_per_step is "
             "the looser count of pairs whose bounding circles meet")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_over_ranks(ms, pairs, dist, device):
    """Whole-job figures of independent replicas: the slowest rank's time and
    the pair evaluations of all ranks (no data-path collective: this is the
    only exchange, after the timed region)."""
    import torch
    if dist is None:
        return float(ms), float(pairs)
    t = torch.tensor([ms, float(pairs)], dtype=torch.float64, device=device)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(t[1])


# ------------------------------------------------------------------ clocks
class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, the
    driver's library, by ctypes) every millisecond on a thread: the timed
    region of a short run is a few milliseconds, below nvidia-smi's period.
    Reading clocks changes no setting of the GPU."""
    HW_SLOWDOWN, SW_THERMAL, HW_THERMAL, SW_POWER_CAP = 0x8, 0x20, 0x40, 0x4

    def __init__(self, index, period_s=0.001):
        import ctypes
        self.ok = False
        self.samples, self.reasons, self.max_mhz = [], 0, None
        self.period = period_s
        try:
            self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return
        self.c = ctypes
        if self.nv.nvmlInit_v2() != 0:
            return
        self.h = ctypes.c_void_p()
        if self.nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            return
        mx = ctypes.c_uint()
        if self.nv.nvmlDeviceGetMaxClockInfo(self.h, ctypes.c_int(1), ctypes.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        try:
            self.reasons_fn = self.nv.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self.reasons_fn = self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        self.ok = True

    def _poll(self):
        c = self.c
        clk, rs = c.c_uint(), c.c_ulonglong()
        while not self.stop:
            if self.nv.nvmlDeviceGetClockInfo(self.h, c.c_int(1), c.byref(clk)) == 0:
                self.samples.append(float(clk.value))
            if self.reasons_fn(self.h, c.byref(rs)) == 0:
                self.reasons |= int(rs.value)
            time.sleep(self.period)

    def __enter__(self):
        self.stop = False
        if self.ok:
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
        return self

    def __exit__(self, *a):
        self.stop = True
        if self.ok:
            self.t.join(timeout=2)

    def summary(self):
        names = []
        for bit, nm in ((self.HW_SLOWDOWN, "hw_slowdown"), (self.HW_THERMAL, "hw_thermal_slowdown"),
                        (self.SW_THERMAL, "sw_thermal_slowdown"), (self.SW_POWER_CAP, "sw_power_cap")):
            if self.reasons & bit:
                names.append(nm)
        return {"sm_mhz": statistics.median(self.samples) if self.samples else None,
                "sm_max_mhz": self.max_mhz, "reasons": sorted(names),
                "samples": len(self.samples), "source": "NVML every 1 ms"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "10"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workload
def make_workload(seed):
    from pycudapolygon_gb300.systems import make_system
    return make_system(N_POLY, N_VERT, PHI, seed=seed)


def candidate_pairs(positions, start, pairs_out=None):
    """Pair evaluations of one contact search, counted with the broad phase's
    rules: (narrow, circle), where circle counts the pairs a < b whose
    bounding circles meet and narrow the subset whose boxes, padded by the
    crossing margin, also meet (the pairs the narrow phase tests).  A list
    given as pairs_out receives the narrow pairs (a, b)."""
    xy = positions.reshape(-1, 2)
    P = len(start) - 1
    cx, cy, R, L = np.zeros(P), np.zeros(P), np.zeros(P), np.zeros(P)
    bw, bh = np.zeros(P), np.zeros(P)
    for p in range(P):
        ring = xy[start[p]:start[p + 1]]
        rel = (ring - ring[0] + 0.5) % 1.0 - 0.5
        lo, hi = rel.min(axis=0), rel.max(axis=0)
        c = (ring[0] + 0.5 * (lo + hi)) % 1.0
        cx[p], cy[p] = c
        R[p] = 0.5 * np.hypot(*(hi - lo)) * 1.0001 + 4e-6
        bw[p], bh[p] = hi - lo
        e = (np.roll(ring, -1, axis=0) - ring + 0.5) % 1.0 - 0.5
        L[p] = np.sqrt((e * e).sum(axis=1)).max()
    circle = narrow = 0
    for p in range(P - 1):
        near, both = _pair_masks(p, cx, cy, R, L, bw, bh)
        circle += int(np.count_nonzero(near))
        narrow += int(np.count_nonzero(both))
        if pairs_out is not None:
            pairs_out.extend((p, p + 1 + int(q)) for q in np.flatnonzero(both))
    return narrow, circle


def _pair_masks(p, cx, cy, R, L, bw, bh):
    """Polygons q > p whose bounding circles meet p's (near), and the subset
    whose boxes, padded by the crossing margin, meet too (both)."""
    dx = (cx[p + 1:] - cx[p] + 0.5) % 1.0 - 0.5
    dy = (cy[p + 1:] - cy[p] + 0.5) % 1.0 - 0.5
    rr = R[p] + R[p + 1:] + 1e-5
    near = dx * dx + dy * dy <= rr * rr
    m = 2.0 * (4e-6 + 1e-3 * L[p] * L[p + 1:]) + 2e-6
    box = (np.abs(dx) <= 0.5 * (bw[p] + bw[p + 1:]) + m) & \
          (np.abs(dy) <= 0.5 * (bh[p] + bh[p + 1:]) + m)
    return near, near & box


def prepare_gpu(seed):
    import pycudapolygon_gb300 as pg
    from pycudapolygon_gb300.systems import load_into
    pg.build()
    lib = pg.load_module()
    s = make_workload(seed)
    m = load_into(lib.Model(s.num_vertices), s)
    m.shakeProject(200, 1e-15)          # start on the constraint manifold
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    m.fireSetup(-1.0, 1e-3, 0, **FIRE_ARGS)
    return lib, m, s


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib, m, s = prepare_gpu(args.seed + rank)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        flush.fill_(1)
        m.fireContinue(1)
    st = m.fireStatus()
    if st[8]:
        raise RuntimeError("contact buffers grew during warm-up; rerun")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    pairs0 = m.getNarrowPairTotal()
    circle0 = m.getPairCount()
    launches0 = m.getLaunchCount()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = NvmlClocks(local)
    if not clk.ok:
        clk = ClockSampler(local)
    with clk:
        for i in range(args.steps):
            flush.fill_(i & 255)
            ev[i][0].record()
            m.fireContinue(1)
            ev[i][1].record()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    st = m.fireStatus()
    if st[8]:
        raise RuntimeError("contact buffers grew inside the timed region; rerun")
    ms = sum(a.elapsed_time(b) for a, b in ev)
    pairs = m.getNarrowPairTotal() - pairs0
    circle = m.getPairCount() - circle0
    narrow_last = m.getNarrowPairCount()
    launches = m.getLaunchCount() - launches0
    ms, pairs = reduce_over_ranks(ms, pairs, dist, "cuda")
    value = pairs / (ms / 1e3)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded bidisperse star polygons; the reference publishes no inputs)",
        "config": dict(CONFIG, parallelism="replicas" if ws > 1 else "single"),
        "pairs": {"rule": PAIR_RULE, "pair_evals_per_step": pairs / max(1, args.steps) / ws,
                  "circle_pairs_per_step": circle / max(1, args.steps),
                  "self_pairs_last_step": narrow_last[1]},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "fire_state": {"energy": st[0], "dt": st[1], "max_force": st[4], "steps": st[5]},
    }
    if rank == 0 and not args.no_roofline:
        result["roofline"], result["fp64"] = roofline(m, s, torch, flush, args)
    if rank == 0 and reference_kernels_record() is not None:
        result["reference_kernels_gb300"] = reference_kernels_record()
    if rank == 0 and not args.no_e2e:
        result["e2e"] = e2e(args, s)
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(args, s, pairs / max(1, args.steps) / ws)
    if rank == 0 and not args.no_stop:
        result["time_to_stop"] = time_to_stop(args, torch)
    if rank == 0 and args.batch_systems > 0:
        result["batched"] = batched(args, torch)
    if rank == 0 and args.warm_start_train > 0:
        from pycudapolygon_gb300 import warmstart
        result["warm_start"] = warmstart.experiment(
            n_train=args.warm_start_train, n_test=max(1, args.warm_start_train // 4),
            epochs=10, physics=0.1)
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result))


def roofline(m, s, torch, flush, args):
    """Dominant contact kernel: the narrow phase (warp per candidate pair).
    Algorithmic bytes per launch: 16 (n_a + n_b) + 24 per pair it is handed
    (both rings and the pair entry) and 16 n + 24 per self pair."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs")
    src = "measured"
    if not hbm:
        hbm, src = 6800.0, "fallback"
    reps = 20
    times = []
    m.updateNeighborCells()
    for _ in range(reps):
        m.contactsStage(0)
        flush.fill_(3)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        m.contactsStage(1)
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    m.contactsStage(2)
    ms = statistics.median(times)
    n = N_VERT
    P = N_POLY
    pairs, selfs = m.getNarrowPairCount()
    bytes_launch = pairs * (16 * 2 * n + 24) + selfs * (16 * n + 24)
    achieved = bytes_launch / (ms / 1e3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "narrow_phase_traffic.json")
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic, "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)",
            "kernel": "k_narrow (+ k_narrow_over, k_narrow_slow, k_fixup: contact stage 1)",
            "launch_ms": ms, "algorithmic_bytes": bytes_launch, "pairs": pairs,
            "self_pairs": selfs}
    # the projection, SHAKE and force kernels are bound by the FP64 pipe, not
    # by HBM: their FP64-pipe activity from the committed ncu capture
    fp64 = None
    p64 = os.path.join(ROOT, "profiles", "fp64_pipe_4096x32.json")
    if os.path.exists(p64):
        try:
            fp64 = json.load(open(p64))
        except (OSError, ValueError):
            fp64 = None
    return roof, fp64


def reference_kernels_record():
    """The reference's own kernels, rebuilt for sm_103a, against this
    repository's on one evaluation of a 4096 x 32 system on a GB300: the
    committed result of oracle/ref_time.py (this benchmark does not run the
    reference's code)."""
    path = os.path.join(ROOT, "profiles", "reference_kernels_4096x32.json")
    try:
        d = json.load(open(path))
        return {"source": "profiles/reference_kernels_4096x32.json (oracle/ref_time.py)",
                "workload": d["workload"], "timing": d["timing"],
                "evaluation_ms": d["evaluation_ms"], "speedup": d["speedup"],
                "stage_ms": {"reference": d["reference_kernels_sm103a"]["stage_ms"],
                             "this_repository": d["this_repository"]["stage_ms"]}}
    except (OSError, ValueError, KeyError, TypeError):
        return None


def e2e(args, s):
    """Same metric through the C ABI with host buffers (pinned), per step:
    positions in, one FIRE step, positions out."""
    import torch

    from pycudapolygon_gb300 import cabi
    from pycudapolygon_gb300.systems import make_system  # noqa: F401
    c = cabi.CModel(s.num_vertices)
    c.set_num_vertices(s.num_vertices)
    c.set_start_indices(s.start_indices)
    c.set_positions(s.positions)
    c.set_target_areas(s.target_areas)
    c.set_target_edge_lengths(s.target_edge_lengths)
    c.initialize_neighbor_cells()
    c.set_max_edge_length(s.max_edge_length)
    c.shake_project(200)
    c.update_polygon_geometry()
    c.update_neighbor_cells()
    c.update_neighbors()
    c.update_outersections()
    c.update_force_energy()
    c.project_force()
    host = torch.empty(2 * s.num_vertices, dtype=torch.float64, pin_memory=True).numpy()
    c.get_positions_into(host)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    dt, alpha, npos = 1e-3, 0.1, 0
    for _ in range(args.warmup):
        _, dt, alpha, npos = c.fire_step(dt, alpha, npos)
    c.get_positions_into(host)
    p0 = c.narrow_pair_total()
    total = 0.0
    steps = args.steps          # same trajectory as the device-timed steps
    for i in range(steps):
        flush.fill_(i & 255)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.set_positions(host)
        _, dt, alpha, npos = c.fire_step(dt, alpha, npos)
        c.get_positions_into(host)
        total += time.perf_counter() - t0
    pairs = c.narrow_pair_total() - p0
    ctrl_bytes = c.L.pcp_control_block_bytes()   # read back after the step
    c.close()
    return {"value": pairs / total, "unit": UNIT,
            "h2d_bytes_per_step": 16 * s.num_vertices,
            "d2h_bytes_per_step": 16 * s.num_vertices + ctrl_bytes,
            "steps": steps, "ms_per_step": total / steps * 1e3,
            "path": "C ABI (pcp_model_set_positions, pcp_model_fire_step, "
                    "pcp_model_get_positions), pinned host buffers, wall clock"}


# ------------------------------------------------------------- time to stop
STOP_SYSTEM = dict(num_polygons=64, n=16, phi=0.85)   # 1024 vertices
STOP_SEEDS = list(range(1, 9))
STOP_THR, STOP_MAX_STEPS = 1e-10, 100000
FIRE_POS = (0.1, 0.1, 0.99, 1.1, 0.5, 5, 5)          # dtMax .. shakeIter


def reference_driver(m, thr=STOP_THR, dt=1e-3, max_steps=STOP_MAX_STEPS):
    """The reference's Python minimizeFIRE for the normal model
    (pyCudaPolygon.py:674-731 with its loop, :653-672) on any object with the
    Model method names: initForceEnergy (which sets the cell size to 0.5),
    the small gradient step, then one minimizeFIREStep and one
    getMaxUnbalancedForce per step until |F|max <= thr or six steps returned
    an energy within 1e-15 of the step before.  Returns (E, dt, steps,
    |F|max, stop reason)."""
    m.resetVelocities()
    m.initializeNeighborCells()
    m.setMaxEdgeLength(0.5)
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    m.updatePolygonGeometry()
    m.updateForceEnergy()
    m.projectForce()
    m.updatePositions(dt)
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    m.updateForceEnergy()
    m.projectForce()
    m.resetVelocities()
    m.resetVelocities()
    m.updatePolygonGeometry()
    m.updateForceEnergy()
    m.projectForce()
    alpha, npos, prev, flat = 0.1, 0, 1e9, 0
    e, f = None, None
    for step in range(max_steps):
        e, dt, alpha, npos = m.minimizeFIREStep(dt, alpha, npos, *FIRE_POS)
        f = m.getMaxUnbalancedForce()
        if abs(e - prev) < 1e-15:
            flat += 1
        if flat > 5:
            return e, dt, step + 1, f, "stagnation"
        prev = e
        if f <= thr:
            return e, dt, step + 1, f, "tolerance"
    return e, dt, max_steps, f, "step limit"


def _stop_system(seed, model):
    from pycudapolygon_gb300.systems import load_into, make_system
    s = make_system(seed=seed, **STOP_SYSTEM)
    m = load_into(model(s.num_vertices), s)
    m.shakeProject(100, 1e-15)
    return m


def time_to_stop(args, torch):
    """Minimisation of the 64 x 16 (phi 0.85) systems to the reference
    driver's stop, per system: on the GPU through the device-resident driver
    (one call, the loop and its stop tests on the device) and through the
    reference's per-step Python loop on the pybind module, and on the CPU
    oracle through the same loop.  Wall time per system includes the calls
    before the loop."""
    import pycudapolygon_gb300 as pg
    from oracle import oracle as orc
    lib = pg.load_module()
    _stop_system(STOP_SEEDS[0], lib.Model).minimizeFIREDevice(STOP_THR, 1e-3, 50)   # warm-up
    dev, loop, cpu = [], [], []
    for seed in STOP_SEEDS:
        m = _stop_system(seed, lib.Model)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = m.minimizeFIREDevice(STOP_THR, 1e-3, STOP_MAX_STEPS)
        t1 = time.perf_counter()
        st = m.fireRunStats()
        dev.append(dict(seconds=t1 - t0, steps=r[2], energy=r[0], max_force=m.getMaxUnbalancedForce(),
                        reason="stagnation" if st[0] else ("tolerance" if r[2] < STOP_MAX_STEPS
                                                           else "step limit")))
        m = _stop_system(seed, lib.Model)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = reference_driver(m)
        t1 = time.perf_counter()
        loop.append(dict(seconds=t1 - t0, steps=r[2], energy=r[0], reason=r[4]))
    threads = cpu_threads()
    orc.set_threads(threads)
    for seed in STOP_SEEDS:
        o = _stop_system(seed, orc.OracleModel)
        t0 = time.perf_counter()
        r = reference_driver(o)
        t1 = time.perf_counter()
        cpu.append(dict(seconds=t1 - t0, steps=r[2], energy=r[0], reason=r[4]))

    def mean(xs, k):
        return sum(x[k] for x in xs) / len(xs)
    same_steps = sum(a["steps"] == b["steps"] for a, b in zip(dev, cpu))
    de = max(abs(a["energy"] - b["energy"]) / max(abs(b["energy"]), 1e-300)
             for a, b in zip(dev, cpu) if a["steps"] == b["steps"]) if same_steps else None
    return {
        "workload": "64 polygons x 16 vertices, phi 0.85, seeds %d-%d; minimised by the "
                    "reference's Python FIRE driver rule (stop at |F|max <= 1e-10 or after six "
                    "steps with |dE| < 1e-15), dt0 1e-3" % (STOP_SEEDS[0], STOP_SEEDS[-1]),
        "converged_to_1e-10": sum(d["reason"] == "tolerance" for d in dev),
        "systems": len(STOP_SEEDS),
        "stop_reasons": sorted(set(d["reason"] for d in dev)),
        "steps": [d["steps"] for d in dev],
        "gpu_device_driver_s_per_system": mean(dev, "seconds"),
        "gpu_python_loop_s_per_system": mean(loop, "seconds"),
        "cpu_oracle_s_per_system": mean(cpu, "seconds"),
        "cpu_cores": threads,
        "gpu_vs_cpu_same_stop_step": "%d/%d" % (same_steps, len(STOP_SEEDS)),
        "gpu_vs_cpu_max_rel_energy_diff": de,
        "final_max_force": [d["max_force"] for d in dev],
    }


# ------------------------------------------------------------- many systems
BATCH_SYSTEMS, BATCH_SEED = 256, 2025


def batched(args, torch):
    """256 independent systems (polygons U{64..1024}, vertices per polygon
    U{12..48}, packing fraction U[0.80, 0.92], seeded) minimised by the
    reference Python driver's rule, per system: all at once through the
    batch (a pool of streams, several FIRE steps per graph launch, launch
    shapes from the autotuner), and one after the other through the
    device-resident single-system driver with the default launch shapes."""
    import pycudapolygon_gb300 as pg
    from pycudapolygon_gb300.systems import batched_specs, load_into, make_system
    lib = pg.load_module()
    specs = batched_specs(args.batch_systems, BATCH_SEED)
    systems = [make_system(P, nv, phi, seed=sd) for P, nv, phi, sd in specs]
    models = []
    for s in systems:
        m = load_into(lib.Model(s.num_vertices), s)
        m.shakeProject(100, 1e-15)
        models.append(m)
    start = [np.asarray(m.getPositions()) for m in models]

    def reset():
        for m, x in zip(models, start):
            m.setPositions(x)
        torch.cuda.synchronize()
    # one after the other, default launch shapes (a 1-step run first builds
    # each system's step graph outside the timed region)
    seq_steps, seq_conv = [], 0
    t_seq = 0.0
    for m, x in zip(models, start):
        m.minimizeFIREDevice(STOP_THR, 1e-3, 1, *FIRE_POS)
        m.setPositions(x)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = m.minimizeFIREDevice(STOP_THR, 1e-3, STOP_MAX_STEPS, *FIRE_POS)
        t_seq += time.perf_counter() - t0
        seq_steps.append(int(r[2]))
        seq_conv += int(m.fireRunStats()[0] == 0 and r[2] < STOP_MAX_STEPS)
    # all together: autotuned shapes, then a 1-step run that builds the
    # multi-step graphs, then the timed run
    reset()
    b = lib.Batch()
    for m in models:
        b.add(m)
    t0 = time.perf_counter()
    b.autotune(8)
    t_tune = time.perf_counter() - t0
    report = json.loads(b.report())
    reset()
    b.minimizeFIRE(1, STOP_THR, 1e-3, 1, *FIRE_POS)
    reset()
    t0 = time.perf_counter()
    out = b.minimizeFIRE(1, STOP_THR, 1e-3, STOP_MAX_STEPS, *FIRE_POS)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    n = len(models)
    return {
        "workload": "%d systems: polygons U{64..1024}, vertices per polygon U{12..48}, "
                    "phi U[0.80,0.92] (seed %d), %d vertices in all; each minimised by the "
                    "reference Python driver's rule (|F|max <= 1e-10 or six steps with "
                    "|dE| < 1e-15), dt0 1e-3" % (n, BATCH_SEED, sum(s.num_vertices for s in systems)),
        "batched_s_per_system": t_batch / n,
        "sequential_s_per_system": t_seq / n,
        "speedup": t_seq / t_batch,
        "batched_steps_total": int(out[:, 2].sum()),
        "sequential_steps_total": int(sum(seq_steps)),
        "batched_converged_to_1e-10": int(np.count_nonzero(out[:, 3] == 1)),
        "sequential_converged_to_1e-10": seq_conv,
        "batched_stopped_by_stagnation": int(np.count_nonzero(out[:, 3] == 2)),
        "batch": "16 streams, 8 FIRE steps per graph launch; both timings include the calls "
                 "before each system's loop",
        "autotune_s": t_tune,
        "autotune": report,
    }


# ------------------------------------------------------------------ CPU legs
def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_cpu_steps(s, steps, warmup, threads):
    """The CPU oracle (restatement of the reference) doing FIRE steps on the
    same system; returns (seconds, pair evals, steps)."""
    from oracle import oracle as orc
    from pycudapolygon_gb300.systems import load_into
    orc.set_threads(threads)
    o = load_into(orc.OracleModel(s.num_vertices), s)
    o.shakeProject(200, 1e-15)
    o.updatePolygonGeometry()
    o.updateNeighborCells()
    o.updateNeighbors()
    o.updateOutersections()
    o.updateForceEnergy()
    o.projectForce()
    dt, alpha, npos = 1e-3, 0.1, 0
    for _ in range(warmup):
        _, dt, alpha, npos = o.minimizeFIREStep(dt, alpha, npos)
    # the pair count moves slowly along a FIRE run: count it at both ends
    first = candidate_pairs(o.getPositions(), s.start_indices)[0]
    total = 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        _, dt, alpha, npos = o.minimizeFIREStep(dt, alpha, npos)
        total += time.perf_counter() - t0
    last = candidate_pairs(o.getPositions(), s.start_indices)[0]
    return total, 0.5 * (first + last) * steps, steps


def cpu_baseline(args, s, gpu_pairs_per_step):
    threads = cpu_threads()
    secs, pairs, steps = run_cpu_steps(s, args.cpu_steps, 1, threads)
    return {"value": pairs / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d FIRE steps of the same 4096x32 system (after 1 warm-up step) "
                      "by the C oracle with OpenMP, %.1f s" % (steps, secs)}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    s = make_workload(args.seed)
    threads = cpu_threads()
    secs, pairs, steps = run_cpu_steps(s, max(1, args.steps), max(0, args.warmup), threads)
    value = pairs / secs
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": secs / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded bidisperse star polygons; the reference publishes no inputs)",
        "config": dict(CONFIG, parallelism="single"),
        "pairs": {"rule": PAIR_RULE, "pair_evals_per_step": pairs / steps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d FIRE steps of the workload by the C restatement of the "
                                   "reference (oracle/), OpenMP on %d threads" % (steps, threads)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU implementation of the path (its kernels are CUDA; "
                "FIRE.h and shake.h are missing from it), so its algorithm is timed through "
                "the CPU restatement, which is checked against the reference's own kernels' "
                "outputs (tests/golden/ref_gpu_*.npz)",
    }))


def run_stages(args):
    """Each stage of one overlap evaluation, constraint projection and SHAKE
    run once per pass through the Model API (no graph, no gates), so that a
    profiler captures exactly one launch of every kernel per pass."""
    import torch
    lib, m, s = prepare_gpu(args.seed)
    for _ in range(args.stages):
        m.updateNeighborCells()
        m.updateNeighbors()
        m.updateOutersections()
        m.updateForceEnergy()
        m.projectForce()
        m.updatePositions(1e-3)          # off the constraint manifold, as after a Verlet move
        m.shakeProject(5, 1e-15)
    torch.cuda.synchronize()
    print(json.dumps({"stages": args.stages, "pairs": m.getPairCount(),
                      "launches": m.getLaunchCount()}))


def run_scrambled(args):
    """Profiling mode: one system of the many-systems workload (by rank in
    polygon count) with every vertex placed at random in the box, as a FIRE
    step whose Verlet move scrambled the polygons leaves it, and one contact
    search and overlap-force evaluation at cell size 0.5."""
    import torch
    import pycudapolygon_gb300 as pg
    from pycudapolygon_gb300.systems import batched_specs, load_into, make_system
    lib = pg.load_module()
    specs = batched_specs(BATCH_SYSTEMS, BATCH_SEED)
    order = sorted(range(len(specs)), key=lambda i: specs[i][0])
    P, nv, phi, sd = specs[order[args.scrambled]]
    s = make_system(P, nv, phi, seed=sd)
    m = load_into(lib.Model(s.num_vertices), s)
    m.setMaxEdgeLength(0.5)
    m.setPositions(np.random.default_rng(0).random(s.positions.size))
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    m.updateForceEnergy()
    torch.cuda.synchronize()
    print(json.dumps({"polygons": P, "vertices": s.num_vertices,
                      "records": m.getNumIntersections(), "pairs": m.getNarrowPairCount()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-steps", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-roofline", action="store_true")
    ap.add_argument("--no-stop", action="store_true")
    ap.add_argument("--warm-start-train", type=int, default=16,
                    help="training pairs of the learned warm start (0: skip it); a quarter "
                         "as many held-out seeds")
    ap.add_argument("--batch-systems", type=int, default=BATCH_SYSTEMS,
                    help="systems of the many-systems leg (0: skip it)")
    ap.add_argument("--stages", type=int, default=0,
                    help="profiling mode: run every stage this many times, no timing")
    ap.add_argument("--scrambled", type=int, default=-1,
                    help="profiling mode: one contact search and force on the scrambled state "
                         "of the many-systems workload's system of this rank in size")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.stages > 0:
        run_stages(args)
        return
    if args.scrambled >= 0:
        run_scrambled(args)
        return
    run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
