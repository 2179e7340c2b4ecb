"""Throughput of the em2d PIC step (push + deposit + current filter + Yee) on
GB300, in particle-steps/s.

Workload (one GPU): uniform thermal plasma, 2048 x 2048 cells, dx = dy = 0.1,
dt = 0.05, 200 steps, periodic, one electron species (m_q = -1), 4 x 4 particles per
cell (67,108,864 particles), isotropic thermal momentum 0.05, compensated
level-1 binomial current smoothing along x and y.  Initial particles are
seeded synthetic data with the reference's loading (ppc lattice, Gaussian
momenta, per-cell mean removed); all state is float32.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

One JSON line on rank 0.  Under torchrun (N > 1) every rank runs its own
independent copy of the workload (replicas, weak scaling, no collective on the
data path); time is the max over ranks.

``--impl reference`` times the reference's CPU algorithm for the same
workload on the host cores: the reference itself when its build is present
(oracle/_ref), else the C restatement under oracle/ built with the
reference's stock -Ofast flags.  Each step of it is a bounded sample of the
workload (a 1024 x 512 cell sub-box at the same density).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s per GB300 (push+deposit+Yee), batched & adjoint vs plain GPU"
UNIT = "particle-steps/s"
WORKLOAD = dict(name="em2d uniform thermal plasma 2048x2048, 4x4 ppc (67,108,864 particles)",
                nx=(2048, 2048), box=(204.8, 204.8), dt=0.05, ppc=(4, 4), uth=0.05, m_q=-1.0,
                smooth=("compensated", 1, "compensated", 1))
# algorithmic bytes: particle record read + written (2 x 28 B); per cell:
# gather E,B (24 B) + deposit J (12 B) in the push kernel, Yee reads E,B,J and
# writes E,B (60 B), each filter pass reads and writes J (24 B)
PART_BYTES = 56
PUSH_CELL_BYTES = 36
STEP_CELL_BYTES = 96
SMOOTH_PASS_BYTES = 24


def synth_particles(nx, ny, ppc, uth, seed):
    """Reference-style loading: particles on the ppc lattice of every cell
    (em2d/particles.c:168-179, 336-349), Gaussian momenta of width uth with the
    mean of every cell removed (particles.c:96-142).  Seeded numpy generator."""
    px, py = ppc
    npc = px * py
    ncell = nx * ny
    dt = np.dtype([("ix", "<i4"), ("iy", "<i4"), ("x", "<f4"), ("y", "<f4"),
                   ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])
    parts = np.empty(ncell * npc, dtype=dt)
    cell = np.arange(ncell, dtype=np.int64)
    parts["ix"] = np.repeat((cell % nx).astype(np.int32), npc)
    parts["iy"] = np.repeat((cell // nx).astype(np.int32), npc)
    lx = (np.float32(1.0 / px) * (np.arange(px) + 0.5)).astype(np.float32)
    ly = (np.float32(1.0 / py) * (np.arange(py) + 0.5)).astype(np.float32)
    parts["x"] = np.tile(np.tile(lx, py), ncell)
    parts["y"] = np.tile(np.repeat(ly, px), ncell)
    rng = np.random.default_rng(seed)
    for f in ("ux", "uy", "uz"):
        u = rng.standard_normal(ncell * npc, dtype=np.float32) * np.float32(uth)
        u = u.reshape(ncell, npc)
        u -= u.mean(axis=1, keepdims=True, dtype=np.float32)
        parts[f] = u.reshape(-1)
    return parts


# ---------------------------------------------------------------------------
# clocks during the timed region: NVML through ctypes (read-only queries)
# ---------------------------------------------------------------------------
class ClockSampler:
    REASONS = {0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap",
               0x8: "hw_slowdown", 0x10: "sync_boost", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
               0x100: "display_clock_setting"}

    def __init__(self, index):
        self.ok = False
        self.samples = []
        self.reasons = 0
        try:
            self.nv = ctypes.CDLL("libnvidia-ml.so.1")
            if self.nv.nvmlInit_v2() != 0:
                return
            self.h = ctypes.c_void_p()
            if self.nv.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(self.h)) != 0:
                return
            self.ok = True
        except OSError:
            return

    def _clock(self, kind, fn="nvmlDeviceGetClockInfo"):
        v = ctypes.c_uint()
        r = getattr(self.nv, fn)(self.h, kind, ctypes.byref(v))
        return v.value if r == 0 else None

    def max_sm(self):
        return self._clock(1, "nvmlDeviceGetMaxClockInfo") if self.ok else None

    def start(self):
        if not self.ok:
            return
        self.stop_flag = False

        def run():
            r = ctypes.c_ulonglong()
            while not self.stop_flag:
                c = self._clock(1)
                if c is not None:
                    self.samples.append(c)
                if self.nv.nvmlDeviceGetCurrentClocksEventReasons(self.h, ctypes.byref(r)) == 0:
                    self.reasons |= r.value
                time.sleep(0.002)

        self.t = threading.Thread(target=run, daemon=True)
        self.t.start()

    def stop(self):
        if not self.ok:
            return None
        self.stop_flag = True
        self.t.join()
        names = [n for b, n in self.REASONS.items() if self.reasons & b and n != "gpu_idle"]
        return {"sm_mhz": statistics.median(self.samples) if self.samples else None,
                "sm_max_mhz": self.max_sm(), "samples": len(self.samples), "reasons": names}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes (read + write) per launch of the push kernel, from one ncu
    capture recorded in profiles/push_traffic.json (None when absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "push_traffic.json")) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except (OSError, KeyError, ValueError):
        return None


# ---------------------------------------------------------------------------
# CPU references
# ---------------------------------------------------------------------------
def cpu_run(nx, ny, steps, warmup, fast=True):
    """Times the reference algorithm on the host: oracle/_ref (the reference
    compiled from its sources) when present, else the oracle port.  Returns
    (particle-steps/s, kind, particles)."""
    from oracle import pyoracle

    pyoracle.build()
    backend = "ref" if pyoracle.ref_available(fast) else "oracle"
    kind = "reference" if backend == "ref" else "port"
    W = WORKLOAD
    dx = W["box"][0] / W["nx"][0]
    if backend == "oracle":
        pyoracle.set_rand_seed(12345, 67890, backend=backend, fast=fast, fresh=True)
    else:
        pyoracle.set_rand_seed(12345, 67890, backend=backend, fast=fast)
    s = pyoracle.CpuSim([nx, ny], [nx * dx, ny * dx], W["dt"], backend=backend, fast=fast)
    # the reference's stock cell sort every 16 steps (particles.c:607); the
    # port keeps buffer order, which for runs this short (particles loaded
    # in cell order, moving 0.025 cells a step) reads the same memory
    s.add_species("electrons", W["m_q"], list(W["ppc"]), ufl=[0, 0, 0], uth=[W["uth"]] * 3, n_sort=16)
    sm = W["smooth"]
    s.set_smooth(sm[0], sm[1], sm[2], sm[3])
    n = s.np_(0)
    s.iter(warmup)
    t0 = time.perf_counter()
    s.iter(steps)
    t = time.perf_counter() - t0
    return n * steps / t, kind, n


def _cpu_worker(a):
    """one host process of the parallel CPU baseline (spawned)"""
    nx, ny, steps, warmup = a
    return cpu_run(nx, ny, steps, warmup)


def cpu_run_parallel(nx, ny, steps, warmup, procs):
    """`procs` concurrent single-threaded runs of the reference algorithm on
    the same sub-box (the reference's fan-out of independent runs); returns
    (aggregate particle-steps/s, kind, particles per run)."""
    import multiprocessing as mp

    from oracle import pyoracle

    pyoracle.build()
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(_cpu_worker, [(nx, ny, steps, warmup)] * procs)
    return sum(r[0] for r in res), res[0][1], res[0][2]


def run_reference(args):
    """The reference's CPU em2d on this host, on the bench's own workload.

    ``value``: the full 2048^2 deck (67,108,864 particles), one run, as the
    reference runs it: single-threaded, up to 2 untimed steps then up to 10
    timed ones (``--warmup`` / ``--steps`` when smaller: some 3.5 s a step on
    one core keeps the arm to about a minute; the rate is per step, so the
    bounded sample measures the same thing).  Beside it,
    ``host_aggregate``: the host-wide figure of independent single-threaded
    runs, one per core, each a 256^2-cell box of the same density (the
    reference's fan-out of independent runs for parameter scans), for the
    requested steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    procs = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    W = WORKLOAD
    nx, ny = W["nx"]
    steps1, warm1 = min(args.steps, 10), min(args.warmup, 2)
    v1, kind, n1 = cpu_run(nx, ny, steps1, warm1)
    vp, kind_p, npr = cpu_run_parallel(256, 256, args.steps, args.warmup, procs)
    line = {
        "impl": "reference", "metric": METRIC, "value": v1, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": n1 / v1 * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded reference loading)",
        "config": {"workload": W["name"], "nx": [nx, ny], "dx": 0.1, "dt": W["dt"], "ppc": list(W["ppc"]),
                   "particles_per_gpu": int(n1), "uth": W["uth"], "smoothing": "compensated level 1, x and y"},
        "cpu_baseline": {"value": v1, "unit": UNIT, "cores": 1, "kind": kind,
                         "sample": f"the whole workload ({n1} particles, {nx}x{ny} cells), one single-threaded "
                                   f"run (the reference is single-threaded), {steps1} timed steps after "
                                   f"{warm1} warm-up steps; host {platform.machine()}"},
        "host_aggregate": {"value": vp, "unit": UNIT, "cores": procs, "kind": kind_p,
                           "sample": f"{procs} concurrent single-threaded runs, each a 256x256-cell box of the "
                                     f"workload's density ({npr} particles), {args.steps} timed steps after "
                                     f"{args.warmup} warm-up steps"},
        "e2e": {"value": v1, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# batched parameter scan
# ---------------------------------------------------------------------------
def run_scan(args):
    """256 two-stream runs (grids 64..256 per axis, ppc 2..8 per axis,
    drift 0.2..0.8, thermal 0.02..0.2, dt = 0.9 Courant, 300 steps, energy
    history every step): batched against the same runs one after another
    through the plain path."""
    from zpic_gb300 import batch  # before anything creates a CUDA context

    import torch

    n_runs = args.scan_runs
    steps = args.steps if args.steps_given else 300
    runs = batch.weibel_scan(n_runs=n_runs, steps=steps)
    if not args.sort_every:
        args.sort_every = batch.scan_sort_every(steps)
    # the autotuner times half the scan's runs side by side: enough members
    # in flight that the batch's own concurrency decides
    tile, rates = batch.autotune_tile(runs, candidates=((16, 16), (32, 16), (16, 8), "by_ppc"),
                                      sample=max(1, n_runs // 2), steps=3 * 2 * args.sort_every,
                                      sort_every=args.sort_every)
    tiles = batch.tiles_for(runs, tile)
    nps = sum(r.particles() * r.steps for r in runs)

    def fresh(graphs):
        t0 = time.perf_counter()
        sims = batch.load_sims(runs, tile=tiles, sort_every=args.sort_every, graphs=graphs)
        return sims, time.perf_counter() - t0

    # warm-up: one small batch (graph capture and instantiation paths, clocks)
    warm = batch.load_sims(runs[:8], tile=tiles[:8], sort_every=args.sort_every)
    batch.run_batched(warm, [batch.ScanRun(r.nx, r.ppc, r.uz, r.uth, r.dx, r.dt, r.seed, 32) for r in runs[:8]])
    for s_ in warm:
        s_.close()

    sims, t_load = fresh(True)
    clk = ClockSampler(0)
    clk.start()
    t0 = time.perf_counter()
    res = batch.run_batched(sims, runs, group=args.scan_group or None)
    t_wall = time.perf_counter() - t0
    clocks = clk.stop()
    hist_bytes = sum(h.nbytes for h in res.histories)
    part_bytes = sum(r.particles() * 28 for r in runs)
    finals = [float(h[-1].sum()) for h in res.histories]
    for s_ in sims:
        s_.close()
    torch.cuda.empty_cache()

    sims, _ = fresh(False)
    seq = batch.run_sequential(sims, runs)
    for s_ in sims:
        s_.close()
    torch.cuda.empty_cache()
    sims, _ = fresh(True)
    seq_g = batch.run_sequential(sims, runs)
    for s_ in sims:
        s_.close()
    torch.cuda.empty_cache()
    # the same runs one by one with the plain path's default tile (16 x 16),
    # which suits a run alone better than the batch's choice
    # (the graph-replayed leg itself when the autotuner chose that tile)
    seq_d = seq_g
    if tiles != batch.tiles_for(runs, (16, 16)):
        sims = batch.load_sims(runs, tile=(16, 16), sort_every=args.sort_every, graphs=True)
        seq_d = batch.run_sequential(sims, runs)
        for s_ in sims:
            s_.close()
    line = {
        "metric": METRIC, "value": res.rate, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": 1,
        "ms_per_step": res.device_ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (reference loading, run k seeded 12345+k, 67890+k)",
        "config": {"workload": f"batched scan: {n_runs} two-stream runs, grids 64..256 per axis (dx=0.1), "
                               f"ppc 2..8 per axis, uz 0.2..0.8, uth 0.02..0.2, dt=0.9 CFL, {steps} steps, "
                               f"energy history every step",
                   "particles_total": int(sum(r.particles() for r in runs)),
                   "tile": tile if isinstance(tile, str) else list(tile),
                   "cell_sort_every": args.sort_every, "tile_slack": 2.0,
                   "batch_groups": res.groups, "fast_math": True},
        "batched": {"rate": res.rate, "device_ms": res.device_ms, "wall_s": t_wall, **res.extra},
        "sequential_plain": {"rate": seq.rate, "device_ms": seq.device_ms, "wall_s": seq.wall_s, **seq.extra,
                             "how": "each run alone through zc_step (eager launches), one after another"},
        "sequential_graphs": {"rate": seq_g.rate, "device_ms": seq_g.device_ms, "wall_s": seq_g.wall_s,
                              "how": "each run alone through zc_step with graph replay, one after another"},
        "speedup_vs_sequential": res.rate / seq.rate,
        "speedup_vs_sequential_graphs": res.rate / seq_g.rate,
        "sequential_graphs_default_tile": {
            "rate": seq_d.rate, "device_ms": seq_d.device_ms, "wall_s": seq_d.wall_s,
            "how": "each run alone through zc_step with graph replay and 16x16 tiles, one after another"},
        "speedup_vs_sequential_graphs_default_tile": res.rate / seq_d.rate,
        # against the faster of the two one-by-one legs
        "speedup_vs_best_sequential": res.rate / max(seq_g.rate, seq_d.rate),
        "autotune_rates": {(t if isinstance(t, str) else f"{t[0]}x{t[1]}"): v for t, v in rates.items()},
        "e2e": {"value": nps / (t_wall + t_load), "unit": UNIT,
                "h2d_bytes_per_step": part_bytes / steps, "d2h_bytes_per_step": hist_bytes / steps,
                "how": "host particle loading and upload of every run, batched stepping, energy histories "
                       "read back; wall clock"},
        "clocks": clocks,
        "energy_final_mean": float(np.mean(finals)),
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# moving-window laser wakefield
# ---------------------------------------------------------------------------
def run_lwfa(args):
    """2000 x 256 cells, box 40 x 51.2 (dx 0.02, dy 0.2), dt 0.014, 3000
    steps, moving window; Gaussian laser a0 2, omega0 10, W0 4, FWHM 2,
    start 17, focus 20, axis 25.6, polarisation along y (polarization 0);
    cold electrons of density 1 from x = 20, 4 x 2 ppc; binomial smoothing
    along x, level 4.  The particles are loaded as spec_new does; the column
    the window uncovers is drawn on the device as spec_move_window draws it
    for a cold species (--host-injection: from the host provider)."""
    from zpic_gb300 import em2d
    from zpic_gb300._zc import PART_DTYPE, CudaSim

    nx, box, dt = (2000, 256), (40.0, 51.2), 0.014
    steps = args.steps if args.steps_given else 3000
    ppc = (4, 2)
    em2d.set_rand_seed(12345, 67890, fresh=True)
    parts, q = em2d.load_particles(-1.0, ppc, nx, box, dt, density=em2d.Density(type="step", start=20.0))
    # the column injected at every window move: the ppc lattice of cells
    # (nx-1, j), cold (the plasma extends past the window's right edge)
    hx, hy = np.float32(1.0) / np.float32(ppc[0]), np.float32(1.0) / np.float32(ppc[1])
    col = np.zeros(nx[1] * ppc[0] * ppc[1], dtype=PART_DTYPE)
    k = 0
    for j in range(nx[1]):
        for b in range(ppc[1]):
            for a in range(ppc[0]):
                col[k] = (nx[0] - 1, j, hx * np.float32(a + 0.5), hy * np.float32(b + 0.5), 0, 0, 0)
                k += 1
    sim = CudaSim(nx, box, dt, tile=(32, 16), fast_math=not args.exact)
    sim.add_species(-1.0, q, ppc, parts)
    sim.add_laser(type="gaussian", start=17.0, fwhm=2.0, a0=2.0, omega0=10.0, W0=4.0, focus=20.0, axis=25.6,
                  polarization=0.0)
    sim.set_moving_window()
    if args.host_injection:
        sim.set_injector(lambda species, n_move: col)
    else:
        sim.set_device_injector(0, "step", start=20.0)
        sim.set_graphs(True)  # blocks keyed by their window moves and injected lattice
    sim.set_smooth("binomial", 4, "none", 0)
    n0 = sim.count(0)
    clk = ClockSampler(0)
    clk.start()
    sim.step(steps)
    ms = sim.last_ms()
    clocks = clk.stop()
    n1 = sim.count(0)
    info = sim.info()
    Ex = sim.E()[nx[1] // 2 + 1, 1:nx[0] + 1, 0]
    sim.close()
    nps = 0.5 * (n0 + n1) * steps
    line = {
        "metric": METRIC, "value": nps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": 0,
        "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (reference loading, step density)",
        "config": {"workload": "moving-window laser wakefield: 2000x256 cells, box 40x51.2, dt 0.014, 3000 steps, "
                               "Gaussian laser a0 2 omega0 10 W0 4 FWHM 2 start 17 focus 20 pol y, density 1 "
                               "from x=20, 4x2 ppc cold, binomial x smoothing level 4",
                   "particles_start": int(n0), "particles_end": int(n1), "window_moves": info["n_move"],
                   "injection": "host provider" if args.host_injection else "device",
                   "graphs": not args.host_injection, "graph_captures": info["captures"],
                   "push_build": "exact" if args.exact else "fast"},
        "how": "value = mean particle count x steps / device time of zc_step(3000) (injection included: "
               + ("host provider" if args.host_injection else "drawn on the device") + ")",
        "wake": {"on_axis_Ex_max_abs": float(np.abs(Ex).max()), "on_axis_Ex_rms": float(np.sqrt(np.mean(Ex ** 2)))},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_dropin(args):
    """The uniform thermal plasma (2048 x 2048, 4 x 4 ppc, uth 0.05,
    compensated level-1 smoothing along x and y) as a reference input deck:
    a C program compiled against the em2d drop-in headers and linked to
    libzpic_em2d (zpic_gb300/csrc/em2d/deck_thermal.c), loading its particles
    with spec_new and stepping with sim_iter, timed on the host wall clock.
    Two runs: host mirrors refreshed on demand, and host mirrors kept valid
    across every sim_iter (the reference's struct semantics)."""
    import subprocess

    from zpic_gb300 import build

    build.build()
    root = os.path.dirname(os.path.abspath(__file__))
    lib = os.path.join(root, "zpic_gb300", "lib")
    out = os.path.join(root, "zpic_gb300", "_build")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "deck_thermal")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(root, "include", "em2d"),
                    os.path.join(root, "zpic_gb300", "csrc", "em2d", "deck_thermal.c"), "-L", lib, "-lzpic_em2d",
                    "-Wl,-rpath," + lib, "-lm", "-o", exe], check=True)
    n = args.nx or 2048
    tile = tuple(int(v) for v in args.tile.split("x"))
    steps = args.steps if args.steps_given else 20
    res = {}
    for mode, k in (("demand", steps), ("every", max(2, min(steps, 6)))):
        r = subprocess.run([exe, str(k), mode, str(n), str(tile[0]), str(tile[1]), "0" if args.exact else "1"],
                           capture_output=True, text=True, timeout=1800)
        if r.returncode != 0:
            raise RuntimeError(f"deck_thermal {mode} failed: {r.stderr[-2000:]}")
        v = dict(line.split() for line in r.stdout.splitlines())
        res[mode] = {"steps": k, "setup_s": float(v["setup_s"]), "first_step_ms": float(v["first_step_ms"]),
                     "step_ms": float(v["step_ms"]), "sync_host_ms": float(v["sync_host_ms"]),
                     "particles": int(v["particles"]),
                     "kinetic": float(v["kinetic"]), "field": float(v["field"])}
    d, e = res["demand"], res["every"]
    mirror_bytes = d["particles"] * 28 + 3 * 3 * 4 * (n + 3) * (n + 3)
    line = {
        "metric": METRIC, "value": d["particles"] / (d["step_ms"] * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": steps, "warmup": 1, "ms_per_step": d["step_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (spec_new loading through the drop-in)",
        "config": {"workload": f"em2d uniform thermal plasma {n}x{n}, 4x4 ppc, uth 0.05, compensated level 1 x "
                               f"and y, dt 0.05: a C deck through the em2d drop-in (sim_iter)",
                   "tile": list(tile), "push_build": "exact" if args.exact else "fast"},
        "how": "value = particles / host wall time of one sim_iter (mirrors on demand), after the first step",
        "mirrors_on_demand": d,
        "mirrors_every_step": {**e, "rate": e["particles"] / (e["step_ms"] * 1e-3),
                               "host_mirror_bytes": mirror_bytes},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# differentiable step: gradient of the final field energy
# ---------------------------------------------------------------------------
def run_adjoint(args):
    """256 x 256 cells, dx = dy = 0.1, dt = 0.06, 200 steps, checkpoints every
    20 steps, one electron species 4 x 4 ppc (1,048,576 particles), uth 0.05,
    weights n(x) = 1 + 0.3 sum of 8 seeded sinusoids: the float32 adjoint's
    cost against its forward run and against the plain forward step, and its
    gradients (8 profile amplitudes, x drift) against float64 central
    differences (eps 1e-4) of the same engine."""
    from zpic_gb300 import adjoint
    from zpic_gb300._zc import CudaSim, PART_DTYPE

    nx, dt, steps, K = (256, 256), 0.06, (args.steps if args.steps_given else 200), 20
    st, amps, kk, q = adjoint.profile_setup(nx=nx, dx=0.1, ppc=(4, 4), uth=0.05, seed=7, drift=0.0)
    n = st["ix"].size
    box = (nx[0] * 0.1, nx[1] * 0.1)
    sim = adjoint.AdjointSim(nx, box, dt, n, q, checkpoint_every=K, precision="float32")

    def load(s, w, drift=0.0):
        s.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"] + drift, st["uy"], st["uz"], w)

    # warm-up, then timed forward + backward
    for _ in range(max(args.warmup, 1)):
        load(sim, st["w"])
        sim.forward(min(steps, 2 * K))
        sim.backward()
    clk = ClockSampler(0)
    clk.start()
    load(sim, st["w"])
    L, _ = sim.forward(steps)
    g = sim.backward()
    fwd_ms, bwd_ms = sim.times()
    clocks = clk.stop()
    ga = adjoint.amplitude_gradient(g["w"], st["X"], kk)
    gd = float(g["ux"].sum())

    # the plain step on the same particles (weights 1: it has no weights)
    parts = np.zeros(n, dtype=PART_DTYPE)
    for f in ("ix", "iy", "x", "y", "ux", "uy", "uz"):
        parts[f] = st[f]
    plain = CudaSim(nx, box, dt, tile=(16, 16), fast_math=False)
    plain.add_species(-1.0, q, (4, 4), parts)
    plain.step(5)
    plain.step(steps)
    plain_ms = plain.last_ms()
    plain.close()

    # float64: the adjoint's own gradient and central differences of the engine
    sim64 = adjoint.AdjointSim(nx, box, dt, n, q, checkpoint_every=K, precision="float64")
    load(sim64, st["w"])
    L64, _ = sim64.forward(steps)
    g64 = sim64.backward()
    f64_ms = sim64.times()
    ga64 = adjoint.amplitude_gradient(g64["w"], st["X"], kk)
    gd64 = float(g64["ux"].sum())

    def Lf(a, drift=0.0):
        load(sim64, adjoint.weights(st["X"], a, kk), drift)
        return sim64.forward(steps)[0]

    # central differences at shrinking steps: the objective is piecewise smooth
    # (kinks where trajectories cross cell edges and the staggered half-cell),
    # so a larger step averages slopes across the kinks it straddles
    fds = {}
    for eps in (1e-4, 1e-5, 1e-6):
        fa = np.array([(Lf(amps + eps * e) - Lf(amps - eps * e)) / (2 * eps) for e in np.eye(len(amps))])
        fds[eps] = (fa, (Lf(amps, eps) - Lf(amps, -eps)) / (2 * eps))
    # the float64 objective's own run-to-run noise (its deposit sums in the
    # order the atomics land): the same inputs three times; a central
    # difference at step eps carries up to noise / eps of it
    reps = [Lf(amps) for _ in range(3)]
    noise = float(max(reps) - min(reps))
    # the drift's differences at still smaller steps
    fd_drift_small = {f"{e:g}": (Lf(amps, e) - Lf(amps, -e)) / (2 * e) for e in (1e-7, 1e-8)}
    # the stated steps: 1e-6 for the amplitudes; 1e-8 for the drift, whose
    # difference quotient straddles the objective's kinks (every particle's
    # trajectory moves) down to 1e-7
    eps, eps_d = 1e-6, 1e-8
    fd = fds[eps][0]
    fdd = fd_drift_small[f"{eps_d:g}"]
    rel_a = float(np.linalg.norm(ga - fd) / np.linalg.norm(fd))
    rel_d = float(abs(gd - fdd) / abs(fdd))
    rel_a64 = float(np.linalg.norm(ga64 - fd) / np.linalg.norm(fd))
    rel_d64 = float(abs(gd64 - fdd) / abs(fdd))
    # why float32 stops near 1e-3: the per-particle gradients of the float32
    # engine carry a small relative error, and the projections onto the
    # drift and the 8 amplitudes cancel them many-fold
    S = np.sin(np.outer(st["X"], kk))
    rho_w = float(np.linalg.norm(g["w"] - g64["w"]) / np.linalg.norm(g64["w"]))
    rho_ux = float(np.linalg.norm(g["ux"] - g64["ux"]) / np.linalg.norm(g64["ux"]))
    canc_d = float(np.abs(g64["ux"]).sum() / abs(np.sum(g64["ux"])))
    canc_a = (np.abs(g64["w"])[:, None] * np.abs(S)).sum(0) / np.abs(g64["w"] @ S)
    fd_steps = {f"{e:g}": {"amplitudes_rel_err_adjoint64": float(np.linalg.norm(ga64 - v[0]) / np.linalg.norm(v[0])),
                           "drift_rel_err_adjoint64": float(abs(gd64 - v[1]) / abs(v[1])),
                           "fd_drift": v[1],
                           "drift_fd_noise_rel": noise / e / abs(v[1]),
                           "amplitudes_fd_noise_rel": noise / e / float(np.linalg.norm(v[0]))}
                for e, v in fds.items()}
    sim.close()
    sim64.close()
    grad_ms = fwd_ms + bwd_ms
    line = {
        "metric": METRIC, "value": n * steps / (grad_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": grad_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lattice, thermal momenta, profile weights)",
        "config": {"workload": "adjoint: 256x256 cells, dx=dy=0.1, dt=0.06, 200 steps, checkpoint every 20, "
                               "4x4 ppc (1,048,576 particles), uth 0.05, weights 1+0.3*sum of 8 sinusoids, "
                               "objective = total field energy at the last step",
                   "checkpoint_every": K, "particles": n},
        "how": "value = particle-steps of the forward run / (forward + backward device time)",
        "adjoint": {"forward_ms": fwd_ms, "backward_ms": bwd_ms,
                    "gradient_over_forward": grad_ms / fwd_ms,
                    "gradient_over_plain_forward": grad_ms / plain_ms, "plain_forward_ms": plain_ms,
                    "objective": L},
        "gradient_check": {"float64_adjoint": {"amplitudes_rel_err_vs_fd64": rel_a64,
                                               "drift_rel_err_vs_fd64": rel_d64,
                                               "forward_ms": f64_ms[0], "backward_ms": f64_ms[1],
                                               "gradient_over_forward": (f64_ms[0] + f64_ms[1]) / f64_ms[0]},
                           "float32_adjoint": {"amplitudes_rel_err_vs_fd64": rel_a, "drift_rel_err_vs_fd64": rel_d},
                           "float32_vs_float64": {
                               "objective_rel": float(abs(L - L64) / abs(L64)),
                               "amplitudes_rel_l2": float(np.linalg.norm(ga - ga64) / np.linalg.norm(ga64)),
                               "drift_rel": float(abs(gd - gd64) / abs(gd64)),
                               "per_particle_dw_rel_l2": rho_w, "per_particle_dux_rel_l2": rho_ux,
                               "drift_cancellation": canc_d,
                               "amplitude_cancellation": canc_a.tolist()},
                           "eps": eps, "eps_drift": eps_d, "fd_by_step": fd_steps, "objective64_noise": noise,
                           "fd_drift_small_steps": {k: {"fd": v, "rel_err_adjoint64": float(abs(gd64 - v) / abs(v))}
                                                    for k, v in fd_drift_small.items()},
                           "objective64": reps[0], "fd_amplitudes": fd.tolist(), "adjoint64_amplitudes": ga64.tolist(),
                           "adjoint32_amplitudes": ga.tolist(), "fd_drift": fdd, "adjoint64_drift": gd64,
                           "adjoint32_drift": gd},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def wakefield_fd_study(W, make, load, steps):
    """Central differences of the float64 engine at shrinking steps, for a0
    and ramp knot 3, with the wake-region objective and with the whole axis,
    beside the float64 adjoint of each."""
    from zpic_gb300 import adjoint

    out = {}
    for label, cells in (("wake_cells_200_899", (200, 900)), ("whole_axis", (0, 0))):
        s_ = make("float64", cells)
        kn = W["knots_n"]

        def Lf(scale, knots):
            load(s_, scale, knots)
            return s_.forward(steps)[0]

        Lf(1.0, kn)
        g = s_.backward()
        r = {"adjoint_a0": float((g["E"] * W["E"]).sum() + (g["B"] * W["B"]).sum()) / W["a0"],
             "adjoint_knot3": float(adjoint.ramp_gradient(g["w"], W["X"], W["knots_x"])[3])}
        for eps in (1e-5, 1e-6, 1e-7, 1e-8):
            e = np.zeros_like(kn)
            e[3] = eps
            r[f"fd_a0_eps{eps:g}"] = (Lf(1 + eps, kn) - Lf(1 - eps, kn)) / (2 * eps * W["a0"])
            r[f"fd_knot3_eps{eps:g}"] = (Lf(1.0, kn + e) - Lf(1.0, kn - e)) / (2 * eps)
        out[label] = r
        s_.close()
    print(json.dumps({"workload": "wakefield adjoint, finite-difference step study (float64)", **out}), flush=True)
    return 0


def run_wakefield_adjoint(args):
    """The moving-window laser wakefield (2000 x 256, 3000 steps) through
    the adjoint engine: gradient of the final on-axis Ex wake (dx sum Ex^2
    along the axis row over cells 200..899: the wake behind the laser, away
    from the absorbing left edge where leaving particles make the objective
    discontinuous) with respect to the laser amplitude a0 and the 16 knots
    of a piecewise-linear density ramp, checkpoints every 100 steps,
    float32; checked against float64 central differences of the same engine
    for a0 and three knots."""
    from zpic_gb300 import adjoint

    nx, box, dt = (2000, 256), (40.0, 51.2), 0.014
    steps = args.steps if args.steps_given else 3000
    K = 100
    W = adjoint.wakefield_setup(nx=nx, box=box, dt=dt, nsteps=steps, smooth=("binomial", 4))
    st, X, kx, kn = W["state"], W["X"], W["knots_x"], W["knots_n"]
    n = st["ix"].size
    row = nx[1] // 2

    def make(prec, cells=(200, 900)):
        s_ = adjoint.AdjointSim(nx, box, dt, n, W["q"], checkpoint_every=K, precision=prec, moving_window=True,
                                objective="axis_ex", objective_row=row, objective_cells=cells)
        s_.set_birth(W["birth"])
        s_.set_smooth(W["passes"])
        return s_

    def load(s_, scale, knots):
        w = adjoint.ramp_density(X, kx, knots)
        s_.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], w, scale * W["E"],
                     scale * W["B"])

    if args.fd_study:
        return wakefield_fd_study(W, make, load, steps)
    sim = make("float32")
    clk = ClockSampler(0)
    clk.start()
    load(sim, 1.0, kn)
    L, _ = sim.forward(steps)
    alive = sim.state()["alive"]
    g = sim.backward()
    fwd_ms, bwd_ms = sim.times()
    clocks = clk.stop()
    a0 = W["a0"]
    ga0 = float((g["E"] * W["E"]).sum() + (g["B"] * W["B"]).sum()) / a0
    gk = adjoint.ramp_gradient(g["w"], X, kx)
    sim.close()
    sim64 = make("float64")
    load(sim64, 1.0, kn)
    L64, _ = sim64.forward(steps)
    g64 = sim64.backward()
    f64_ms = sim64.times()
    ga0_64 = float((g64["E"] * W["E"]).sum() + (g64["B"] * W["B"]).sum()) / a0
    gk64 = adjoint.ramp_gradient(g64["w"], X, kx)

    def Lf(scale, knots):
        load(sim64, scale, knots)
        return sim64.forward(steps)[0]

    eps = 1e-7
    fd_a0 = (Lf(1 + eps, kn) - Lf(1 - eps, kn)) / (2 * eps * a0)
    fd_k = {}
    for k in (2, 5, 8):
        e = np.zeros_like(kn)
        e[k] = eps
        fd_k[k] = (Lf(1.0, kn + e) - Lf(1.0, kn - e)) / (2 * eps)
    sim64.close()
    rel = lambda a, b: float(abs(a - b) / max(abs(b), 1e-300))
    ks = sorted(fd_k)

    def l2(g_):
        # the checked knots' gradient as one vector against the differences
        d = np.array([g_[k] - fd_k[k] for k in ks])
        return float(np.linalg.norm(d) / np.linalg.norm([fd_k[k] for k in ks]))
    nps = sum(int(((W["birth"] <= s_) ).sum()) for s_ in range(0, steps, max(steps // 30, 1))) * max(steps // 30, 1)
    line = {
        "metric": METRIC, "value": nps / ((fwd_ms + bwd_ms) * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": 0, "ms_per_step": (fwd_ms + bwd_ms) / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (reference loading, step density, host-planned injection)",
        "config": {"workload": "adjoint of the moving-window laser wakefield: 2000x256 cells, box 40x51.2, dt 0.014, "
                               "3000 steps, laser a0 2 omega0 10 W0 4 FWHM 2 start 17 focus 20 pol y, step density "
                               "from x=20 times a 16-knot ramp, 4x2 ppc cold, binomial x smoothing level 4, "
                               "checkpoints every 100 steps; objective dx sum Ex^2 on the axis row",
                   "particle_pool": n, "initial_particles": W["n_initial"], "window_moves": len(W["moves"]),
                   "particles_at_end": int(((alive == 1) & (W["birth"] <= steps)).sum()),
                   "objective": "dx sum Ex^2, axis row, cells 200..899"},
        "how": "value = particle-steps (particles present, sampled every 100 steps) / (forward + backward device time)",
        "adjoint": {"forward_ms": fwd_ms, "backward_ms": bwd_ms, "gradient_over_forward": (fwd_ms + bwd_ms) / fwd_ms,
                    "objective": L, "dL_da0": ga0, "dL_dknots": gk.tolist()},
        "gradient_check": {"eps": eps,
                           "float64_adjoint": {"forward_ms": f64_ms[0], "backward_ms": f64_ms[1],
                                               "dL_da0_rel_err_vs_fd64": rel(ga0_64, fd_a0),
                                               "knots_rel_err_vs_fd64": {str(k): rel(gk64[k], v)
                                                                         for k, v in fd_k.items()},
                                               "knots_rel_l2_vs_fd64": l2(gk64)},
                           "float32_adjoint": {"dL_da0_rel_err_vs_fd64": rel(ga0, fd_a0),
                                               "knots_rel_err_vs_fd64": {str(k): rel(gk[k], v)
                                                                         for k, v in fd_k.items()},
                                               "knots_rel_l2_vs_fd64": l2(gk)},
                           "fd_da0": fd_a0, "fd_knots": {str(k): v for k, v in fd_k.items()},
                           # how far float32 arithmetic alone moves the run: the objective and the
                           # whole gradient of the float32 engine against the float64 engine's
                           "float32_vs_float64": {
                               "objective_rel": rel(L, L64),
                               "dL_da0_rel": rel(ga0, ga0_64),
                               "knots_rel_l2": float(np.linalg.norm(gk - gk64) / np.linalg.norm(gk64)),
                               "knots_rel": [rel(a, b) for a, b in zip(gk, gk64)]}},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# the em1d step: the reference's own 1-D laser wakefield deck
# ---------------------------------------------------------------------------
# em1d/input/lwfa.c: 1000 cells, box 20, dt 0.019, tmax 22.8; electrons
# (m_q -1) of density 1 from x = 20, 128 ppc, cold; laser start 17, FWHM 2,
# a0 2, omega0 10, polarisation pi/2; moving window; compensated level-4
# smoothing.  All plasma enters through the window's right edge.
EM1D = dict(nx=1000, box=20.0, dt=0.019, tmax=22.8, ppc=128, m_q=-1.0, density=("step", 20.0, 0.0),
            laser=dict(start=17.0, fwhm=2.0, a0=2.0, omega0=10.0, polarization=float(np.pi / 2)),
            smooth=("compensated", 4))
# algorithmic bytes of the push per particle: the 20-byte record read and
# written (fields and current stay in L1/L2: 1000 cells)
EM1D_PART_BYTES = 40


def em1d_steps(dt, tmax):
    """iterations of the reference's main loop, for (n=0,t=0; t<=tmax; n++,
    t=n*dt) in float (em1d/main.c:55)"""
    n = 0
    while np.float32(n) * np.float32(dt) <= np.float32(tmax):
        n += 1
    return n


def em1d_deck():
    """the deck as a dict for the CPU checker (oracle/pyoracle_em1d)"""
    W = EM1D
    return dict(nx=W["nx"], box=W["box"], dt=W["dt"],
                species=[dict(name="electrons", m_q=W["m_q"], ppc=W["ppc"],
                              density=dict(type="step", start=W["density"][1]))],
                laser=W["laser"], moving_window=True, smooth=dict(type=W["smooth"][0], level=W["smooth"][1]))


def _em1d_sim():
    from zpic_gb300.em1d_gpu import PART_DTYPE, CudaSim1D

    W = EM1D
    sim = CudaSim1D(W["nx"], W["box"], W["dt"], moving_window=True)
    q = float(np.float32(np.copysign(1.0, W["m_q"]) / W["ppc"]))  # spec_new, em1d/particles.c:529
    sim.add_species(W["m_q"], q, W["ppc"], np.zeros(0, dtype=PART_DTYPE), density=W["density"])
    L = W["laser"]
    sim.add_laser(L["start"], L["a0"], L["omega0"], fwhm=L["fwhm"], polarization=L["polarization"])
    sim.set_smooth(*W["smooth"])
    return sim


def em1d_cpu(steps, fast=True):
    """the deck on one host core: the reference em1d (stock -Ofast build)
    where it is built, else the C restatement; returns (particle-steps/s,
    kind, seconds, particle-steps)"""
    from oracle import pyoracle, pyoracle_em1d

    pyoracle.build()
    backend = "ref" if pyoracle_em1d.available("ref", fast) else "oracle"
    s = pyoracle_em1d.RefSim1D(em1d_deck(), stock_sort=True, backend=backend, fast=fast)
    pushed = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        pushed += s.np_(0)
        s.iter()
    t = time.perf_counter() - t0
    s.close()
    return pushed / t, ("reference" if backend == "ref" else "port"), t, pushed


def run_em1d(args):
    """The em1d step on the reference's 1-D wakefield deck (em1d/input/lwfa.c),
    the whole run of 1201 steps.  A profiled pass gives each kernel's device
    time; the timed pass is one zc1_step call of the whole run (CUDA events on
    the simulation's stream), its particle-steps the device's count of the
    particles pushed; e2e is the same run through the public API on the wall
    clock, from creating the simulation to reading E and B back."""
    W = EM1D
    steps = args.steps if args.steps_given else em1d_steps(W["dt"], W["tmax"])
    # profiled pass: per-kernel device times (event-record nodes around
    # every kernel of the step graphs)
    sim = _em1d_sim()
    sim.set_profile(True)
    sim.step(steps)
    prof = sim.profile()
    sim.close()
    # warm-up runs of the timed pass, then the timed pass
    for _ in range(max(args.warmup, 3)):
        sim = _em1d_sim()
        sim.step(min(steps, 100))
        sim.close()
    sim = _em1d_sim()
    clk = ClockSampler(0)
    clk.start()
    sim.step(steps)
    ms = sim.last_ms()
    clocks = clk.stop()
    launches = sim.launches()
    info = sim.info()
    n_end = sim.count(0)
    pushed = sim.pushed(0)
    sim.close()
    # e2e: public API, wall clock, fields back on the host
    t0 = time.perf_counter()
    sim = _em1d_sim()
    sim.step(steps)
    E, B = sim.E(), sim.B()
    t_e2e = time.perf_counter() - t0
    sim.close()
    value = pushed / (ms * 1e-3)
    # roofline of the dominant kernel
    dom = max(prof, key=lambda k: prof[k][0])
    hbm, peak_kind = peaks()
    push_ms, push_n = push_prof
    push_bytes = EM1D_PART_BYTES * pushed / max(push_n, 1)
    achieved = push_bytes / (push_ms * 1e-3 / max(push_n, 1)) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3),
        "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the reference deck's cold plasma, injected by the moving window)",
        "config": {"workload": "em1d laser wakefield (em1d/input/lwfa.c): 1000 cells, box 20, dt 0.019, "
                               f"{steps} steps (tmax 22.8), moving window, laser a0 2 omega0 10 FWHM 2 start 17 "
                               "pol pi/2, density 1 from x=20, 128 ppc cold, compensated smoothing level 4",
                   "particles_end": int(n_end), "particle_steps": int(pushed), "window_moves": info["n_move"],
                   "l2": "working set L2-resident (under 6 MB); no flush"},
        "how": "value = particles pushed summed over the steps / device time of one zc1_step call of the whole run "
               "(blocks of 16 steps replayed as CUDA graphs)",
        "e2e": {"value": pushed / t_e2e, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": (E.nbytes + B.nbytes) / steps,
                "how": "wall clock of create + laser + zc1_step(all) + E/B read; the deck's plasma is injected "
                       "on the device, so nothing is uploaded"},
        "gpu_launches": launches,
        "kernels": {k: {"ms": v[0], "launches": v[1], "share": v[0] / max(sum(x[0] for x in prof.values()), 1e-30)}
                    for k, v in prof.items()},
        "roofline": {"bound": "hbm", "kernel": "k1_push", "dominant_kernel_kind": dom, "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                     "peak_source": peak_kind,
                     "note": "40 B per particle read and written; a push moves at most 6 MB, L2-resident, so "
                             "latency (launch, last-CTA bookkeeping), not HBM, bounds it"},
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        v, kind, t, n = em1d_cpu(steps)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": f"the whole deck ({steps} steps, {n} particle-steps, {t:.2f} s), "
                                          "stock sort every 16 steps"}
    print(json.dumps(line), flush=True)
    return 0


def run_em1d_scan(args):
    """A parameter scan of the em1d wakefield deck (mods/em1d_param_scan: the
    laser FWHM spread evenly over [1.5, 2.5] across the runs, the rest as
    em1d/input/lwfa.c, full 1201 steps).  The runs go once one after another
    (each zc1_step to completion) and once side by side (every run on its
    own stream, blocks of 16 steps enqueued round-robin, one wait per run at
    the end).  Both are timed on the wall clock; particle-steps are the
    device's counts of the particles pushed."""
    W = EM1D
    n_runs = args.scan_runs if args.scan_runs_given else 64
    steps = args.steps if args.steps_given else em1d_steps(W["dt"], W["tmax"])
    fwhm = [1.5 + k * (1.0 / max(n_runs - 1, 1)) for k in range(n_runs)]

    def make(k, ctas=0):
        from zpic_gb300.em1d_gpu import PART_DTYPE, CudaSim1D

        sim = CudaSim1D(W["nx"], W["box"], W["dt"], moving_window=True, push_ctas=ctas)
        q = float(np.float32(np.copysign(1.0, W["m_q"]) / W["ppc"]))
        sim.add_species(W["m_q"], q, W["ppc"], np.zeros(0, dtype=PART_DTYPE), density=W["density"])
        L = W["laser"]
        sim.add_laser(L["start"], L["a0"], L["omega0"], fwhm=fwhm[k], polarization=L["polarization"])
        sim.set_smooth(*W["smooth"])
        return sim

    # warm-up: both launch modes once on a short run
    for _ in range(max(args.warmup, 3)):
        w = [make(k) for k in range(2)]
        for s in w:
            s.step(32, wait=False)
        for s in w:
            s.synchronize()
            s.close()
    # one after another
    sims = [make(k) for k in range(n_runs)]
    t0 = time.perf_counter()
    for s in sims:
        s.step(steps)
    t_seq = time.perf_counter() - t0
    ps_seq = sum(s.pushed(0) for s in sims)
    for s in sims:
        s.close()
    # side by side, for a few caps of the push's CTAs per run
    sweep = {}
    best = None
    for ctas in (0, 128, 64, 32):
        sims = [make(k, ctas) for k in range(n_runs)]
        clk = ClockSampler(0)
        clk.start()
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            blk = min(16, steps - done)
            for s in sims:
                s.step(blk, wait=False)
            done += blk
        for s in sims:
            s.synchronize()
        t_par = time.perf_counter() - t0
        clocks = clk.stop()
        ps_par = sum(s.pushed(0) for s in sims)
        launches = sum(s.launches() for s in sims)
        moves = [s.info()["n_move"] for s in sims]
        for s in sims:
            s.close()
        sweep[str(ctas)] = ps_par / t_par
        if best is None or ps_par / t_par > best[0]:
            best = (ps_par / t_par, ctas, t_par, ps_par, clocks, launches, moves)
    _, best_ctas, t_par, ps_par, clocks, launches, moves = best
    line = {
        "metric": METRIC, "value": ps_par / t_par, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * t_par / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (the reference deck's cold plasma, injected by the moving window)",
        "config": {"workload": f"em1d parameter scan: {n_runs} runs of the em1d wakefield deck (em1d/input/lwfa.c, "
                               f"{steps} steps each), laser FWHM 1.5..2.5 across the runs "
                               "(mods/em1d_param_scan/input/lwfa.c)",
                   "runs": n_runs, "particle_steps": int(ps_par), "window_moves": moves[0],
                   "push_ctas_per_run": best_ctas,
                   "l2": "working set L2-resident; no flush"},
        "how": "value = particle-steps of all runs / wall clock of the side-by-side pass (one stream per run, "
               "16-step graph blocks enqueued round-robin)",
        "sequential": {"value": ps_seq / t_seq, "seconds": t_seq,
                       "how": "the same runs one after another, each zc1_step(all) to completion"},
        "speedup_over_sequential": (ps_par / t_par) / (ps_seq / t_seq),
        "push_ctas_sweep": sweep,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        v, kind, t, n = em1d_cpu(steps)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": f"one run of the deck ({steps} steps, {n} particle-steps, {t:.2f} s)"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--tile", default="32x16")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-exact-line", action="store_true", help="skip the exact push build's figure")
    ap.add_argument("--exact", action="store_true",
                    help="bit-exact push build (every float32 op rounded as the reference C)")
    ap.add_argument("--sort-every", type=int, default=0)
    ap.add_argument("--nx", type=int, default=0, help="square grid override (profiling runs)")
    ap.add_argument("--workload", default="plain", choices=["plain", "scan", "adjoint", "lwfa", "wakefield_adjoint",
                                                              "em1d", "em1d_scan", "dropin"])
    ap.add_argument("--deterministic", action="store_true", help="fixed-point (bit-reproducible) deposition")
    ap.add_argument("--fd-study", action="store_true", help="wakefield adjoint: finite differences at shrinking steps")
    ap.add_argument("--scan-runs", type=int, default=256)
    ap.add_argument("--scan-group", type=int, default=0, help="runs per batch graph (0: all)")
    ap.add_argument("--host-injection", action="store_true",
                    help="lwfa: the window's new column from the host provider instead of the device")
    args = ap.parse_args()
    args.steps_given = any(a.startswith("--steps") for a in sys.argv[1:])
    args.scan_runs_given = any(a.startswith("--scan-runs") for a in sys.argv[1:])
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "scan":
        return run_scan(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "lwfa":
        return run_lwfa(args)
    if args.workload == "wakefield_adjoint":
        return run_wakefield_adjoint(args)
    if args.workload == "em1d":
        return run_em1d(args)
    if args.workload == "em1d_scan":
        return run_em1d_scan(args)
    if args.workload == "dropin":
        return run_dropin(args)

    from zpic_gb300.replicas import Replicas

    rep = Replicas()  # torchrun: one independent replica per GPU, no data-path collective
    rank, world, local = rep.rank, rep.world, rep.local
    barrier, allmax = rep.barrier, rep.allmax

    from zpic_gb300._zc import CudaSim

    W = dict(WORKLOAD)
    if args.nx:
        W.update(nx=(args.nx, args.nx), box=(args.nx * 0.1, args.nx * 0.1),
                 name=f"em2d uniform thermal plasma {args.nx}x{args.nx}, 4x4 ppc")
    nx, ny = W["nx"]
    tile = tuple(int(v) for v in args.tile.split("x"))
    parts = synth_particles(nx, ny, W["ppc"], W["uth"], seed=1234 + rank)
    N = parts.size
    q = np.float32(-1.0) / np.float32(W["ppc"][0] * W["ppc"][1])
    sim = CudaSim(W["nx"], W["box"], W["dt"], device=local, tile=tile, fast_math=not args.exact,
                  sort_every=args.sort_every, deterministic=args.deterministic)
    sim.add_species(W["m_q"], float(q), W["ppc"], parts)
    sm = W["smooth"]
    sim.set_smooth(sm[0], sm[1], sm[2], sm[3])
    # blocks of 2 x sort_every steps replay as CUDA graphs (the steps before
    # the first block boundary and after the last run eagerly)
    sim.set_graphs(True)

    # ---- device-resident timed region: CUDA events around the whole run
    # (zc_step) and around every push launch (the roofline's kernel: event
    # launches in the eager steps, event-record nodes in the graphs) ----
    sim.step(args.warmup)
    sim.set_profiling("push")
    sim.reset_profile()
    clk = ClockSampler(local)
    barrier()
    sim.synchronize()
    clk.start()
    sim.step(args.steps)  # returns after the stream has drained
    ms = sim.last_ms()
    clocks = clk.stop()
    barrier()
    ms = allmax(ms)
    timed_prof = sim.profile()  # launch counts of every phase; device time of the push
    push_prof = timed_prof["push"]
    value = N * args.steps * world / (ms / 1e3)
    # the per-phase breakdown: more steps with every phase bracketed by
    # events (untimed; the events add a little to each step)
    sim.set_profiling(True)
    sim.reset_profile()
    nph = max(16, min(args.steps, 64))
    sim.step(nph)
    prof = sim.profile()
    sim.set_profiling(False)

    # ---- end to end through the C-ABI with host buffers ----
    import torch

    if args.no_e2e:
        args_steps_e2e = 0
    else:
        args_steps_e2e = args.steps

    pinned = torch.empty(parts.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(parts.dtype)
    pinned[:] = parts
    fshape = (ny + 3, nx + 3, 3)
    Eh = torch.zeros(int(np.prod(fshape)), dtype=torch.float32, pin_memory=True).numpy().reshape(fshape)
    Bh = torch.zeros(int(np.prod(fshape)), dtype=torch.float32, pin_memory=True).numpy().reshape(fshape)
    # every step's energies land in page-locked host rows: 6 field
    # components and the kinetic energy of the species
    ehist = torch.zeros((max(args_steps_e2e, 1), 7), dtype=torch.float64, pin_memory=True).numpy()

    def end_to_end(queued):
        """Uploads fields and particles from the pinned host buffers, then
        runs the steps with every step's energies reaching host memory:
        queued (the steps queued with zc_step_async, 16-step blocks replayed
        as graphs, every step writing its energy row straight into the
        pinned rows: zc_history_stream; one wait at the end) or waiting
        (zc_step(1) + zc_energy, a wait per step)."""
        if queued:
            sim.history_stream(ehist[:args_steps_e2e])
        barrier()
        sim.synchronize()
        t0 = time.perf_counter()
        sim.set_fields(E=Eh, B=Bh)
        t_f = time.perf_counter()
        sim.set_particles(0, pinned)
        t_p = time.perf_counter()
        if queued:
            sim.step_async(args_steps_e2e)
        else:
            for i in range(args_steps_e2e):
                sim.step(1)
                emf, kin = sim.energy()
                ehist[i, :6], ehist[i, 6] = emf, kin[0]
        sim.synchronize()
        t = time.perf_counter() - t0
        if queued:
            assert len(sim.history()) == args_steps_e2e, "an energy row for every step"
            sim.history_stream(None)
        parts = {"fields_upload_s": t_f - t0, "particles_upload_s": t_p - t_f, "steps_with_readback_s": t0 + t - t_p}
        barrier()
        return allmax(t), parts

    e2e = e2e_wait = None
    e2e_parts = e2e_wait_parts = {}
    if args_steps_e2e:
        # untimed first pass: the device's first reads of the page-locked
        # buffers pay one-time mapping costs (up to 6 ms more on the upload)
        saved, args_steps_e2e = args_steps_e2e, 1
        end_to_end(queued=True)
        args_steps_e2e = saved
        t_e2e, e2e_parts = end_to_end(queued=True)
        e2e = N * args_steps_e2e * world / t_e2e
        t_wait, e2e_wait_parts = end_to_end(queued=False)
        e2e_wait = N * args_steps_e2e * world / t_wait
    h2d = (parts.nbytes + Eh.nbytes + Bh.nbytes) / args.steps
    d2h = (6 + 1) * 8

    # ---- roofline of the dominant kernel (push + deposit) ----
    push_ms, push_n = push_prof
    push_avg = push_ms / max(push_n, 1)
    cells = nx * ny
    push_bytes = N * PART_BYTES + cells * PUSH_CELL_BYTES
    peak, peak_kind = peaks()
    achieved = push_bytes / (push_avg / 1e3) / 1e9
    traffic = ncu_traffic()
    step_bytes = N * PART_BYTES + cells * (STEP_CELL_BYTES + 4 * SMOOTH_PASS_BYTES)
    launches = sum(n for _, n in timed_prof.values())

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded reference-style loading)",
        "config": {"workload": W["name"], "nx": [nx, ny], "dx": 0.1, "dt": W["dt"], "ppc": list(W["ppc"]),
                   "particles_per_gpu": int(N), "uth": W["uth"],
                   "smoothing": "compensated level 1, x and y", "tile": list(tile),
                   "push_build": "exact (no FMA contraction)" if args.exact else "fast (FMA contraction)",
                   "deposition": "64-bit fixed point (bit-reproducible)" if args.deterministic else "float32",
                   "cell_sort_every": args.sort_every or 8,
                   "launch": "CUDA graphs of 16-step blocks, the steps outside whole blocks eager",
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (1.88 GB of particles read and written per step)"},
        "clocks": clocks,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "how": "fields and particles uploaded from pinned host buffers through the C-ABI, then "
                       "zc_step_async over the steps (graph replay of 16-step blocks) with every step writing "
                       "its energy row into pinned host memory (zc_history_stream), one wait at the end",
                **e2e_parts,
                "waiting_each_step": {"value": e2e_wait, "how": "the same with zc_step(1) + zc_energy, "
                                      "a host wait per step", **e2e_wait_parts}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_push_tiles", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": push_bytes,
                     "avg_launch_ms": push_avg,
                     "step_achieved_gbs": step_bytes / (ms / args.steps / 1e3) / 1e9},
        "phases_ms_per_step": {k: round(v[0] / nph, 5) for k, v in prof.items() if v[1] or v[0]},
        "phases_how": f"{nph} more steps after the timed ones, every phase bracketed by CUDA events",
    }
    # ---- the exact push build on the same workload and timed region,
    # beside the fast build's headline ----
    sim.close()
    if not args.exact and not args.deterministic and not args.no_exact_line:
        ex = CudaSim(W["nx"], W["box"], W["dt"], device=local, tile=tile, fast_math=False,
                     sort_every=args.sort_every)
        ex.add_species(W["m_q"], float(q), W["ppc"], parts)
        ex.set_smooth(sm[0], sm[1], sm[2], sm[3])
        ex.set_graphs(True)
        ex.step(args.warmup)
        barrier()
        ex.synchronize()
        ex.step(args.steps)
        ms_x = allmax(ex.last_ms())
        ex.close()
        line["exact_build"] = {"value": N * args.steps * world / (ms_x / 1e3), "unit": UNIT,
                               "ms_per_step": ms_x / args.steps,
                               "parity": "every field component within 1e-5 of the oracle (IEEE float32 "
                                         "operations as the reference)"}
        line["config"]["parity"] = ("fast push build: every field within 1e-5 relative L2 of the oracle over "
                                    "10 steps, and every component on a 256x256 box of this workload "
                                    "(tests/test_gpu_configs.py)")
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, kind, n = cpu_run(512, 512, 3, 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": kind,
                                "sample": f"512x512-cell sub-box of the workload ({n} particles), 3 timed "
                                          f"steps, single-threaded C, host {platform.machine()}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    rep.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
