"""Batched parameter scans: many independent em2d runs sharing one GPU.

The reference scans parameters by running one process per point of the scan
(mods/em1d_param_scan/main.c:112-133).  Here every run is a ``CudaSim`` with
its own device state, and a ``CudaBatch`` advances many of them with one
CUDA graph per group of runs and block of steps, whose branches are the
runs: small grids that cannot fill the GPU alone share it, and one graph
launch replaces the hundreds of kernel launches of a block.  The groups run
on their own streams, so the first group starts while the next one's graph
is still being recorded.  Each run records its energy history
(field energy per component and kinetic energy per species, every step) on
the device.

Particles are loaded on the host exactly as spec_new does
(em2d/particles.c:535-612), run k from the seeds (12345 + k, 67890 + k) of a
freshly started process, so every run starts as it would alone; runs are
loaded by a pool of host threads (the generator is per thread).
"""
from __future__ import annotations

import math
import os
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

# The branches of a batch graph run concurrently on the GPU's hardware work
# queues; CUDA opens 8 of them per process by default, too few for hundreds
# of small runs.  This takes effect only if no CUDA context exists yet, and
# leaves a value the caller set alone.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import em2d  # noqa: E402
from ._zc import CudaBatch, CudaSim  # noqa: E402

TILES = ((16, 16), (32, 16), (16, 8), (8, 8), (32, 32), (16, 32), (8, 16))


@dataclass
class ScanRun:
    """One point of a scan: a two-stream (Weibel) plasma of two electron
    species drifting along z in opposite directions with a thermal spread."""
    nx: tuple
    ppc: tuple
    uz: float
    uth: float
    dx: float
    dt: float
    seed: tuple
    steps: int

    @property
    def box(self):
        return (self.nx[0] * self.dx, self.nx[1] * self.dx)

    def particles(self) -> int:
        return 2 * self.nx[0] * self.nx[1] * self.ppc[0] * self.ppc[1]


def weibel_scan(n_runs=256, steps=300, dx=0.1, seed=2024, nx_range=(64, 256), ppc_range=(2, 8),
                uz_range=(0.2, 0.8), uth_range=(0.02, 0.2), courant_frac=0.9):
    """Seeded table of scan points: nx, ny ~ U{64..256}, ppc per axis
    ~ U{2..8}, drift uz ~ U[0.2, 0.8] (+uz and -uz for the two species),
    thermal spread uth ~ U[0.02, 0.2], dt = 0.9 of the Courant limit
    (em2d/simulation.c:105-110)."""
    rng = np.random.default_rng(seed)
    runs = []
    for k in range(n_runs):
        nx = tuple(int(v) for v in rng.integers(nx_range[0], nx_range[1] + 1, size=2))
        ppc = tuple(int(v) for v in rng.integers(ppc_range[0], ppc_range[1] + 1, size=2))
        uz = float(rng.uniform(*uz_range))
        uth = float(rng.uniform(*uth_range))
        d = np.float32(dx)
        cour = math.sqrt(1.0 / (1.0 / (d * d) + 1.0 / (d * d)))
        runs.append(ScanRun(nx, ppc, uz, uth, float(d), float(np.float32(courant_frac * cour)),
                            (12345 + k, 67890 + k), steps))
    return runs


def load_run(run: ScanRun):
    """[(m_q, q, ppc, particles)] of the two species of a run."""
    em2d.set_rand_seed(*run.seed, fresh=True)
    out = []
    for sgn in (1.0, -1.0):
        parts, q = em2d.load_particles(-1.0, run.ppc, run.nx, run.box, run.dt, ufl=(0.0, 0.0, sgn * run.uz),
                                       uth=(run.uth, run.uth, run.uth))
        out.append((-1.0, q, run.ppc, parts))
    return out


def make_sim(run: ScanRun, species, tile=(32, 16), fast_math=True, sort_every=0, history=True, graphs=True,
             device=0, tile_slack=2.0) -> CudaSim:
    """The run's simulation.  Tiles get room for three times their initial
    particles (``tile_slack``): filaments of the two-stream instability
    gather particles, and between two cell sorts a tile also holds the holes
    its leavers left beside the particles that arrived; a tile that overflows
    sends particles to the slower spill path until the next re-layout."""
    sim = CudaSim(run.nx, run.box, run.dt, device=device, tile=tile, fast_math=fast_math, sort_every=sort_every,
                  tile_slack=tile_slack)
    for m_q, q, ppc, parts in species:
        sim.add_species(m_q, q, ppc, parts)
    if history:
        sim.history_enable(run.steps)
    sim.set_graphs(graphs)
    return sim


def load_sims(runs, tile=(32, 16), fast_math=True, sort_every=0, workers=None, **kw):
    """Creates the runs' simulations; particles are drawn by a thread pool
    and uploaded in run order."""
    workers = workers or min(16, os.cpu_count() or 1)
    tiles = tile if isinstance(tile, list) else [tile] * len(runs)
    sims = [None] * len(runs)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        for k, sp in enumerate(ex.map(load_run, runs)):
            sims[k] = make_sim(runs[k], sp, tile=tiles[k], fast_math=fast_math, sort_every=sort_every, **kw)
    return sims


@dataclass
class ScanResult:
    histories: list            # per run: [steps, 6 + n_species] energies
    device_ms: float           # device time of the stepping (CUDA events)
    wall_s: float              # host wall time of the stepping
    particle_steps: int
    groups: int
    extra: dict = field(default_factory=dict)

    @property
    def rate(self):
        """particle-steps per second of device time"""
        return self.particle_steps / (self.device_ms * 1e-3)


def run_batched(sims, runs, group=None, stream_groups=None) -> ScanResult:
    """Advances every run by its step count, ``group`` runs per batch (all
    at once by default), one after another; each batch deals its members
    into ``stream_groups`` graph groups (None: the batch's default)."""
    group = group or len(sims)
    steps = runs[0].steps
    if any(r.steps != steps for r in runs):
        raise ValueError("batched runs must share the step count")
    t0 = time.perf_counter()
    ms = 0.0
    ngroups = 0
    sg = []
    for g0 in range(0, len(sims), group):
        b = CudaBatch(sims[g0:g0 + group], groups=stream_groups)
        sg.append(b.groups)
        b.step(steps)
        ms += b.last_ms()
        b.close()
        ngroups += 1
    wall = time.perf_counter() - t0
    hist = [s.history() for s in sims]
    nps = sum(r.particles() * r.steps for r in runs)
    return ScanResult(hist, ms, wall, nps, ngroups, {**_counters(sims), "stream_groups": sg})


def run_sequential(sims, runs) -> ScanResult:
    """The plain path: each run stepped alone, one after another."""
    t0 = time.perf_counter()
    ms = 0.0
    for s, r in zip(sims, runs):
        s.step(r.steps)
        ms += s.last_ms()
    wall = time.perf_counter() - t0
    hist = [s.history() for s in sims]
    nps = sum(r.particles() * r.steps for r in runs)
    return ScanResult(hist, ms, wall, nps, len(sims), _counters(sims))


def _counters(sims):
    info = [s.info() for s in sims]
    return {"relayouts": sum(i["relayouts"] for i in info), "captures": sum(i["captures"] for i in info)}


def scan_sort_every(steps, longest=8):
    """The longest cell-sort interval up to ``longest`` whose block of
    2 x interval steps divides the run: the batch then replays whole blocks
    only, with no shorter tail block to record."""
    for k in range(longest, 0, -1):
        if steps % (2 * k) == 0:
            return k
    return longest


def tile_by_ppc(run):
    """A tile shape that holds some thousands of particles of a species:
    larger tiles for runs with few particles per cell, so that a tile's fixed
    work (its field halo, the neighbours' outboxes, the sums at its end) is
    spread over enough particles."""
    ppc = run.ppc[0] * run.ppc[1]
    t = (32, 32) if ppc <= 6 else ((32, 16) if ppc <= 12 else (16, 16))
    return (min(t[0], run.nx[0]), min(t[1], run.nx[1])) if min(run.nx) >= 32 else (16, 16)


def tiles_for(runs, choice):
    """The per-run tiles of an autotuner choice: one shape for every run, or
    the policy ``"by_ppc"`` (tile_by_ppc per run)."""
    if choice == "by_ppc":
        return [tile_by_ppc(r) for r in runs]
    return [tuple(choice)] * len(runs)


def autotune_tile(runs, candidates=((16, 16), (32, 16), (16, 8), "by_ppc"), sample=64, steps=32, fast_math=True,
                  sort_every=0):
    """Picks the particle tiles of a scan: times a batch of ``sample`` runs
    (spread evenly over the scan's sizes) for ``steps`` steps with each
    candidate (one tile shape for every run, or the per-run policy
    ``"by_ppc"``), after one untimed pass of as many steps (graph capture),
    and returns (best candidate, {candidate: particle-steps/s})."""
    order = np.argsort([r.nx[0] * r.nx[1] * r.ppc[0] * r.ppc[1] for r in runs])
    pick = [runs[int(order[int(i)])] for i in np.linspace(0, len(runs) - 1, min(sample, len(runs)))]
    probe = [ScanRun(r.nx, r.ppc, r.uz, r.uth, r.dx, r.dt, r.seed, steps) for r in pick]
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        species = list(ex.map(load_run, probe))
    rates = {}
    for t in candidates:
        sims = [make_sim(r, sp, tile=tt, fast_math=fast_math, sort_every=sort_every, history=True)
                for r, sp, tt in zip(probe, species, tiles_for(probe, t))]
        b = CudaBatch(sims)
        b.step(steps)  # warm-up (graph capture and instantiation)
        b.step(steps)
        rates[t] = sum(r.particles() * steps for r in probe) / (b.last_ms() * 1e-3)
        b.close()
        for s in sims:
            s.close()
    best = max(rates, key=rates.get)
    return best, rates
