"""The host side of batched parameter scans, without a GPU: the run table,
and particle loading of every run as a fresh process of the reference would
do it (bit-exact against the oracle, whatever the loading order or thread)."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_scan_table():
    from zpic_gb300 import batch

    runs = batch.weibel_scan(n_runs=256)
    again = batch.weibel_scan(n_runs=256)
    assert runs == again
    nx = np.array([r.nx for r in runs])
    ppc = np.array([r.ppc for r in runs])
    assert nx.min() >= 64 and nx.max() <= 256
    assert ppc.min() >= 2 and ppc.max() <= 8
    assert all(0.2 <= r.uz <= 0.8 and 0.02 <= r.uth <= 0.2 for r in runs)
    for r in runs:
        cour = (1.0 / (1.0 / r.dx ** 2 + 1.0 / r.dx ** 2)) ** 0.5
        assert r.dt < cour and abs(r.dt - 0.9 * cour) < 1e-6
    assert [r.seed for r in runs[:2]] == [(12345, 67890), (12346, 67891)]
    mean_parts = np.mean([r.particles() for r in runs])
    assert 0.8e6 < mean_parts < 2.2e6


def test_tile_choices():
    """The autotuner's candidates: one shape for every run, or the per-run
    policy that gives runs with few particles per cell larger tiles; every
    tile fits its grid and is a shape the kernels are built for."""
    from zpic_gb300 import batch

    runs = batch.weibel_scan(n_runs=64)
    assert batch.tiles_for(runs, (32, 16)) == [(32, 16)] * len(runs)
    tiles = batch.tiles_for(runs, "by_ppc")
    supported = {(16, 16), (8, 8), (16, 8), (32, 16), (32, 32), (8, 16), (16, 32)}
    for r, t in zip(runs, tiles):
        assert t in supported and t[0] <= r.nx[0] and t[1] <= r.nx[1]
        ppc = r.ppc[0] * r.ppc[1]
        assert t == ((32, 32) if ppc <= 6 else (32, 16) if ppc <= 12 else (16, 16))
    # the sort interval's block (2 sort_every steps) divides the run
    for steps in (300, 96, 50):
        se = batch.scan_sort_every(steps)
        assert 1 <= se <= 8 and steps % (2 * se) == 0


_CHILD = r"""
import sys
sys.path[:0] = [{root!r}]
from concurrent.futures import ThreadPoolExecutor
from oracle import pyoracle as P
from zpic_gb300 import batch
runs = batch.weibel_scan(n_runs=6, steps=10, nx_range=(16, 40), ppc_range=(2, 4), seed=3)
# loaded in reverse order on four threads
with ThreadPoolExecutor(4) as ex:
    got = list(ex.map(batch.load_run, runs[::-1]))[::-1]
for r, sp in zip(runs, got):
    P.set_rand_seed(*r.seed, fresh=True)
    cpu = P.CpuSim(r.nx, r.box, r.dt)
    for sgn, (m_q, q, ppc, parts) in zip((1.0, -1.0), sp):
        cpu.add_species("e", -1.0, list(r.ppc), ufl=[0, 0, sgn * r.uz], uth=[r.uth] * 3)
    for k, (m_q, q, ppc, parts) in enumerate(sp):
        ref = cpu.particles(k)
        assert parts.tobytes() == ref.tobytes(), (r, k)
        assert q == cpu.q(k)
print("OK")
"""


def test_scan_loading_matches_oracle():
    from zpic_gb300 import build
    from oracle import pyoracle

    build.build()
    pyoracle.build()
    code = _CHILD.format(root=ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_cell_mean_removed_when_ny_exceeds_nx():
    """With more rows than columns the reference's per-cell momentum table
    is indexed past its end (undefined behaviour); the oracle and the host
    loader define it as removing each cell's mean momentum."""
    from oracle import pyoracle as P

    P.build()
    P.set_rand_seed(11, 22, fresh=True)
    cpu = P.CpuSim((8, 12), (0.8, 1.2), 0.05)
    cpu.add_species("e", -1.0, [3, 3], ufl=[0.0, 0.0, 0.3], uth=[0.1, 0.1, 0.1])
    p = cpu.particles(0)
    cell = p["ix"] + 8 * p["iy"]
    assert np.unique(cell).size == 96
    for c in range(96):
        m = p[cell == c]
        assert m.size == 9
        for f, want in (("ux", 0.0), ("uy", 0.0), ("uz", 0.3)):
            assert abs(float(np.mean(m[f].astype(np.float64))) - want) < 1e-6
