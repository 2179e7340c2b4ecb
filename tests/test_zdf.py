"""ZDF diagnostic files (include/em2d/zdf.h, zpic_gb300/csrc/em2d/zdf_io.c).

* The writer against the reference's own em2d/zdf.c, byte for byte, on the
  calls of zdf_cases.py (fixtures in tests/golden/zdf/writer, made by
  tests/golden/make_zdf_golden.py).
* The species reports of the drop-in library (charge, phase space,
  particles) on a freshly loaded species, on the CPU: byte for byte against
  the reference's reports of the same loading (tests/golden/zdf/report0).
* On the GPU: every report of a simulation after 30 steps with a moving
  window against the reference's after the same steps: the metadata bytes
  identical, the values within the forward tolerance.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import zdf_cases
import zdf_read

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "zdf")


def _golden_files(sub):
    out = []
    for dirpath, _, names in os.walk(os.path.join(GOLD, sub)):
        out += [os.path.relpath(os.path.join(dirpath, n), os.path.join(GOLD, sub)) for n in names]
    return sorted(out)


@pytest.fixture(scope="module")
def em2d():
    from zpic_gb300 import build

    build.build()
    from zpic_gb300 import em2d as m

    return m


def test_writer_bytes_match_reference(em2d, tmp_path):
    lib = zdf_cases.bind(C.CDLL(em2d.LIB_PATH))
    files = zdf_cases.write_all(lib, str(tmp_path))
    assert sorted(files) == _golden_files("writer")
    for f in files:
        ours = (tmp_path / f).read_bytes()
        ref = open(os.path.join(GOLD, "writer", f), "rb").read()
        assert ours == ref, f


def test_reader_reads_reference_reports():
    files = _golden_files("report")
    assert len(files) == 12
    for f in files:
        recs, raw = zdf_read.read(os.path.join(GOLD, "report", f))
        kinds = [k for k, _, _ in recs]
        assert recs[0] == (3, "TYPE", "particles" if f.startswith("PARTICLES") else "grid"), f
        it = [v for k, n, v in recs if k == 0x20][0]
        assert it["n"] == zdf_cases.REPORT_STEPS
        assert kinds.count(0x10) == (5 if f.startswith("PARTICLES") else 1)
        payload = sum(v["data"].nbytes for k, _, v in recs if k == 0x10)
        assert len(zdf_read.header_bytes(raw)) == len(raw) - payload


_CHILD_HOST = r"""
import ctypes as C, sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
import zdf_cases
from zpic_gb300 import em2d as m

d = zdf_cases.REPORT_DECK
sp = d["species"][0]
lib = m._load()
lib.set_rand_seed(12345, 67890)
ts = m.t_species()
dens = m.Density(type="step", start=sp["density"]["start"])
arr = lambda v, t: np.ascontiguousarray(v, dtype=t)
ppc, uth = arr(sp["ppc"], np.int32), arr(sp["uth"], np.float32)
ufl, nx, box = arr([0, 0, 0], np.float32), arr(d["nx"], np.int32), arr(d["box"], np.float32)
lib.spec_new(C.byref(ts), sp["name"].encode(), sp["m_q"], m._ptr(ppc), m._ptr(ufl), m._ptr(uth),
             m._ptr(nx), m._ptr(box), d["dt"], C.byref(dens._d))
ts.moving_window = 1
nxp = arr(zdf_cases.PHA_NX, np.int32)
rg = arr(zdf_cases.PHA_RANGE, np.float32)
lib.spec_report(C.byref(ts), 0x1000, None, None)
lib.spec_report(C.byref(ts), zdf_cases.PHA_TYPE, m._ptr(nxp), m._ptr(rg))
lib.spec_report(C.byref(ts), 0x3000, None, None)
assert m.zdf_flush() == 0
print("OK")
"""


def test_species_reports_match_reference_at_load(em2d, tmp_path):
    code = _CHILD_HOST.format(root=ROOT, tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
    for f in _golden_files("report0"):
        assert (tmp_path / f).read_bytes() == open(os.path.join(GOLD, "report0", f), "rb").read(), f


_CHILD_GPU = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import zdf_cases
from zpic_gb300 import em2d

d = zdf_cases.REPORT_DECK
em2d.gpu_options(fast_math=False)
em2d.set_rand_seed(12345, 67890)
sp = d["species"][0]
species = [em2d.Species(sp["name"], sp["m_q"], sp["ppc"], uth=sp["uth"],
                        density=em2d.Density(type="step", start=sp["density"]["start"]))]
sim = em2d.Simulation(d["nx"], d["box"], d["dt"], species=species)
sim.add_laser(em2d.Laser(**d["laser"]))
sim.set_moving_window()
sim.set_smooth(em2d.Smooth(**d["smooth"]))
for _ in range(zdf_cases.REPORT_STEPS):
    sim.iter()
for t in ("E", "B"):
    for fc in range(3):
        sim.emf.report(t, fc)
for jc in range(3):
    sim.current.report(jc)
species[0].report("charge")
species[0].report("pha", quants=("x1", "u1"), pha_nx=zdf_cases.PHA_NX, pha_range=zdf_cases.PHA_RANGE)
species[0].report("particles")
assert em2d.zdf_flush() == 0
print("OK")
"""


def _rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
def test_reports_match_reference_after_steps(em2d, tmp_path):
    code = _CHILD_GPU.format(root=ROOT, tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
    for f in _golden_files("report"):
        ours_recs, ours_raw = zdf_read.read(str(tmp_path / f))
        ref_recs, ref_raw = zdf_read.read(os.path.join(GOLD, "report", f))
        # every metadata record, the dataset headers and the particle count
        assert zdf_read.header_bytes(ours_raw) == zdf_read.header_bytes(ref_raw), f
        ours_d = [v["data"] for k, _, v in ours_recs if k == 0x10]
        ref_d = [v["data"] for k, _, v in ref_recs if k == 0x10]
        if f.startswith("PARTICLES"):
            # particle order differs (tiles on the GPU): compare each
            # quantity's sorted values
            for a, b in zip(ours_d, ref_d):
                assert np.allclose(np.sort(a), np.sort(b), rtol=0, atol=1e-4 * max(np.abs(b).max(), 1e-6)), f
        else:
            err = _rel_l2(ours_d[0], ref_d[0])
            assert err <= 1e-4, f"{f}: relative error {err:.2e}"
