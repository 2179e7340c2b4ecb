"""A C input deck compiled against the em2d drop-in headers and linked to
libzpic_em2d (as a reference deck is linked to the reference's objects):
it builds here without a GPU, and on a GPU its energies after 10 steps match
the oracle's run of the same deck."""
import os
import subprocess

import numpy as np
import pytest

from decks import build_cpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "zpic_gb300", "lib")


def _build(tmp_path):
    from zpic_gb300 import build

    build.build()
    exe = str(tmp_path / "deck_weibel")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include", "em2d"),
                    os.path.join(ROOT, "tests", "c_deck", "deck_weibel.c"), "-L", LIB, "-lzpic_em2d",
                    f"-Wl,-rpath,{LIB}", "-lm", "-o", exe], check=True)
    return exe


def test_c_deck_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_c_deck_matches_oracle(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "10"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = {"emf": [], "kin": [], "np": []}
    for line in r.stdout.splitlines():
        key, v = line.split()
        vals[key].append(float(v))
    cpu = build_cpu("weibel_smooth")
    cpu.iter(10)
    emf_c = cpu.emf_energy()
    assert np.all(np.abs(np.array(vals["emf"]) - emf_c) <= 1e-5 * np.abs(emf_c).max())
    for k in range(2):
        assert abs(vals["kin"][k] - cpu.energy(k)) <= 1e-5 * abs(cpu.energy(k))
        assert int(vals["np"][k]) == cpu.np_(k)


def _build_thermal(tmp_path):
    from zpic_gb300 import build

    build.build()
    exe = str(tmp_path / "deck_thermal")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include", "em2d"),
                    os.path.join(ROOT, "zpic_gb300", "csrc", "em2d", "deck_thermal.c"), "-L", LIB, "-lzpic_em2d",
                    f"-Wl,-rpath,{LIB}", "-lm", "-o", exe], check=True)
    return exe


def test_thermal_deck_compiles_and_links(tmp_path):
    """The throughput workload's C deck (the bench's drop-in leg)."""
    exe = _build_thermal(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("mirrors", ["every", "demand"])
def test_thermal_deck_matches_oracle(tmp_path, mirrors):
    """The thermal C deck on a 32 x 32 grid (box 3.2, 4 x 4 ppc, uth 0.05,
    compensated level-1 smoothing on both axes), 10 steps with either mirror
    policy, against the oracle's run of the same deck."""
    exe = _build_thermal(tmp_path)
    r = subprocess.run([exe, "10", mirrors, "32"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    v = dict(line.split() for line in r.stdout.splitlines())
    deck = dict(nx=[32, 32], box=[3.2, 3.2], dt=0.05,
                species=[dict(name="electrons", m_q=-1.0, ppc=[4, 4], uth=[0.05, 0.05, 0.05])],
                smooth=dict(xtype="compensated", xlevel=1, ytype="compensated", ylevel=1))
    cpu = build_cpu(None, deck=deck)
    cpu.iter(10)
    assert int(v["particles"]) == cpu.np_(0)
    assert abs(float(v["kinetic"]) - cpu.energy(0)) <= 1e-5 * abs(cpu.energy(0))
    emf = float(cpu.emf_energy().sum())
    assert abs(float(v["field"]) - emf) <= 1e-5 * abs(emf)


def test_mirror_passes_split_over_threads(tmp_path):
    """The drop-in's threaded compare and copy of the host mirrors (no GPU
    call): spans around the 4 MB split between threads, flipped bytes at
    the ends and in the middle."""
    from zpic_gb300 import build

    build.build()
    exe = str(tmp_path / "mirror_passes")
    subprocess.run(["gcc", "-O2", "-std=c99", "-D_DEFAULT_SOURCE", "-pthread", "-w",
                    os.path.join(ROOT, "tests", "c_deck", "mirror_passes.c"),
                    os.path.join(ROOT, "zpic_gb300", "csrc", "em2d", "zdf_io.c"), "-L", LIB, "-lzpic_cuda",
                    f"-Wl,-rpath,{LIB}", "-lm", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
