"""The em1d drop-in C API (include/em1d/*.h, libzpic_em1d) against the
reference em1d.

* The library exports every function the headers declare.
* The reference's own em1d decks (main.c and input/*.c) compile and link
  against the drop-in headers and library (where the reference tree exists).
* tests/em1d_deck.c, built against the drop-in, writes reports after loading
  that equal the reference's byte for byte (no GPU involved before the first
  step); the fixtures in tests/golden/em1d_reports come from the same program
  built against the reference (tests/golden/make_em1d_reports.py).
* On the GPU, after 40-60 steps: the reports' metadata bytes equal the
  reference's, the values within the forward tolerance, the energy lines and
  window moves as the reference's.
"""
import ctypes
import glob
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import zdf_read

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "em1d_reports")
INC = os.path.join(ROOT, "include", "em1d")
LIBDIR = os.path.join(ROOT, "zpic_gb300", "lib")
REF = os.path.join(os.environ.get("ZPIC_REFERENCE", "/root/reference"), "em1d")
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_em1d_reports import LOAD_ONLY, STEPS  # noqa: E402

# functions the deck itself defines
DECK_FUNCS = {"sim_init", "sim_report"}


@pytest.fixture(scope="module")
def built():
    from zpic_gb300 import build

    build.build()
    return os.path.join(LIBDIR, "libzpic_em1d.so")


def declared():
    names = set()
    for h in glob.glob(os.path.join(INC, "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for line in text.splitlines():
            if "(*" in line or line.startswith("#") or line.startswith(" "):
                continue
            m = re.match(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-z_0-9]*)\s*\(", line)
            if m:
                names.add(m.group(1))
    return sorted(names - DECK_FUNCS)


def test_every_declared_function_is_exported(built):
    lib = ctypes.CDLL(built)
    names = declared()
    assert len(names) >= 35, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


GUARDS = ["__SIMULATION__", "__PARTICLES__", "__EMF__", "__CURRENT__", "__ZPIC__", "__TIMER__", "__RANDOM__",
          "__ZDF__"]


def _compile_against_dropin(src, obj):
    """Compiles a reference source with the drop-in's declarations: its own
    headers are emptied by defining their guards, ours are included first."""
    cmd = ["gcc", "-c", "-std=c99", "-D_DEFAULT_SOURCE", "-w", "-o", obj, src]
    for h in ("simulation.h", "timer.h", "zdf.h", "random.h"):
        cmd += ["-include", os.path.join(INC, h)]
    cmd += ["-D" + g for g in GUARDS]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _link(objs, exe):
    cmd = ["gcc", "-o", exe] + objs + ["-L", LIBDIR, "-lzpic_em1d", "-Wl,-rpath," + LIBDIR, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_reference_decks_build_against_dropin(built, tmp_path):
    if not os.path.isdir(REF):
        pytest.skip("reference tree not present")
    # the reference's main.c with its default deck, linked into a program
    _compile_against_dropin(os.path.join(REF, "main.c"), str(tmp_path / "main.o"))
    _link([str(tmp_path / "main.o")], str(tmp_path / "zpic_em1d"))
    # every input deck, linked with a main of our own (built, not run)
    main = tmp_path / "deck_main.c"
    main.write_text('#include "simulation.h"\n'
                    "int main(void) { t_simulation s; sim_init(&s); sim_report(&s); sim_iter(&s);\n"
                    "  sim_timings(&s, 0, 1); sim_delete(&s); return 0; }\n")
    r = subprocess.run(["gcc", "-c", "-std=c99", "-I", INC, "-o", str(tmp_path / "deck_main.o"), str(main)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    decks = sorted(glob.glob(os.path.join(REF, "input", "*.c")))
    assert len(decks) >= 5
    for deck in decks:
        name = os.path.basename(deck)[:-2]
        _compile_against_dropin(deck, str(tmp_path / f"{name}.o"))
        _link([str(tmp_path / "deck_main.o"), str(tmp_path / f"{name}.o")], str(tmp_path / f"deck_{name}"))


def _build_deck(tmp_path):
    exe = str(tmp_path / "em1d_deck")
    cmd = ["gcc", "-O2", "-std=c99", "-D_DEFAULT_SOURCE", "-I", INC, os.path.join(ROOT, "tests", "em1d_deck.c"),
           "-L", LIBDIR, "-lzpic_em1d", "-Wl,-rpath," + LIBDIR, "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run_deck(exe, deck, steps, cwd):
    os.makedirs(cwd, exist_ok=True)
    r = subprocess.run([exe, deck, str(steps)], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def _files(root, it):
    out = []
    for dirpath, _, names in os.walk(root):
        out += [os.path.relpath(os.path.join(dirpath, n), root) for n in names if f"-{it:06d}.zdf" in n]
    return sorted(out)


@pytest.mark.parametrize("deck", sorted(STEPS) + LOAD_ONLY)
def test_reports_at_load_match_reference(built, tmp_path, deck):
    exe = _build_deck(tmp_path)
    out = _run_deck(exe, deck, 0, str(tmp_path / deck))
    ref = os.path.join(GOLD, deck)
    files = _files(ref, 0)
    assert len(files) >= 10
    assert files == _files(str(tmp_path / deck), 0)
    for f in files:
        assert open(os.path.join(ref, f), "rb").read() == (tmp_path / deck / f).read_bytes(), f
    assert out.splitlines()[0] == open(os.path.join(ref, "stdout.txt")).read().splitlines()[0]


def test_external_fields_stop_the_program(built, tmp_path):
    """The 1-D GPU step has no external fields: the drop-in stops with a
    message and the reference's exit status for invalid settings."""
    exe = _build_deck(tmp_path)
    r = subprocess.run([exe, "extfld", "0"], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert r.returncode == 255
    assert "external fields are not supported" in r.stderr


def test_golden_reports_are_the_references(tmp_path):
    """The committed fixtures are what the reference writes (where it exists)."""
    if not os.path.isdir(REF):
        pytest.skip("reference tree not present")
    import make_em1d_reports as M

    exe = str(tmp_path / "ref_deck")
    M.build_reference(exe)
    for deck, steps in list(STEPS.items()) + [(d, 0) for d in LOAD_ONLY]:
        d = str(tmp_path / deck)
        os.makedirs(d)
        out = M.run(exe, deck, steps, d)
        assert out == open(os.path.join(GOLD, deck, "stdout.txt")).read()
        for it in sorted({0, steps}):
            for f in _files(os.path.join(GOLD, deck), it):
                assert open(os.path.join(GOLD, deck, f), "rb").read() == open(os.path.join(d, f), "rb").read(), f


def _rel(a, b, floor):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), floor, 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("deck", sorted(STEPS))
def test_reports_after_steps_match_reference(built, tmp_path, deck):
    exe = _build_deck(tmp_path)
    steps = STEPS[deck]
    out = _run_deck(exe, deck, steps, str(tmp_path / deck))
    ref = os.path.join(GOLD, deck)
    files = _files(ref, steps)
    assert files == _files(str(tmp_path / deck), steps)
    data = {}
    for f in files:
        ours_recs, ours_raw = zdf_read.read(str(tmp_path / deck / f))
        ref_recs, ref_raw = zdf_read.read(os.path.join(ref, f))
        # every metadata record, the dataset headers and the particle count
        assert zdf_read.header_bytes(ours_raw) == zdf_read.header_bytes(ref_raw), f
        data[f] = ([v["data"] for k, _, v in ours_recs if k == 0x10], [v["data"] for k, _, v in ref_recs if k == 0x10])
    # fields and currents measured against the largest norm of their kind
    # (components at fluctuation level do not turn round-off into large
    # relative errors)
    for kind in ("EMF", "CURRENT"):
        group = [f for f in files if f.startswith(kind)]
        scale = max(np.linalg.norm(np.asarray(data[f][1][0], dtype=np.float64)) for f in group)
        for f in group:
            err = _rel(data[f][0][0], data[f][1][0], 1e-2 * scale)
            assert err <= 1e-4, f"{f}: relative error {err:.2e}"
    for f in files:
        if f.startswith("CHARGE") or f.startswith("PHASESPACE"):
            err = _rel(data[f][0][0], data[f][1][0], 0.0)
            assert err <= 1e-4, f"{f}: relative error {err:.2e}"
        elif f.startswith("PARTICLES"):
            # particle order differs (the GPU compacts and sorts its own way)
            for a, b in zip(*data[f]):
                assert np.allclose(np.sort(a), np.sort(b), rtol=0, atol=1e-4 * max(np.abs(b).max(), 1e-6)), f
    ref_out = open(os.path.join(ref, "stdout.txt")).read().splitlines()
    ours_out = out.splitlines()
    assert ours_out[-1] == ref_out[-1]  # window moves
    for a, b in zip(ours_out[:2], ref_out[:2]):
        va = [float(x) for x in a.split("=")[1].split()]
        vb = [float(x) for x in b.split("=")[1].split()]
        assert np.allclose(va, vb, rtol=1e-4, atol=1e-9), (a, b)
