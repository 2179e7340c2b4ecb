"""The reference's own callers of the em2d C API, built against the drop-in
(``include/em2d`` + ``libzpic_em2d``) instead of the reference's C sources:

* its ``em2d/main.c`` with its default deck, and every deck in
  ``em2d/input/`` linked with a main of ours;
* its Cython module (``python/source/em2d.pyx`` + ``em2d.pxd``),
  unmodified, translated and linked by ``oracle/cython_em2d.py``; importing
  it with immediate symbol binding shows that every function it calls is
  exported.

These build and link here without a GPU (where the reference tree is
present); the GPU run of the Cython module is in
``tests/test_gpu_cython_dropin.py``.
"""
import glob
import os
import subprocess
import sys

import pytest

from oracle.pyoracle import REFERENCE_ROOT

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include", "em2d")
LIBDIR = os.path.join(ROOT, "zpic_gb300", "lib")
REF = os.path.join(REFERENCE_ROOT, "em2d")
GUARDS = ["__SIMULATION__", "__PARTICLES__", "__EMF__", "__CURRENT__", "__ZPIC__", "__TIMER__", "__RANDOM__",
          "__ZDF__"]


@pytest.fixture(scope="module")
def built():
    from zpic_gb300 import build

    build.build()
    return os.path.join(LIBDIR, "libzpic_em2d.so")


def _compile_against_dropin(src, obj):
    """Compiles a reference source with the drop-in's declarations: its own
    headers are emptied by defining their guards, ours are included first."""
    cmd = ["gcc", "-c", "-std=c99", "-D_DEFAULT_SOURCE", "-w", "-o", obj, src]
    for h in ("zpic.h", "simulation.h", "timer.h", "zdf.h", "random.h"):
        cmd += ["-include", os.path.join(INC, h)]
    cmd += ["-D" + g for g in GUARDS]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def _link(objs, exe):
    cmd = ["gcc", "-o", exe] + objs + ["-L", LIBDIR, "-lzpic_em2d", "-Wl,-rpath," + LIBDIR,
                                       "-Wl,--no-undefined", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_reference_decks_build_against_dropin(built, tmp_path):
    if not os.path.isdir(REF):
        pytest.skip("reference tree not present")
    # the reference's main.c with its default deck (input/weibel.c), linked
    _compile_against_dropin(os.path.join(REF, "main.c"), str(tmp_path / "main.o"))
    _link([str(tmp_path / "main.o")], str(tmp_path / "zpic_em2d"))
    # every input deck, linked with a main of our own (built, not run)
    main = tmp_path / "deck_main.c"
    main.write_text('#include "simulation.h"\n'
                    "int main(void) { t_simulation s; sim_init(&s); sim_report(&s); sim_iter(&s);\n"
                    "  sim_report_energy(&s); sim_timings(&s, 0, 1); sim_delete(&s); return 0; }\n")
    r = subprocess.run(["gcc", "-c", "-std=c99", "-I", INC, "-o", str(tmp_path / "deck_main.o"), str(main)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    decks = sorted(glob.glob(os.path.join(REF, "input", "*.c")))
    assert len(decks) >= 6
    for deck in decks:
        name = os.path.basename(deck)[:-2]
        _compile_against_dropin(deck, str(tmp_path / f"{name}.o"))
        _link([str(tmp_path / "deck_main.o"), str(tmp_path / f"{name}.o")], str(tmp_path / f"deck_{name}"))


def test_reference_cython_module_builds_against_dropin(built):
    from oracle import cython_em2d

    pytest.importorskip("Cython")
    if not cython_em2d.generate():
        pytest.skip("reference tree not present")
    path = cython_em2d.compile()
    assert path and os.path.exists(path)
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from oracle import cython_em2d\n"
            "m = cython_em2d.load()\n"
            "names = {'Simulation', 'Species', 'EMF', 'Current', 'Density', 'Laser', 'Smooth',\n"
            "         'ExternalField', 'InitialField'}\n"
            "assert names <= set(dir(m)), sorted(names - set(dir(m)))\n"
            "print('ok')\n" % ROOT)
    env = dict(os.environ, LD_BIND_NOW="1")  # every symbol resolved at load
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr[-3000:]
