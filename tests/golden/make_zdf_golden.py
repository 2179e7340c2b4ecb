"""Generate the ZDF fixtures in tests/golden/zdf/ from the REFERENCE itself.

* writer/: the calls of tests/zdf_cases.py made on the reference's own
  em2d/zdf.c (compiled into oracle/_ref/libzpic_ref.so by oracle/Makefile);
  libzpic_em2d must write the same bytes for the same calls.
* report/: the reference's emf_report, current_report and spec_report
  (charge, phase space, particles) after REPORT_STEPS steps of the deck
  REPORT_DECK (a plasma with a moving window and a laser, so that the
  window offset shows in the charge axis).
* report0/: the species reports of the same deck right after loading
  (iteration 0), which the host path of libzpic_em2d reproduces on a CPU.

Usage (where the reference tree and a C compiler are present)::

    python tests/golden/make_zdf_golden.py
"""
import ctypes as C
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import zdf_cases  # noqa: E402
from oracle import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "zdf")

from zdf_cases import PHA_NX, PHA_RANGE, PHA_TYPE, REPORT_DECK, REPORT_STEPS  # noqa: E402


def species_reports(sim):
    sim.report_spec(0, 0x1000)
    sim.report_spec(0, PHA_TYPE, PHA_NX, PHA_RANGE)
    sim.report_spec(0, 0x3000)


def reports(sim):
    """The report calls, in the order the tests make them."""
    for field in (0, 1):
        for fc in range(3):
            sim.report_emf(field, fc)
    for jc in range(3):
        sim.report_current(jc)
    sim.report_spec(0, 0x1000)
    sim.report_spec(0, PHA_TYPE, PHA_NX, PHA_RANGE)
    sim.report_spec(0, 0x3000)


def main():
    pyoracle.build()
    if not pyoracle.ref_available():
        sys.exit("reference build not available (oracle/_ref missing)")
    shutil.rmtree(OUT, ignore_errors=True)
    lib = zdf_cases.bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libzpic_ref.so")))
    files = zdf_cases.write_all(lib, os.path.join(OUT, "writer"))
    print("writer:", files)
    # the reference keeps its generator in process globals: a fresh process
    if os.fork() == 0:
        from decks import build_cpu
        os.makedirs(os.path.join(OUT, "report"), exist_ok=True)
        os.chdir(os.path.join(OUT, "report"))
        s = build_cpu("zdf", backend="ref", deck=REPORT_DECK)
        for _ in range(REPORT_STEPS):
            s.iter()
        reports(s)
        os._exit(0)
    _, st = os.wait()
    if st != 0:
        sys.exit("report run failed")
    if os.fork() == 0:
        from decks import build_cpu
        os.makedirs(os.path.join(OUT, "report0"), exist_ok=True)
        os.chdir(os.path.join(OUT, "report0"))
        s = build_cpu("zdf", backend="ref", deck=REPORT_DECK)
        species_reports(s)
        os._exit(0)
    _, st = os.wait()
    if st != 0:
        sys.exit("report0 run failed")
    for dirpath, _, names in sorted(os.walk(OUT)):
        for n in names:
            print("report:", os.path.relpath(os.path.join(dirpath, n), OUT))


if __name__ == "__main__":
    main()
