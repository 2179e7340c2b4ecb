"""Generate tests/golden/em1d_reports/<deck>/ from the REFERENCE em1d: the
deck program tests/em1d_deck.c compiled against the reference's own em1d
sources (where they lie; nothing is copied) with the oracle's strict IEEE
flags, run for STEPS[deck] steps in an empty directory.  Kept: every report
file it writes (after loading and after the last step) and its printed
lines (energies, window moves) in stdout.txt.

Usage (where the reference tree and a C compiler are present)::

    python tests/golden/make_em1d_reports.py
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(os.environ.get("ZPIC_REFERENCE", "/root/reference"), "em1d")
OUT = os.path.join(HERE, "em1d_reports")
DECK_C = os.path.join(ROOT, "tests", "em1d_deck.c")
STEPS = {"lwfa": 60, "twostream": 40, "absorbing": 60}
# decks compared at loading only (profiles the GPU step loads but does not inject)
LOAD_ONLY = ["density"]
REF_SRC = ["particles.c", "current.c", "emf.c", "simulation.c", "random.c", "timer.c", "zdf.c"]
FLAGS = ["-O2", "-std=c99", "-fno-fast-math", "-ffp-contract=off", "-D_DEFAULT_SOURCE", "-w"]


def build_reference(exe):
    cmd = ["gcc"] + FLAGS + ["-I", REF, DECK_C] + [os.path.join(REF, f) for f in REF_SRC] + ["-lm", "-o", exe]
    subprocess.run(cmd, check=True)


def run(exe, deck, steps, cwd):
    r = subprocess.run([exe, deck, str(steps)], cwd=cwd, capture_output=True, text=True, check=True)
    return r.stdout


def main():
    if not os.path.isdir(REF):
        sys.exit("reference em1d sources not found")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "em1d_deck_ref")
        build_reference(exe)
        for deck, steps in list(STEPS.items()) + [(d, 0) for d in LOAD_ONLY]:
            d = os.path.join(OUT, deck)
            shutil.rmtree(d, ignore_errors=True)
            os.makedirs(d)
            out = run(exe, deck, steps, d)
            with open(os.path.join(d, "stdout.txt"), "w") as f:
                f.write(out)
            print("wrote", deck)


if __name__ == "__main__":
    main()
