"""Generate the long-run fixtures of the benchmark configurations from the
REFERENCE itself.

Runs the unmodified reference em2d (compiled from its own sources into
``oracle/_ref/libzpic_ref.so`` by ``oracle/Makefile``; strict IEEE build, and
the stock ``-Ofast`` build for the spread between two builds of the same
code) on the decks of ``tests/decks.py:CONFIG_DECKS`` and stores:

``c1_weibel_history.npz``
    the Weibel deck (128^2, two electron streams, 4x4 ppc, 500 steps): after
    every step the six field-energy components and the kinetic energy of
    both species (row 0 is the initial state), for the strict build
    (``hist``) and the ``-Ofast`` build (``hist_fast``).

``c5_wake.npz``
    the moving-window wakefield deck (2000 x 256, 3000 steps): the on-axis
    Ex row (cells 0..nx-1 of row ny/2) after steps 1000, 2000 and 3000, the
    field energies after every step, the particle count and window moves at
    the end (strict build only: the run takes about a quarter of an hour on
    one core).

Usage (where the reference tree and a C compiler are present)::

    python tests/golden/make_config_golden.py [c1] [c5]   # default: both
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from decks import CONFIG_DECKS, build_cpu  # noqa: E402
from oracle import pyoracle  # noqa: E402

C5_SNAPSHOTS = (1000, 2000, 3000)


def history(s, steps, n_species):
    h = np.zeros((steps + 1, 6 + n_species))
    h[0, :6] = s.emf_energy()
    for i in range(steps):
        s.iter()
        h[i + 1, :6] = s.emf_energy()
        h[i + 1, 6:] = [s.energy(k) for k in range(n_species)]
    return h


def make_c1():
    d = CONFIG_DECKS["c1_weibel"]
    out = {}
    for key, fast in (("hist", False), ("hist_fast", True)):
        t = time.time()
        s = build_cpu("c1_weibel", backend="ref", fast=fast, deck=d)
        out[key] = history(s, d["steps"], len(d["species"]))
        print(f"c1 ({'-Ofast' if fast else 'strict'}): {time.time() - t:.1f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "c1_weibel_history.npz"), **out)


def make_c5():
    d = CONFIG_DECKS["c5_lwfa"]
    nx, ny = d["nx"]
    s = build_cpu("c5_lwfa", backend="ref", deck=d)
    emf = np.zeros((d["steps"], 6))
    ex = {}
    t = time.time()
    for i in range(d["steps"]):
        s.iter()
        emf[i] = s.emf_energy()
        if i + 1 in C5_SNAPSHOTS:
            ex[f"ex_{i + 1}"] = s.E()[ny // 2 + 1, 1:nx + 1, 0].copy()
            print(f"c5 step {i + 1}: {time.time() - t:.0f} s, {s.np_(0)} particles", flush=True)
    np.savez_compressed(os.path.join(HERE, "c5_wake.npz"), emf=emf, np_end=s.np_(0), n_move=s.n_move(),
                        **ex)


def main():
    pyoracle.build()
    if not pyoracle.ref_available() or not pyoracle.ref_available(fast=True):
        sys.exit("reference build not available (oracle/_ref missing)")
    which = sys.argv[1:] or ["c1", "c5"]
    if "c1" in which:
        make_c1()
    if "c5" in which:
        make_c5()


if __name__ == "__main__":
    main()
