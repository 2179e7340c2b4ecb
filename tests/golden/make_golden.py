"""Generate the golden vectors in this directory from the REFERENCE itself.

Runs the unmodified reference em2d (compiled from its own sources into
``oracle/_ref/libzpic_ref.so`` by ``oracle/Makefile``, strict IEEE build) on
every deck of ``tests/decks.py`` and stores, per deck:

* the initial particles of every species (the reference's own ``spec_new``);
* the field energies (6 components) and kinetic energy of every species after
  every step;
* after the last step: E, B, J buffers (with guard cells) and the particles.

Usage (where the reference tree and a C compiler are present)::

    python tests/golden/make_golden.py [deck ...]   # default: every deck

The reference's ``spec_sort`` is disabled (``n_sort=0``) so that particle
buffer order is comparable; sorting only permutes the buffer.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from decks import DECKS, build_cpu  # noqa: E402
from oracle import pyoracle  # noqa: E402


def run(name):
    d = DECKS[name]
    s = build_cpu(name, backend="ref")
    out = {}
    for k in range(len(d["species"])):
        out[f"p0_{k}"] = s.particles(k)
    emf_hist, kin_hist, np_hist = [], [], []
    for _ in range(d["steps"]):
        s.iter()
        emf_hist.append(s.emf_energy())
        kin_hist.append([s.energy(k) for k in range(len(d["species"]))])
        np_hist.append([s.np_(k) for k in range(len(d["species"]))])
    out["emf_energy"] = np.array(emf_hist)
    out["kin_energy"] = np.array(kin_hist)
    out["np"] = np.array(np_hist, dtype=np.int64)
    out["E"] = s.E()
    out["B"] = s.B()
    out["J"] = s.J()
    for k in range(len(d["species"])):
        out[f"p_{k}"] = s.particles(k)
    return out


def main():
    pyoracle.build()
    if not pyoracle.ref_available():
        sys.exit("reference build not available (oracle/_ref missing)")
    names = sys.argv[1:] or list(DECKS)
    for name in names:
        # the reference keeps its generator in process globals: one fresh
        # process per deck
        if os.fork() == 0:
            out = run(name)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
            os._exit(0)
        _, st = os.wait()
        if st != 0:
            sys.exit(f"deck {name} failed")
        print("wrote", name)


if __name__ == "__main__":
    main()
