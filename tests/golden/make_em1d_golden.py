"""Generate the 1-D fixtures in tests/golden/em1d/ from the REFERENCE em1d
itself (oracle/_ref/libzpic_ref_em1d.so, built by oracle/Makefile from the
reference's own sources), one fresh process per deck of tests/decks_em1d.py.

Per deck: the initial particles of every species and the initial E, B (the
laser included), the field energies, kinetic energies and particle counts
after every step, E, B, J after each of the first 10 steps, and E, B, J plus
the window count after the last step.  The reference's sort is disabled
(sorting only permutes its buffer).

Usage (where the reference tree and a C compiler are present)::

    python tests/golden/make_em1d_golden.py [deck ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from decks_em1d import DECKS_1D  # noqa: E402
from oracle import pyoracle, pyoracle_em1d  # noqa: E402

NEAR = 10


def run(name, decks=DECKS_1D, backend="ref"):
    """the fixture arrays of deck `name` of `decks`, on the reference
    (backend "ref") or on the C restatement (backend "oracle")"""
    d = decks[name]
    s = pyoracle_em1d.RefSim1D(d, backend=backend)
    ns = s.nspec
    out = {"q": np.array([s.q(k) for k in range(ns)], dtype=np.float32)}
    for k in range(ns):
        out[f"p0_{k}"] = s.particles(k)
    out["E0"], out["B0"] = s.E(), s.B()
    emf, kin, npart, nmove, near = [], [], [], [], {"E": [], "B": [], "J": []}
    for step in range(d["steps"]):
        s.iter()
        emf.append(s.emf_energy())
        kin.append([s.energy(k) for k in range(ns)])
        npart.append([s.np_(k) for k in range(ns)])
        nmove.append(s.n_move())
        if step < NEAR:
            near["E"].append(s.E())
            near["B"].append(s.B())
            near["J"].append(s.J())
    out["emf_energy"] = np.array(emf)
    out["kin_energy"] = np.array(kin)
    out["np"] = np.array(npart, dtype=np.int64)
    out["n_move"] = np.array(nmove, dtype=np.int64)
    for f in ("E", "B", "J"):
        out[f + "_near"] = np.array(near[f])
    out["E"], out["B"], out["J"] = s.E(), s.B(), s.J()
    return out


def main():
    pyoracle.build()
    if not pyoracle_em1d.available():
        sys.exit("reference em1d build not available (oracle/_ref missing)")
    os.makedirs(HERE + "/em1d", exist_ok=True)
    for name in sys.argv[1:] or list(DECKS_1D):
        if os.fork() == 0:
            np.savez_compressed(os.path.join(HERE, "em1d", f"{name}.npz"), **run(name))
            os._exit(0)
        _, st = os.wait()
        if st != 0:
            sys.exit(f"deck {name} failed")
        print("wrote", name)


if __name__ == "__main__":
    main()
