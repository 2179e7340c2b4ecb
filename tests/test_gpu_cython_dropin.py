"""The reference's own Cython em2d module, unmodified, driving the drop-in on
the GPU (built by ``oracle/cython_em2d.py``; skipped where it was not built).

A Weibel deck set up through the module's classes, as the reference's Python
users write it, is compared with the oracle:

* the initial particles read through ``Species.particles`` equal the
  oracle's (the drop-in loads them with the reference's generator);
* after every one of 10 ``Simulation.iter()`` calls, ``EMF.Ex`` ... and
  ``Current.Jz`` -- numpy views of the structs' host buffers, taken once
  before the first step -- follow the oracle per component within 1e-5
  relative L2, and ``Species.particles`` holds the oracle's particles
  (positions within 1e-4 of a cell);
* edits made through the particle view and ``Species.add`` between steps
  reach the GPU, as they reach the reference's own buffers.
"""
import ctypes
import os

import numpy as np
import pytest

from decks import build_cpu
from gpu_util import canon

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def em2d():
    from oracle import cython_em2d

    cython_em2d.compile()
    mod = cython_em2d.load()
    if mod is None:
        pytest.skip("the reference's Cython module was not built here (needs its sources and Cython at build)")
    return mod


def _interior(a):
    return np.asarray(a, dtype=np.float64)[1:-2, 1:-2]


def _rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb else float(np.linalg.norm(a))


def _fresh_generator():
    # the module seeds the reference's generator itself (em2d.pyx:1781); a
    # Box-Muller deviate cached by earlier runs in this thread is dropped
    # first, as a fresh process would start
    lib = ctypes.CDLL(os.path.join(ROOT, "zpic_gb300", "lib", "libzpic_em2d.so"))
    lib.rand_seed_fresh.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    lib.rand_seed_fresh(12345, 67890)


def _positions(p):
    c = canon(p)
    return c["ix"] + c["x"].astype(np.float64), c["iy"] + c["y"].astype(np.float64)


def test_reference_cython_module_on_gpu(em2d):
    _fresh_generator()
    species = [em2d.Species("e1", -1.0, [2, 2], ufl=[0.0, 0.0, 0.6], uth=[0.1, 0.1, 0.1]),
               em2d.Species("e2", -1.0, [2, 2], ufl=[0.0, 0.0, -0.6], uth=[0.1, 0.1, 0.1])]
    smooth = em2d.Smooth(xtype="compensated", xlevel=2, ytype="binomial", ylevel=1)
    sim = em2d.Simulation([32, 24], [3.2, 2.4], 0.07, species=species, smooth=smooth)
    cpu = build_cpu("weibel_smooth")

    for k in range(2):
        got = np.asarray(species[k].particles)
        want = cpu.particles(k)
        assert got.size == want.size
        for f in ("ix", "iy", "x", "y", "ux", "uy", "uz"):
            assert np.array_equal(got[f], want[f]), f

    views = {"E": [sim.emf.Ex, sim.emf.Ey, sim.emf.Ez], "B": [sim.emf.Bx, sim.emf.By, sim.emf.Bz],
             "J": [sim.current.Jx, sim.current.Jy, sim.current.Jz]}
    for step in range(10):
        sim.iter()
        cpu.iter()
        for f, vs in views.items():
            ref = _interior(getattr(cpu, f)())
            for c, v in enumerate(vs):
                err = _rel(np.asarray(v, dtype=np.float64), ref[..., c])
                assert err <= 1e-5, f"{f}{'xyz'[c]} relative error {err:.2e} at step {step}"
        for k in range(2):
            got, want = _positions(np.asarray(species[k].particles)), _positions(cpu.particles(k))
            assert got[0].size == want[0].size
            assert np.abs(got[0] - want[0]).max() < 1e-4 and np.abs(got[1] - want[1]).max() < 1e-4

    # edits between steps: halve the momenta of species 0 through the view,
    # add a particle to species 1 with Species.add, on both sides
    p = species[0].particles
    p["ux"] *= 0.5
    p["uz"] *= 0.5
    q = cpu.particles(0)
    q["ux"] *= 0.5
    q["uz"] *= 0.5
    cpu.set_particles(0, q)
    species[1].add(np.array([3, 4], dtype=np.int32), np.array([0.25, 0.75], dtype=np.float32),
                   np.array([0.1, -0.2, 0.3], dtype=np.float32))
    r = cpu.particles(1)
    extra = np.zeros(1, dtype=r.dtype)
    extra[0] = (3, 4, 0.25, 0.75, 0.1, -0.2, 0.3)
    cpu.set_particles(1, np.concatenate([r, extra]))
    for step in range(3):
        sim.iter()
        cpu.iter()
    for k in range(2):
        assert np.asarray(species[k].particles).size == cpu.np_(k)
    ref = _interior(cpu.E())
    for c, v in enumerate(views["E"]):
        assert _rel(np.asarray(v, dtype=np.float64), ref[..., c]) <= 1e-5, "E after edits"
    del sim
