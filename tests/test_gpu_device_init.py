"""Device-side loading (zc_species_create_device): positions are the
lattice spec_new places (bit-exact against the oracle for uniform, step and
slab profiles); momenta come from a counter-based generator, so they are
checked statistically: every cell's mean is the drift, the spread is uth,
the same seed repeats and another seed differs."""
import numpy as np
import pytest

from decks import DECKS, build_cpu
from gpu_util import canon

pytestmark = pytest.mark.gpu


def _positions(p):
    a = np.sort(np.rec.fromarrays([p["ix"], p["iy"], p["x"], p["y"]], names="ix,iy,x,y"), order=["ix", "iy", "x", "y"])
    return a


@pytest.mark.parametrize("name", ["thermal", "lwfa_window", "plane_slab", "weibel_smooth"])
def test_positions_match_spec_new(name):
    from zpic_gb300._zc import CudaSim

    d = DECKS[name]
    cpu = build_cpu(name)
    g = CudaSim(d["nx"], d["box"], d["dt"], tile=(16, 16))
    for k, sp in enumerate(d["species"]):
        dens = sp.get("density", {"type": "uniform"})
        kk = g.add_species_device(sp["m_q"], sp["ppc"], density=dens["type"], start=dens.get("start", 0.0),
                                  end=dens.get("end", 0.0), ufl=sp.get("ufl", (0, 0, 0)), uth=sp.get("uth", (0, 0, 0)),
                                  seed=100 + k)
        a, b = _positions(g.particles(kk)), _positions(cpu.particles(k))
        assert a.size == b.size
        assert a.tobytes() == b.tobytes()
        emf, kin = g.energy()
    g.close()


def test_momenta_statistics():
    from zpic_gb300._zc import CudaSim

    nx, ppc, uth, ufl = (96, 64), (4, 4), (0.05, 0.1, 0.02), (0.0, 0.0, 0.3)
    g = CudaSim(nx, (9.6, 6.4), 0.05, tile=(16, 16))
    k = g.add_species_device(-1.0, ppc, ufl=ufl, uth=uth, seed=7)
    p = g.particles(k)
    assert p.size == nx[0] * nx[1] * ppc[0] * ppc[1]
    cell = p["ix"].astype(np.int64) + nx[0] * p["iy"]
    order = np.argsort(cell, kind="stable")
    for c, (f, u0, s0) in enumerate(zip(("ux", "uy", "uz"), ufl, uth)):
        v = p[f][order].astype(np.float64).reshape(-1, ppc[0] * ppc[1])
        assert np.abs(v.mean(axis=1) - u0).max() < 1e-6
        # per-cell mean removed: the spread is (ppc-1)/ppc of the drawn one
        npc = ppc[0] * ppc[1]
        assert abs(v.std() / (s0 * np.sqrt((npc - 1) / npc)) - 1.0) < 0.02
    # the same seed repeats, another seed differs
    g2 = CudaSim(nx, (9.6, 6.4), 0.05, tile=(16, 16))
    k2 = g2.add_species_device(-1.0, ppc, ufl=ufl, uth=uth, seed=7)
    k3 = g2.add_species_device(-1.0, ppc, ufl=ufl, uth=uth, seed=8)
    assert canon(g2.particles(k2)).tobytes() == canon(p).tobytes()
    assert not np.array_equal(np.sort(g2.particles(k3)["ux"]), np.sort(p["ux"]))
    g.close()
    g2.close()


def test_device_loaded_plasma_steps():
    """A thermal plasma loaded on the device steps like the same lattice
    loaded from the host with the same momenta (the step itself is the same
    code path: fields agree to the forward bar)."""
    from zpic_gb300._zc import CudaSim

    d = DECKS["thermal"]
    g = CudaSim(d["nx"], d["box"], d["dt"], tile=(16, 16))
    k = g.add_species_device(-1.0, (4, 4), uth=(0.05, 0.05, 0.05), seed=3)
    parts = g.particles(k)
    h = CudaSim(d["nx"], d["box"], d["dt"], tile=(16, 16))
    h.add_species(-1.0, -1.0 / 16, (4, 4), parts)
    for s in (g, h):
        s.set_smooth("compensated", 1, "compensated", 1)
        s.step(10)
    from gpu_util import field_err
    for f in ("E", "B", "J"):
        assert field_err(g.__getattribute__(f)(), h.__getattribute__(f)()) <= 1e-5
    g.close()
    h.close()
