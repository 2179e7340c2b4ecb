"""The benchmark configurations against the reference, at their own sizes.

* Weibel instability (128^2, two electron streams, 4x4 ppc, 524,288
  particles, 500 steps): the first 10 steps against the oracle run live, each
  field (E, B, J) within 1e-5 relative L2 and each component within 1e-5 or,
  for Ez and Jz, where the streams' currents cancel, within twice the drift
  of the oracle against itself with its particles reordered (the float32
  floor of any other summation order: 2.6e-5 by step 10); then the whole 500-step
  run against the reference's own energy history (``tests/golden/
  c1_weibel_history.npz``, made by ``make_config_golden.py`` from the
  reference compiled from its sources): the growth rate of the in-plane
  magnetic energy (Bx^2 + By^2) fitted over the exponential phase, the
  saturated level, and the field, magnetic and kinetic energies at every step,
  each within 2 %.
* The 2048^2 thermal throughput workload on a 256^2 box of the same cell size,
  time step, density, ppc and smoothing: 10 steps against the oracle, per
  field component within 1e-5.
* Moving-window laser wakefield (2000 x 256, 3000 steps, 2099 window moves):
  the on-axis Ex wake against the reference's (``tests/golden/c5_wake.npz``)
  after 1000, 2000 and 3000 steps: the wake amplitude (largest |Ex| behind the
  laser) within 2 %.

Every check runs for the exact push build and for the fast build (FMA
contraction, approximate division and square root) that the throughput
figures use.
"""
import os

import numpy as np
import pytest

from decks import CONFIG_DECKS, build_cpu
from gpu_util import check_fields, field_err, mirror, reordered_twin

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BUILDS = pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])

# exponential phase of the Weibel deck's in-plane magnetic energy (steps):
# it grows from 0.3 % to 11 % of its saturated level there, by a factor of
# about 3.6 every 25 steps, in the reference's history
C1_FIT = (100, 160)


def _bperp(h):
    return h[:, 3] + h[:, 4]


def _growth_rate(h, dt):
    """Field growth rate: half the slope of log(Bx^2 + By^2 energy) against
    time over the exponential phase (least squares)."""
    a, b = C1_FIT
    t = dt * np.arange(a, b + 1)
    slope = np.polyfit(t, np.log(_bperp(h)[a:b + 1]), 1)[0]
    return 0.5 * slope


def _first_steps(name, fast, tile, per_component):
    d = CONFIG_DECKS[name]
    cpu, g = mirror(name, deck=d, cpu=build_cpu(name, deck=d), tile=tile, fast_math=fast)
    twin = reordered_twin(name, deck=d)
    try:
        for step in range(10):
            cpu.iter()
            twin.iter()
            g.step(1)
            check_fields(g, cpu, twin, f"at step {step}")
            if per_component:
                for f in ("E", "B", "J"):
                    err = field_err(getattr(g, f)(), getattr(cpu, f)())
                    assert err <= 1e-5, f"{f} relative error {err:.2e} (worst component) at step {step}"
            emf_g, kin_g = g.energy()
            emf_c = cpu.emf_energy()
            assert np.all(np.abs(emf_g - emf_c) <= 1e-5 * np.abs(emf_c)), step
            for k in range(cpu.n_species):
                assert abs(kin_g[k] - cpu.energy(k)) <= 1e-5 * abs(cpu.energy(k))
                assert g.count(k) == cpu.np_(k)
    finally:
        g.close()


@BUILDS
def test_c1_weibel_first_steps(fast):
    # the two streams' z currents cancel cell by cell: Ez and Jz move by up
    # to 2.6e-5 when only the order of the oracle's own sums changes, so
    # those two components are held to the reordering floor
    _first_steps("c1_weibel", fast, (16, 16), per_component=False)


@BUILDS
def test_c2_thermal_box_first_steps(fast):
    # every component within 1e-5, both push builds
    _first_steps("c2_thermal_256", fast, (32, 16), per_component=True)


@BUILDS
def test_c1_weibel_500_steps_against_reference(fast):
    d = CONFIG_DECKS["c1_weibel"]
    ref = np.load(os.path.join(GOLDEN, "c1_weibel_history.npz"))["hist"]
    steps = d["steps"]
    cpu = build_cpu("c1_weibel", deck=d)
    _, g = mirror("c1_weibel", deck=d, cpu=cpu, tile=(16, 16), fast_math=fast)
    try:
        g.set_graphs(True)
        g.history_enable(steps)
        g.step(steps)
        hist = g.history()
    finally:
        g.close()
    assert hist.shape == (steps, 8)
    gpu = np.vstack([ref[:1], hist])  # row 0: the shared initial state

    gam_ref, gam = _growth_rate(ref, d["dt"]), _growth_rate(gpu, d["dt"])
    assert abs(gam / gam_ref - 1) <= 0.02, f"growth rate {gam:.5f} against {gam_ref:.5f}"
    sat_ref, sat = _bperp(ref)[300:].mean(), _bperp(gpu)[300:].mean()
    assert abs(sat / sat_ref - 1) <= 0.02, f"saturated magnetic energy {sat:.4f} against {sat_ref:.4f}"
    rows = slice(1, steps + 1)
    for what, f in (("field", lambda h: h[:, :6].sum(1)), ("magnetic", _bperp),
                    ("kinetic", lambda h: h[:, 6:].sum(1)), ("total", lambda h: h.sum(1))):
        r = np.abs(f(gpu)[rows] / f(ref)[rows] - 1)
        assert r.max() <= 0.02, f"{what} energy off by {r.max():.3e} at step {int(r.argmax()) + 1}"


def _c5_run(fast):
    """The wakefield deck on the GPU: the reference's initial particles and
    laser fields (from the oracle), the window's new column drawn on the
    device, blocks of steps replayed as graphs (the throughput set-up)."""
    from zpic_gb300._zc import CudaSim

    d = CONFIG_DECKS["c5_lwfa"]
    nx, ny = d["nx"]
    cpu = build_cpu("c5_lwfa", deck=d)
    g = CudaSim(d["nx"], d["box"], d["dt"], tile=(32, 16), fast_math=fast)
    sp = d["species"][0]
    g.add_species(sp["m_q"], cpu.q(0), sp["ppc"], cpu.particles(0))
    g.set_fields(E=cpu.E(), B=cpu.B())
    del cpu
    g.set_moving_window()
    g.set_device_injector(0, "step", start=sp["density"]["start"])
    g.set_graphs(True)
    g.set_smooth(**d["smooth"])
    ex = {}
    done = 0
    try:
        for s in (1000, 2000, 3000):
            g.step(s - done)
            done = s
            ex[s] = g.E()[ny // 2 + 1, 1:nx + 1, 0].astype(np.float64)
        count, moves = g.count(0), g.info()["n_move"]
    finally:
        g.close()
    return ex, count, moves


@BUILDS
def test_c5_wake_against_reference(fast):
    ref = np.load(os.path.join(GOLDEN, "c5_wake.npz"))
    ex, count, moves = _c5_run(fast)
    assert moves == int(ref["n_move"])
    assert abs(count / int(ref["np_end"]) - 1) <= 1e-3
    # the wake: cells behind the laser (x < 15 of the 40-long window)
    wake = slice(0, 750)
    for s in (1000, 2000, 3000):
        a, b = ex[s][wake], ref[f"ex_{s}"].astype(np.float64)[wake]
        amp, amp_ref = np.abs(a).max(), np.abs(b).max()
        assert abs(amp / amp_ref - 1) <= 0.02, f"wake amplitude {amp:.4f} against {amp_ref:.4f} after {s} steps"
