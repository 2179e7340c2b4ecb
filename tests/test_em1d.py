"""The em1d step on the GPU (zc1_*, zpic_gb300/em1d_gpu.py) and the C
restatement of the em1d step (oracle/zpic_oracle_em1d.c) against the
reference em1d: fixtures made by tests/golden/make_em1d_golden.py from the
reference compiled here, decks in tests/decks_em1d.py (periodic two-stream,
open boundaries with a laser and a slab, moving-window wakefield).

The laser's initial fields (zc1_add_laser) within 1e-6 of the reference's.
Per step: the particle counts equal, field and kinetic energies within
1e-5; after each of the first 10 steps E, B, J within 1e-5 relative L2 per
component (E and B measured on their common scale); after the last step the
window count equal and the fields within 1e-3 (long runs amplify
round-off)."""
import os

import numpy as np
import pytest

from decks_em1d import DECKS_1D, WIDE_1D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "em1d")
NAMES = sorted(DECKS_1D)


def _err(a, b, scale=None):
    """largest component-wise relative L2 error over the interior cells; a
    component below 1% of the field's scale (`scale`: the largest component
    norm, by default of `b` itself) is measured against 1% of that scale, so
    that fluctuation-level components (a magnetic field that is the curl of
    an almost uniform E) do not turn round-off into large relative errors"""
    a = np.asarray(a, dtype=np.float64)[1:-2]
    b = np.asarray(b, dtype=np.float64)[1:-2]
    norms = [np.linalg.norm(b[:, c]) for c in range(3)]
    floor = 1e-2 * (max(norms) if scale is None else scale)
    errs = []
    for c in range(3):
        na = np.linalg.norm(a[:, c] - b[:, c])
        errs.append(0.0 if norms[c] == 0 and na == 0 else na / max(norms[c], floor, 1e-30))
    return max(errs)


def _scale(*grids):
    return max(np.linalg.norm(np.asarray(g, dtype=np.float64)[1:-2, c]) for g in grids for c in range(3))


def test_fixtures_match_live_reference():
    """The committed fixtures are what the reference computes (first 10 steps)."""
    from oracle import pyoracle, pyoracle_em1d

    pyoracle.build()
    if not pyoracle_em1d.available():
        pytest.skip("reference em1d not built here")
    import subprocess
    import sys
    code = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
from decks_em1d import DECKS_1D, WIDE_1D
from oracle.pyoracle_em1d import RefSim1D
g = np.load({path!r})
s = RefSim1D(DECKS_1D[{name!r}])
assert s.particles(0).tobytes() == g["p0_0"].tobytes()
for step in range(10):
    s.iter()
    assert s.E().tobytes() == g["E_near"][step].tobytes(), step
    assert s.J().tobytes() == g["J_near"][step].tobytes(), step
print("OK")
"""
    for name in NAMES:
        r = subprocess.run([sys.executable, "-c", code.format(root=ROOT, tests=os.path.join(ROOT, "tests"),
                                                              path=os.path.join(GOLD, name + ".npz"), name=name)],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0 and "OK" in r.stdout, name + r.stdout[-2000:] + r.stderr[-2000:]


_CHILD_ORACLE = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
from decks_em1d import DECKS_1D, WIDE_1D
from oracle.pyoracle_em1d import RefSim1D
g = np.load({path!r})
d = DECKS_1D[{name!r}]
s = RefSim1D(d, backend="oracle")
assert s.particles(0).tobytes() == g["p0_0"].tobytes(), "loading"
assert s.E().tobytes() == g["E0"].tobytes() and s.B().tobytes() == g["B0"].tobytes(), "laser"
for step in range(d["steps"]):
    s.iter()
    if step < len(g["E_near"]):
        for f in "EBJ":
            assert getattr(s, f)().tobytes() == g[f + "_near"][step].tobytes(), (step, f)
    assert np.array_equal(s.emf_energy(), g["emf_energy"][step]), step
    for k in range(s.nspec):
        assert s.np_(k) == g["np"][step][k] and s.energy(k) == g["kin_energy"][step][k], (step, k)
for f in "EBJ":
    assert getattr(s, f)().tobytes() == g[f].tobytes(), f
print("OK")
"""


def _run_child(code):
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_fixtures(name):
    """The C restatement (oracle/zpic_oracle_em1d.c, strict IEEE build)
    reproduces the reference's fixtures bit for bit: the loaded particles,
    the laser, E/B/J after each of the first 10 steps and after the last,
    and the energies and particle counts of every step."""
    from oracle import pyoracle, pyoracle_em1d

    pyoracle.build()
    assert pyoracle_em1d.available("oracle")
    _run_child(_CHILD_ORACLE.format(root=ROOT, tests=os.path.join(ROOT, "tests"),
                                    path=os.path.join(GOLD, name + ".npz"), name=name))


_CHILD_SORTED = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
from decks_em1d import DECKS_1D, WIDE_1D
from oracle.pyoracle_em1d import RefSim1D
d = DECKS_1D[{name!r}]
s = RefSim1D(d, stock_sort=True, backend={backend!r})
for _ in range(d["steps"]):
    s.iter()
np.savez({out!r}, E=s.E(), J=s.J(), p=s.particles(0))
print("OK")
"""


def test_oracle_sort_matches_reference(tmp_path):
    """With the reference's stock sort (every 16 steps) the restatement and
    the reference leave the same particle order and fields (lwfa deck)."""
    from oracle import pyoracle, pyoracle_em1d

    pyoracle.build()
    if not pyoracle_em1d.available("ref"):
        pytest.skip("reference em1d not built here")
    out = {}
    for b in ("ref", "oracle"):
        out[b] = str(tmp_path / f"{b}.npz")
        _run_child(_CHILD_SORTED.format(root=ROOT, tests=os.path.join(ROOT, "tests"), name="lwfa", backend=b,
                                        out=out[b]))
    a, b = np.load(out["ref"]), np.load(out["oracle"])
    for k in a.files:
        assert a[k].tobytes() == b[k].tobytes(), k


def _mirror(d, g):
    from zpic_gb300.em1d_gpu import CudaSim1D

    sim = CudaSim1D(d["nx"], d["box"], d["dt"], open_fields=d.get("open_fields", False),
                    open_particles=d.get("open_particles", False), moving_window=d.get("moving_window", False))
    for k, sp in enumerate(d["species"]):
        dens = sp.get("density", {})
        sim.add_species(sp["m_q"], float(g["q"][k]), sp["ppc"], g[f"p0_{k}"], ufl=sp.get("ufl", (0, 0, 0)),
                        uth=sp.get("uth", (0, 0, 0)),
                        density=(dens.get("type", "uniform"), dens.get("start", 0.0), dens.get("end", 0.0)))
    if "laser" in d:
        L = d["laser"]
        sim.add_laser(L["start"], L["a0"], L["omega0"], fwhm=L["fwhm"], polarization=L.get("polarization", 0.0))
    else:
        sim.set_fields(g["E0"], g["B0"])
    if "smooth" in d:
        sim.set_smooth(d["smooth"]["type"], d["smooth"]["level"])
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if "laser" in DECKS_1D[n]])
def test_em1d_laser_matches_reference(name):
    """zc1_add_laser against the reference's emf_add_laser: the fields of the
    deck before the first step, guard cells included, within 1e-6 of the
    field's largest value (double cos on the device against the host's)"""
    g = np.load(os.path.join(GOLD, name + ".npz"))
    sim = _mirror(DECKS_1D[name], g)
    for f, ref in (("E", g["E0"]), ("B", g["B0"])):
        got = getattr(sim, f)()
        assert np.abs(ref).max() > 0
        assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max(), f
    sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_em1d_matches_reference(name):
    _check_run(DECKS_1D[name], np.load(os.path.join(GOLD, name + ".npz")))


_CHILD_WIDE = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}, {golden!r}]
import numpy as np
from decks_em1d import WIDE_1D
import make_em1d_golden
np.savez({out!r}, **make_em1d_golden.run({name!r}, WIDE_1D, backend="oracle"))
print("OK")
"""


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(WIDE_1D))
def test_em1d_wide_matches_oracle(name, tmp_path):
    """6000-cell grids, beyond the fields kernel's shared memory (its
    global-memory variant: periodic, open and moving-window boundaries),
    against the C restatement run live in a fresh process, same bars"""
    from oracle import pyoracle

    pyoracle.build()
    out = str(tmp_path / f"{name}.npz")
    _run_child(_CHILD_WIDE.format(root=ROOT, tests=os.path.join(ROOT, "tests"),
                                  golden=os.path.join(ROOT, "tests", "golden"), name=name, out=out))
    _check_run(WIDE_1D[name], np.load(out))


@pytest.mark.gpu
def test_em1d_async_side_by_side():
    """Two simulations stepped side by side (zc1_step_async on their own
    streams, interleaved) keep the fixtures' per-step bars; the device's
    pushed count equals the sum of the per-step counts."""
    runs = []
    for name in ("lwfa", "open_slab"):
        g = np.load(os.path.join(GOLD, name + ".npz"))
        runs.append((DECKS_1D[name], g, _mirror(DECKS_1D[name], g)))
    steps = min(d["steps"] for d, _, _ in runs)
    pushed_ref = [0, 0]
    for step in range(steps):
        for r, (d, g, sim) in enumerate(runs):
            pushed_ref[r] += int(g["np"][step - 1][0]) if step else int(len(g["p0_0"]))
            sim.step(1, wait=False)
        for d, g, sim in runs:
            sim.synchronize()
            emf, _ = sim.energy()
            ref = g["emf_energy"][step]
            assert np.all(np.abs(emf - ref) <= 1e-5 * max(np.abs(ref).max(), 1e-30) + 1e-12), step
            assert sim.count(0) == g["np"][step][0], step
    for r, (d, g, sim) in enumerate(runs):
        assert sim.pushed(0) == pushed_ref[r]
        sim.close()


def _check_run(d, g):
    sim = _mirror(d, g)
    ns = len(d["species"])
    for step in range(d["steps"]):
        sim.step(1)
        emf, kin = sim.energy()
        ref_emf = g["emf_energy"][step]
        scale = max(np.abs(ref_emf).max(), 1e-30)
        assert np.all(np.abs(emf - ref_emf) <= 1e-5 * scale + 1e-12), (step, emf, ref_emf)
        for k in range(ns):
            assert sim.count(k) == g["np"][step][k], (step, k)
            rk = g["kin_energy"][step][k]
            assert abs(kin[k] - rk) <= 1e-5 * abs(rk) + 1e-12, (step, k, kin[k], rk)
        if step < len(g["E_near"]):
            em = _scale(g["E_near"][step], g["B_near"][step])  # E and B share one scale
            for f, ref, sc in (("E", g["E_near"][step], em), ("B", g["B_near"][step], em),
                               ("J", g["J_near"][step], None)):
                err = _err(getattr(sim, f)(), ref, sc)
                assert err <= 1e-5, f"{f} relative error {err:.2e} at step {step}"
    assert sim.info()["n_move"] == g["n_move"][-1]
    em = _scale(g["E"], g["B"])
    for f in ("E", "B"):
        err = _err(getattr(sim, f)(), g[f], em)
        assert err <= 1e-3, f"{f} relative error {err:.2e} after {d['steps']} steps"
    sim.close()
