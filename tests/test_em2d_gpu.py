"""The em2d Python API (zpic_gb300.em2d, the reference's Cython class
interface) on the GPU against the CPU oracle: every deck, 10 steps, per-step
field relative L2 error <= 1e-5 (each field as a whole; each component
within 1e-5 or within twice the oracle's own drift when its particles are
summed in another order), same particle counts, energies within 1e-5.  Each
deck runs in a fresh process (both generators are process-global)."""
import os
import subprocess
import sys

import pytest

from decks import DECKS

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_CHILD = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
from decks import DECKS, _resolve, build_cpu
from gpu_util import field_err_components, field_err_joint, reordered_twin
from zpic_gb300 import em2d

name = {name!r}
d = DECKS[name]
em2d.gpu_options(fast_math={fast!r})

def density(sp):
    if "density" not in sp:
        return None
    r = _resolve(sp["density"])
    return em2d.Density(type=r.get("type", "uniform"), n=r.get("n", 1.0), start=r.get("start", 0.0),
                        end=r.get("end", 0.0), custom_x=r.get("custom_x"), custom_y=r.get("custom_y"))

species = [em2d.Species(sp["name"], sp["m_q"], sp["ppc"], ufl=sp.get("ufl", [0, 0, 0]),
                        uth=sp.get("uth", [0, 0, 0]), density=density(sp)) for sp in d["species"]]
kw = {{}}
for key, cls in (("init_fld", em2d.InitialField), ("ext_fld", em2d.ExternalField)):
    if key in d:
        r = _resolve(d[key])
        kw[key] = cls(E_type=r.get("E_type", "none"), B_type=r.get("B_type", "none"), E_0=r.get("E_0"),
                      B_0=r.get("B_0"), E_custom=r.get("E_custom"), B_custom=r.get("B_custom"))
sim = em2d.Simulation(d["nx"], d["box"], d["dt"], species=species, **kw)
if "laser" in d:
    sim.add_laser(em2d.Laser(**d["laser"]))
if d.get("moving_window"):
    sim.set_moving_window()
if "smooth" in d:
    sim.set_smooth(em2d.Smooth(**d["smooth"]))

cpu = build_cpu(name)
# the reordered twin shares the oracle's process-wide generator, which a
# moving window draws from every step: only the other decks get one
twin = None if d.get("moving_window") else reordered_twin(name)
for k in range(len(species)):
    a = np.sort(species[k].particles.copy(), order=["iy", "ix", "y", "x"])
    b = np.sort(cpu.particles(k), order=["iy", "ix", "y", "x"])
    assert a.tobytes() == b.tobytes(), "initial particles"
steps = 40 if d.get("moving_window") else 10
for n in range(steps):
    sim.iter()
    cpu.iter()
    if twin is not None:
        twin.iter()
    for k in range(len(species)):
        assert species[k].particles.size == cpu.np_(k), (n, k)
        assert abs(species[k].energy - cpu.energy(k)) <= 1e-5 * abs(cpu.energy(k)) + 1e-12
    E = np.stack([sim.emf.Ex, sim.emf.Ey, sim.emf.Ez], -1)
    B = np.stack([sim.emf.Bx, sim.emf.By, sim.emf.Bz], -1)
    Ec, Bc = cpu.E()[1:-2, 1:-2], cpu.B()[1:-2, 1:-2]
    pad = lambda a: np.pad(a, ((1, 2), (1, 2), (0, 0)))
    bar = 1e-5 if n < 10 else 1e-4
    for g, c, f in ((E, Ec, "E"), (B, Bc, "B")):
        full = cpu.E() if f == "E" else cpu.B()
        assert field_err_joint(pad(g), pad(c)) <= bar, (f, n, field_err_joint(pad(g), pad(c)))
        err = field_err_components(pad(g), pad(c))
        floor = field_err_components(getattr(twin, f)(), full) if twin is not None else np.zeros(3)
        for comp in range(3):
            assert err[comp] <= max(bar, 2 * floor[comp]), (f, comp, n, err[comp], floor[comp])
    en = sim.emf.energy
    assert np.allclose(en, cpu.emf_energy(), rtol=1e-4, atol=1e-12), n
assert sim.n_move == cpu.n_move()
print("OK")
"""


@pytest.mark.parametrize("name", sorted(DECKS))
def test_em2d_api_matches_oracle(name):
    code = _CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), name=name, fast=False)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]


def test_em2d_species_edit_reaches_gpu():
    """Edits through Species.particles / Species.add are sent to the GPU."""
    code = f"""
import sys
sys.path[:0] = [{ROOT!r}]
import numpy as np
from zpic_gb300 import em2d
sp = em2d.Species("e", -1.0, [2, 2], uth=[0.01, 0.01, 0.01])
sim = em2d.Simulation([32, 32], [3.2, 3.2], 0.05, species=sp)
sim.iter()
n0 = sp.particles.size
sp.add([3, 4], [0.25, 0.5], [0.0, 0.5, 0.0])
p = sp.particles
p["uz"][:] = 0.0
sim.iter()
p = sp.particles
assert p.size == n0 + 1
assert np.abs(p["uz"]).max() < 0.05
print("OK")
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
