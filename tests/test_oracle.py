"""The CPU oracle against the reference: golden vectors (always) and the
reference compiled from its own sources (where the reference tree exists).

Every comparison here is bit-exact: the oracle restates the reference's
float32 arithmetic operation by operation and both are built with strict
IEEE flags (no fast-math, no FMA contraction)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from decks import DECKS, build_cpu
from oracle import pyoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    pyoracle.build()


@pytest.mark.parametrize("name", sorted(DECKS))
def test_oracle_matches_golden(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = DECKS[name]
    s = build_cpu(name, backend="oracle")
    ns = len(d["species"])
    for k in range(ns):
        assert s.particles(k).tobytes() == g[f"p0_{k}"].tobytes(), f"initial particles of species {k}"
    for step in range(d["steps"]):
        s.iter()
        assert np.array_equal(s.emf_energy(), g["emf_energy"][step]), f"field energy at step {step}"
        for k in range(ns):
            assert s.np_(k) == g["np"][step][k]
            assert s.energy(k) == g["kin_energy"][step][k], f"kinetic energy at step {step}"
    assert s.E().tobytes() == g["E"].tobytes()
    assert s.B().tobytes() == g["B"].tobytes()
    assert s.J().tobytes() == g["J"].tobytes()
    for k in range(ns):
        assert s.particles(k).tobytes() == g[f"p_{k}"].tobytes()


_CHILD = r"""
import sys, numpy as np
sys.path[:0] = [{root!r}, {tests!r}]
from decks import DECKS, build_cpu
name = {name!r}
d = DECKS[name]
a = build_cpu(name, backend="oracle")
b = build_cpu(name, backend="ref")
ns = len(d["species"])
for step in range(d["steps"] + 10):
    for k in range(ns):
        assert a.particles(k).tobytes() == b.particles(k).tobytes(), (step, k)
    for g in ("E", "B", "J", "E_part", "B_part"):
        assert getattr(a, g)().tobytes() == getattr(b, g)().tobytes(), (step, g)
    a.current_zero(); b.current_zero()
    for k in range(ns):
        a.spec_advance(k); b.spec_advance(k)
        assert a.energy(k) == b.energy(k)
    assert a.J().tobytes() == b.J().tobytes(), (step, "J after deposit")
    a.current_update(); b.current_update()
    assert a.J().tobytes() == b.J().tobytes(), (step, "J after update")
    a.emf_advance(); b.emf_advance()
    assert np.array_equal(a.emf_energy(), b.emf_energy())
    assert a.n_move() == b.n_move()
for k in range(ns):
    assert np.array_equal(a.charge(k), b.charge(k))
    for qs, rg in ((("x1", "u1"), ((0.0, 4.0), (-0.5, 0.5))), (("x2", "u3"), ((0.0, 3.0), (-1.0, 1.0))),
                   (("u1", "u2"), ((-0.3, 0.3), (-0.3, 0.3)))):
        assert np.array_equal(a.phasespace(k, qs, (32, 24), rg), b.phasespace(k, qs, (32, 24), rg))
print("OK")
"""


@pytest.mark.skipif(not pyoracle.ref_available() and not os.path.isdir(os.path.join(pyoracle.REFERENCE_ROOT, "em2d")),
                    reason="reference sources not present on this machine")
@pytest.mark.parametrize("name", sorted(DECKS))
def test_oracle_matches_reference_phase_by_phase(name):
    """Each phase of sim_iter (deposit, current update, field advance) is
    compared separately against the reference, in a fresh process because the
    reference keeps its generator state in process globals."""
    if not pyoracle.ref_available():
        pytest.skip("oracle/_ref not built")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = _CHILD.format(root=root, tests=os.path.join(root, "tests"), name=name)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_rand_norm_sequence_matches_reference():
    if not pyoracle.ref_available():
        pytest.skip("oracle/_ref not built")
    code = (f"import sys; sys.path.insert(0, {os.path.dirname(os.path.dirname(os.path.abspath(__file__)))!r})\n"
            "from oracle import pyoracle as P\n"
            "a = P._load('oracle', False); b = P._load('ref', False)\n"
            "a['set_rand_seed'](777, 4242); b['set_rand_seed'](777, 4242)\n"
            "xs = [a['rand_norm']() for _ in range(10001)]; ys = [b['rand_norm']() for _ in range(10001)]\n"
            "assert xs == ys\nprint('OK')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_courant_violation_is_rejected():
    with pytest.raises(ValueError, match="courant"):
        pyoracle.CpuSim([16, 16], [1.6, 1.6], 0.2)


def test_oracle_deposit_conserves_charge():
    """The oracle's deposit satisfies discrete continuity (the property the
    full-size GPU test checks at 67M particles)."""
    import continuity
    from decks import DECKS, build_cpu

    d = dict(DECKS["thermal"])
    d.pop("smooth")
    cpu = build_cpu("thermal", deck=d)
    nx, ny = d["nx"]
    dx = np.float32(d["box"][0]) / np.float32(nx)
    dy = np.float32(d["box"][1]) / np.float32(ny)
    rho0 = cpu.charge(0)
    cpu.current_zero()
    cpu.spec_advance(0)
    res, dmax = continuity.residual(rho0, cpu.charge(0), cpu.J(), nx, ny, dx, dy, np.float32(d["dt"]))
    assert dmax > 1e-3 and res < 2e-6, (res, dmax)
