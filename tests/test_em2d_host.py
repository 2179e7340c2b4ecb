"""The host side of the em2d drop-in layer (libzpic_em2d), without a GPU:
particle loading against the oracle (bit-exact), the generator, and the C
struct layouts seen by the Python module."""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from decks import DECKS, _resolve
from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def em2d():
    from zpic_gb300 import build

    build.build()
    pyoracle.build()
    from zpic_gb300 import em2d as m

    return m


def _host_species(m, deck, k):
    """spec_new of the drop-in library on a stand-alone t_species."""
    lib = m._load()
    sp = deck["species"][k]
    ts = m.t_species()
    dens = None
    keep = []
    if "density" in sp:
        d = _resolve(sp["density"])
        dd = m.Density(type=d.get("type", "uniform"), n=d.get("n", 1.0), start=d.get("start", 0.0),
                       end=d.get("end", 0.0), custom_x=d.get("custom_x"), custom_y=d.get("custom_y"))
        keep.append(dd)
        dens = C.byref(dd._d)
    arr = lambda v, t: np.ascontiguousarray(v, dtype=t)
    ppc = arr(sp["ppc"], np.int32)
    ufl = arr(sp.get("ufl", [0, 0, 0]), np.float32)
    uth = arr(sp.get("uth", [0, 0, 0]), np.float32)
    nx = arr(deck["nx"], np.int32)
    box = arr(deck["box"], np.float32)
    keep += [ppc, ufl, uth, nx, box]
    lib.spec_new(C.byref(ts), sp["name"].encode(), sp["m_q"], m._ptr(ppc), m._ptr(ufl), m._ptr(uth),
                 m._ptr(nx), m._ptr(box), deck["dt"], dens)
    parts = np.frombuffer((m.t_part * ts.np).from_address(C.addressof(ts.part.contents)),
                          dtype=m.PART_DTYPE).copy() if ts.np else np.zeros(0, dtype=m.PART_DTYPE)
    return parts, ts.q


_CHILD = r"""
import sys
sys.path[:0] = [{root!r}, {tests!r}]
import numpy as np
from decks import DECKS, build_cpu
from test_em2d_host import _host_species
from zpic_gb300 import em2d as m
name = {name!r}
d = DECKS[name]
m._load().set_rand_seed(12345, 67890)
cpu = build_cpu(name)   # the oracle, seeded the same way
for k in range(len(d["species"])):
    p, q = _host_species(m, d, k)
    assert p.tobytes() == cpu.particles(k).tobytes(), k
    assert q == cpu.q(k)
print("OK")
"""


@pytest.mark.parametrize("name", sorted(DECKS))
def test_spec_new_matches_oracle(em2d, name):
    """spec_new draws the same particles as the reference (fresh process:
    the generator is process-global in both)."""
    code = _CHILD.format(root=ROOT, tests=os.path.join(ROOT, "tests"), name=name)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_generator_matches_oracle(em2d):
    code = (f"import sys; sys.path[:0] = [{ROOT!r}]\n"
            "import ctypes as C\n"
            "from zpic_gb300 import em2d as m\n"
            "from oracle import pyoracle as P\n"
            "lib = m._load(); lib.rand_norm.restype = C.c_double\n"
            "o = P._load('oracle', False)\n"
            "lib.set_rand_seed(4321, 8765); o['set_rand_seed'](4321, 8765)\n"
            "a = [lib.rand_norm() for _ in range(20001)]; b = [o['rand_norm']() for _ in range(20001)]\n"
            "assert a == b\nprint('OK')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


def test_struct_layouts_match_headers(em2d):
    """The ctypes structures of the Python module against the C headers
    (sizes and field offsets, from a program compiled here)."""
    fields = {
        "t_species": ["part", "np", "m_q", "energy", "q", "density", "ufl", "nx", "dt", "iter", "n_move",
                      "n_sort"],
        "t_density": ["n", "type", "custom_x", "custom_x_total_part", "custom_x_total_q"],
        "t_emf": ["E_buf", "B_buf", "nx", "nrow", "dx", "iter", "n_move", "ext_fld"],
        "t_current": ["J_buf", "nx", "smooth", "iter"],
        "t_simulation": ["dt", "n_species", "species", "emf", "current", "moving_window"],
        "t_emf_laser": ["type", "a0", "axis"],
        "t_emf_ext_fld": ["E_0", "B_custom", "E_part_buf"],
    }
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "simulation.h"', "int main(void){"]
    for t, fs in fields.items():
        src.append(f'printf("{t} %zu\\n", sizeof({t}));')
        for f in fs:
            src.append(f'printf("{t}.{f} %zu\\n", offsetof({t}, {f}));')
    src.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "lay.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(d, "lay")
        subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include", "em2d"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(line.split() for line in out if line)
    for t, fs in fields.items():
        cls = getattr(em2d, t)
        assert int(got[t]) == C.sizeof(cls), t
        for f in fs:
            assert int(got[f"{t}.{f}"]) == getattr(cls, f).offset, f"{t}.{f}"
