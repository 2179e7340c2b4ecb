"""ctypes access to the em1d checker libraries, the checker of the 1-D GPU
step.  TEST INFRASTRUCTURE ONLY.

* ``backend="ref"``    -- oracle/_ref/libzpic_ref_em1d.so: the reference em1d
  built by oracle/Makefile from its own sources (only where they exist);
* ``backend="oracle"`` -- oracle/liboracle_em1d.so: our C restatement
  (zpic_oracle_em1d.c), which builds anywhere.

Both export the same zr1_* entry points.  ``fast=True`` picks the build with
the reference's stock -Ofast flags (timing); the default strict IEEE build is
the one that reproduces the reference's bits."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PART_DTYPE = np.dtype([("ix", "<i4"), ("x", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])
DENSITY = {"uniform": 0, "empty": 1, "step": 2, "slab": 3}
SMOOTH = {"none": 0, "binomial": 1, "compensated": 2}

_libs = {}


def lib_path(backend="ref", fast=False):
    if backend == "ref":
        return os.path.join(HERE, "_ref", "libzpic_ref_em1d_fast.so" if fast else "libzpic_ref_em1d.so")
    return os.path.join(HERE, "liboracle_em1d_fast.so" if fast else "liboracle_em1d.so")


def available(backend="ref", fast=False):
    return os.path.exists(lib_path(backend, fast))


def _load(backend="ref", fast=False):
    path = lib_path(backend, fast)
    if path in _libs:
        return _libs[path]
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "zr1_set_rand_seed": (None, [C.c_uint32, C.c_uint32]),
        "zr1_sim_new": (P, [C.c_int, C.c_float, C.c_float]),
        "zr1_add_species": (C.c_int, [P, C.c_char_p, C.c_float, C.c_int, P, P, C.c_int, C.c_float, C.c_float,
                                      C.c_float]),
        "zr1_finalize": (None, [P]),
        "zr1_sim_delete": (None, [P]),
        "zr1_set_smooth": (None, [P, C.c_int, C.c_int]),
        "zr1_set_moving_window": (None, [P]),
        "zr1_set_open": (None, [P, C.c_int, C.c_int]),
        "zr1_add_laser": (None, [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
        "zr1_iter": (None, [P]),
        "zr1_spec_np": (C.c_int, [P, C.c_int]),
        "zr1_spec_q": (C.c_float, [P, C.c_int]),
        "zr1_spec_energy": (C.c_double, [P, C.c_int]),
        "zr1_n_move": (C.c_int, [P]),
        "zr1_set_n_sort": (None, [P, C.c_int, C.c_int]),
        "zr1_get_particles": (None, [P, C.c_int, P]),
        "zr1_get_E": (None, [P, P]),
        "zr1_get_B": (None, [P, P]),
        "zr1_get_J": (None, [P, P]),
        "zr1_emf_energy": (None, [P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _libs[path] = lib
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class RefSim1D:
    """A reference em1d simulation built from a deck dict (tests/decks_em1d.py)."""

    def __init__(self, deck, stock_sort=False, backend="ref", fast=False):
        f = self.f = _load(backend, fast)
        f.zr1_set_rand_seed(12345, 67890)
        self.nx = int(deck["nx"])
        self.h = f.zr1_sim_new(self.nx, float(deck["box"]), float(deck["dt"]))
        self.nspec = 0
        for sp in deck["species"]:
            ufl = np.asarray(sp.get("ufl", [0, 0, 0]), dtype=np.float32)
            uth = np.asarray(sp.get("uth", [0, 0, 0]), dtype=np.float32)
            d = sp.get("density", {})
            f.zr1_add_species(self.h, sp["name"].encode(), float(sp["m_q"]), int(sp["ppc"]), _p(ufl), _p(uth),
                              DENSITY[d.get("type", "uniform")], float(d.get("start", 0.0)),
                              float(d.get("end", 0.0)), float(d.get("n", 1.0)))
            self.nspec += 1
        f.zr1_finalize(self.h)
        if not stock_sort:
            # sorting only permutes the buffer; off for bit comparisons of the
            # particle records, on (every 16 steps, spec_new) for timing
            for k in range(self.nspec):
                f.zr1_set_n_sort(self.h, k, 0)
        if "laser" in deck:
            L = deck["laser"]
            f.zr1_add_laser(self.h, L["start"], L["fwhm"], L["a0"], L["omega0"], L.get("polarization", 0.0))
        if deck.get("moving_window"):
            f.zr1_set_moving_window(self.h)
        if deck.get("open_fields") or deck.get("open_particles"):
            f.zr1_set_open(self.h, int(bool(deck.get("open_fields"))), int(bool(deck.get("open_particles"))))
        if "smooth" in deck:
            s = deck["smooth"]
            f.zr1_set_smooth(self.h, SMOOTH[s["type"]], int(s["level"]))

    def iter(self):
        self.f.zr1_iter(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.f.zr1_sim_delete(self.h)
            self.h = None

    def np_(self, k):
        return int(self.f.zr1_spec_np(self.h, k))

    def q(self, k):
        return float(self.f.zr1_spec_q(self.h, k))

    def energy(self, k):
        return float(self.f.zr1_spec_energy(self.h, k))

    def n_move(self):
        return int(self.f.zr1_n_move(self.h))

    def particles(self, k):
        out = np.zeros(self.np_(k), dtype=PART_DTYPE)
        if len(out):
            self.f.zr1_get_particles(self.h, k, _p(out))
        return out

    def _grid(self, fn):
        out = np.zeros((self.nx + 3, 3), dtype=np.float32)
        fn(self.h, _p(out))
        return out

    def E(self):
        return self._grid(self.f.zr1_get_E)

    def B(self):
        return self._grid(self.f.zr1_get_B)

    def J(self):
        return self._grid(self.f.zr1_get_J)

    def emf_energy(self):
        out = np.zeros(6, dtype=np.float64)
        self.f.zr1_emf_energy(self.h, _p(out))
        return out
