"""ctypes access to the reference em1d (oracle/_ref/libzpic_ref_em1d.so,
built by oracle/Makefile from the reference's own sources): the checker of
the 1-D GPU step.  TEST INFRASTRUCTURE ONLY."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libzpic_ref_em1d.so")
PART_DTYPE = np.dtype([("ix", "<i4"), ("x", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])
DENSITY = {"uniform": 0, "empty": 1, "step": 2, "slab": 3}
SMOOTH = {"none": 0, "binomial": 1, "compensated": 2}

_lib = None


def available():
    return os.path.exists(LIB)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    lib = C.CDLL(LIB)
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
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class RefSim1D:
    """A reference em1d simulation built from a deck dict (tests/decks_em1d.py)."""

    def __init__(self, deck):
        f = self.f = _load()
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
        for k in range(self.nspec):
            f.zr1_set_n_sort(self.h, k, 0)  # sorting only permutes the buffer
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
