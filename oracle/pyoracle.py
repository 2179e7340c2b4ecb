"""ctypes driver for the CPU checkers (TEST INFRASTRUCTURE ONLY).

Two interchangeable back ends share one Python class, ``CpuSim``:

* ``backend="oracle"``  -- ``oracle/liboracle.so``, the C restatement of the
  ZPIC em2d step (``oracle/zpic_oracle.c``), strict IEEE float32;
* ``backend="ref"``     -- ``oracle/_ref/libzpic_ref.so``, the reference em2d
  sources compiled unmodified by ``oracle/Makefile`` (only where the reference
  tree is present; never on machines without it).

``fast=True`` selects the ``-Ofast`` build of either (CPU timing baseline).
Only the tests, the smoke check and the CPU-baseline leg of ``bench.py`` use
this module; the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# root of the reference source tree (its em2d/, em1d/, python/ folders); the
# checker builds and the fixture generators read it there, nothing else does
REFERENCE_ROOT = os.environ.get("ZPIC_REFERENCE", "/root/reference")

PART_DTYPE = np.dtype([("ix", "<i4"), ("iy", "<i4"), ("x", "<f4"), ("y", "<f4"),
                       ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])

DENSITY_TYPES = {"uniform": 0, "empty": 1, "step": 2, "slab": 3, "custom": 4}
SMOOTH_TYPES = {"none": 0, "binomial": 1, "compensated": 2}
FLD_TYPES = {"none": 0, "uniform": 1, "custom": 2}
LASER_TYPES = {"plane": 0, "gaussian": 1}


class _F3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


DENS_FN = C.CFUNCTYPE(C.c_float, C.c_float, C.c_void_p)
FIELD_FN = C.CFUNCTYPE(None, C.c_int, C.c_float, C.c_int, C.c_float, C.c_void_p,
                       C.POINTER(C.c_float))


class _Density(C.Structure):
    _fields_ = [("n", C.c_float), ("type", C.c_int), ("start", C.c_float), ("end", C.c_float),
                ("custom_x", DENS_FN), ("custom_data_x", C.c_void_p),
                ("custom_y", DENS_FN), ("custom_data_y", C.c_void_p)]


class _Laser(C.Structure):
    _fields_ = [("type", C.c_int), ("start", C.c_float), ("fwhm", C.c_float), ("rise", C.c_float),
                ("flat", C.c_float), ("fall", C.c_float), ("a0", C.c_float), ("omega0", C.c_float),
                ("polarization", C.c_float), ("W0", C.c_float), ("focus", C.c_float),
                ("axis", C.c_float)]


def build(quiet: bool = True) -> None:
    """Compile the checker libraries with ``make`` (oracle always, _ref when
    the reference sources exist)."""
    out = subprocess.run(["make", "-C", HERE, "-j4", "all", f"ZPIC_REFERENCE={REFERENCE_ROOT}"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def ref_available(fast: bool = False) -> bool:
    name = "libzpic_ref_fast.so" if fast else "libzpic_ref.so"
    return os.path.exists(os.path.join(HERE, "_ref", name))


_LIBS: dict = {}


def _load(backend: str, fast: bool):
    key = (backend, fast)
    if key in _LIBS:
        return _LIBS[key]
    if backend == "oracle":
        path = os.path.join(HERE, "liboracle_fast.so" if fast else "liboracle.so")
        pre = "zo_"
    elif backend == "ref":
        path = os.path.join(HERE, "_ref", "libzpic_ref_fast.so" if fast else "libzpic_ref.so")
        pre = "zr_"
    else:
        raise ValueError(backend)
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "set_rand_seed": (None, [C.c_uint32, C.c_uint32]),
        "rand_norm": (C.c_double, []),
        "sim_add_species": (C.c_int, [P, C.c_char_p, C.c_float, P, P, P, P]),
        "sim_delete": (None, [P]),
        "sim_set_smooth": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int]),
        "sim_set_moving_window": (None, [P]),
        "sim_add_laser": (C.c_int, [P, P]),
        "sim_set_ext_fld": (C.c_int, [P, C.c_int, P, FIELD_FN, P, C.c_int, P, FIELD_FN, P]),
        "sim_init_fld": (C.c_int, [P, C.c_int, P, FIELD_FN, P, C.c_int, P, FIELD_FN, P]),
        "sim_iter": (None, [P]),
        "current_zero": (None, [P]),
        "spec_advance": (None, [P, C.c_int]),
        "current_update": (None, [P]),
        "emf_advance": (None, [P]),
        "nrow": (C.c_int, [P]),
        "buf_cells": (C.c_int, [P]),
        "n_species": (C.c_int, [P]),
        "spec_np": (C.c_int, [P, C.c_int]),
        "spec_q": (C.c_float, [P, C.c_int]),
        "spec_energy": (C.c_double, [P, C.c_int]),
        "spec_n_move": (C.c_int, [P, C.c_int]),
        "emf_n_move": (C.c_int, [P]),
        "emf_iter": (C.c_int, [P]),
        "get_particles": (None, [P, C.c_int, P]),
        "set_particles": (None, [P, C.c_int, P, C.c_int]),
        "get_E": (None, [P, P]), "get_B": (None, [P, P]), "get_J": (None, [P, P]),
        "get_E_part": (None, [P, P]), "get_B_part": (None, [P, P]),
        "set_E": (None, [P, P]), "set_B": (None, [P, P]), "set_J": (None, [P, P]),
        "emf_energy": (None, [P, P]),
        "spec_charge": (None, [P, C.c_int, P]),
        "spec_pha": (None, [P, C.c_int, C.c_int, C.c_int, P, P, P]),
    }
    fns = {}
    for name, (res, args) in sig.items():
        f = getattr(lib, pre + name)
        f.restype = res
        f.argtypes = args
        fns[name] = f
    if backend == "oracle":
        g = lib.zo_rand_fresh
        g.restype = None
        g.argtypes = []
        fns["rand_fresh"] = g
        f = lib.zo_sim_new
        f.restype = P
        f.argtypes = [P, P, C.c_float, C.c_char_p, C.c_int]
        fns["sim_new"] = f
    else:
        f = lib.zr_sim_new
        f.restype = P
        f.argtypes = [P, P, C.c_float]
        fns["sim_new"] = f
        for name, res, args in [("sim_finalize", None, [P]),
                                ("spec_set_n_sort", None, [P, C.c_int, C.c_int]),
                                ("spec_time", C.c_double, []),
                                ("spec_npush", C.c_double, []),
                                ("report_emf", None, [P, C.c_int, C.c_int]),
                                ("report_current", None, [P, C.c_int]),
                                ("report_spec", None, [P, C.c_int, C.c_int, P, P])]:
            g = getattr(lib, "zr_" + name)
            g.restype = res
            g.argtypes = args
            fns[name] = g
    _LIBS[key] = fns
    return fns


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class CpuSim:
    """One em2d simulation on the CPU checker.

    Species must all be added before the first setter/step call (the reference
    binds its species array in ``sim_new``); ``finalize`` is called implicitly.
    """

    def __init__(self, nx, box, dt, backend: str = "oracle", fast: bool = False):
        self.backend = backend
        self.f = _load(backend, fast)
        self.nx = [int(nx[0]), int(nx[1])]
        self.box = [float(box[0]), float(box[1])]
        self.dt = float(dt)
        self._nx = np.array(self.nx, dtype=np.int32)
        self._box = np.array(self.box, dtype=np.float32)
        self._keep = []
        if backend == "oracle":
            err = C.create_string_buffer(256)
            self.h = self.f["sim_new"](_ptr(self._nx), _ptr(self._box), self.dt, err, 256)
            if not self.h:
                raise ValueError(err.value.decode())
        else:
            self.h = self.f["sim_new"](_ptr(self._nx), _ptr(self._box), self.dt)
        self._final = backend == "oracle"

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.f["sim_delete"](h)
            self.h = None

    def _fin(self):
        if not self._final:
            self.f["sim_finalize"](self.h)
            self._final = True

    # ---- set-up ----
    def add_species(self, name, m_q, ppc, ufl=None, uth=None, density=None, n_sort=0):
        """``density``: None or dict(type=..., n=..., start=..., end=...,
        custom_x=callable, custom_y=callable)."""
        assert not self._final or self.backend == "oracle", "add species before stepping"
        ppc_a = np.array(ppc, dtype=np.int32)
        ufl_a = None if ufl is None else np.array(ufl, dtype=np.float32)
        uth_a = None if uth is None else np.array(uth, dtype=np.float32)
        self._keep += [ppc_a, ufl_a, uth_a]
        dptr = None
        if density is not None:
            d = _Density()
            d.n = float(density.get("n", 1.0))
            d.type = DENSITY_TYPES[density.get("type", "uniform")]
            d.start = float(density.get("start", 0.0))
            d.end = float(density.get("end", 0.0))
            for ax in ("x", "y"):
                fn = density.get("custom_" + ax)
                if fn is not None:
                    cb = DENS_FN(lambda v, _d, fn=fn: float(fn(v)))
                    self._keep.append(cb)
                    setattr(d, "custom_" + ax, cb)
            self._keep.append(d)
            dptr = C.cast(C.pointer(d), C.c_void_p)
        k = self.f["sim_add_species"](self.h, name.encode(), float(m_q), _ptr(ppc_a),
                                      None if ufl_a is None else _ptr(ufl_a),
                                      None if uth_a is None else _ptr(uth_a), dptr)
        if self.backend == "ref":
            self.f["spec_set_n_sort"](self.h, k, int(n_sort))
        return k

    def set_smooth(self, xtype="none", xlevel=0, ytype="none", ylevel=0):
        self._fin()
        return self.f["sim_set_smooth"](self.h, SMOOTH_TYPES[xtype], int(xlevel),
                                        SMOOTH_TYPES[ytype], int(ylevel))

    def set_moving_window(self):
        self._fin()
        self.f["sim_set_moving_window"](self.h)

    def add_laser(self, type="plane", start=0.0, fwhm=0.0, rise=0.0, flat=0.0, fall=0.0,
                  a0=0.0, omega0=0.0, polarization=0.0, W0=0.0, focus=0.0, axis=0.0):
        self._fin()
        L = _Laser(LASER_TYPES[type], start, fwhm, rise, flat, fall, a0, omega0, polarization,
                   W0, focus, axis)
        return self.f["sim_add_laser"](self.h, C.cast(C.pointer(L), C.c_void_p))

    def _fld_args(self, typ, val, fn):
        t = FLD_TYPES[typ]
        v = None if val is None else np.array(val, dtype=np.float32)
        if fn is not None:
            def cb(ix, dx, iy, dy, _d, out, fn=fn):
                r = fn(ix, dx, iy, dy)
                out[0], out[1], out[2] = float(r[0]), float(r[1]), float(r[2])
            c = FIELD_FN(cb)
        else:
            c = FIELD_FN()
        self._keep += [v, c]
        return t, (None if v is None else _ptr(v)), c

    def set_ext_fld(self, E_type="none", E_0=None, E_custom=None,
                    B_type="none", B_0=None, B_custom=None):
        self._fin()
        a = self._fld_args(E_type, E_0, E_custom)
        b = self._fld_args(B_type, B_0, B_custom)
        return self.f["sim_set_ext_fld"](self.h, a[0], a[1], a[2], None, b[0], b[1], b[2], None)

    def init_fld(self, E_type="none", E_0=None, E_custom=None,
                 B_type="none", B_0=None, B_custom=None):
        self._fin()
        a = self._fld_args(E_type, E_0, E_custom)
        b = self._fld_args(B_type, B_0, B_custom)
        return self.f["sim_init_fld"](self.h, a[0], a[1], a[2], None, b[0], b[1], b[2], None)

    # ---- stepping ----
    def iter(self, n: int = 1):
        self._fin()
        for _ in range(n):
            self.f["sim_iter"](self.h)

    def current_zero(self):
        self._fin(); self.f["current_zero"](self.h)

    def spec_advance(self, k):
        self._fin(); self.f["spec_advance"](self.h, k)

    def current_update(self):
        self._fin(); self.f["current_update"](self.h)

    def emf_advance(self):
        self._fin(); self.f["emf_advance"](self.h)

    # ---- data ----
    @property
    def n_species(self):
        return self.f["n_species"](self.h)

    def np_(self, k):
        return self.f["spec_np"](self.h, k)

    def q(self, k):
        return self.f["spec_q"](self.h, k)

    def energy(self, k):
        return self.f["spec_energy"](self.h, k)

    def n_move(self):
        return self.f["emf_n_move"](self.h)

    def particles(self, k) -> np.ndarray:
        out = np.zeros(self.np_(k), dtype=PART_DTYPE)
        if out.size:
            self.f["get_particles"](self.h, k, _ptr(out))
        return out

    def set_particles(self, k, parts: np.ndarray):
        parts = np.ascontiguousarray(parts, dtype=PART_DTYPE)
        self.f["set_particles"](self.h, k, _ptr(parts), int(parts.size))

    def _grid(self, name) -> np.ndarray:
        """Full buffer incl. guard cells, shape (ny+3, nx+3, 3)."""
        out = np.zeros((self.nx[1] + 3, self.nx[0] + 3, 3), dtype=np.float32)
        self.f[name](self.h, _ptr(out))
        return out

    def E(self):
        return self._grid("get_E")

    def B(self):
        return self._grid("get_B")

    def J(self):
        return self._grid("get_J")

    def E_part(self):
        return self._grid("get_E_part")

    def B_part(self):
        return self._grid("get_B_part")

    def _set_grid(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(self.nx[1] + 3, self.nx[0] + 3, 3)
        self.f[name](self.h, _ptr(a))

    def set_E(self, a):
        self._fin(); self._set_grid("set_E", a)

    def set_B(self, a):
        self._fin(); self._set_grid("set_B", a)

    def set_J(self, a):
        self._fin(); self._set_grid("set_J", a)

    def emf_energy(self) -> np.ndarray:
        out = np.zeros(6, dtype=np.float64)
        self.f["emf_energy"](self.h, _ptr(out))
        return out

    def charge(self, k) -> np.ndarray:
        out = np.zeros((self.nx[1] + 1, self.nx[0] + 1), dtype=np.float32)
        self.f["spec_charge"](self.h, k, _ptr(out))
        return out

    PHA = {"x1": 1, "x2": 2, "u1": 4, "u2": 5, "u3": 6}

    def phasespace(self, k, quants, pha_nx, pha_range) -> np.ndarray:
        n = np.ascontiguousarray(pha_nx, dtype=np.int32)
        r = np.ascontiguousarray(np.asarray(pha_range, dtype=np.float32).reshape(4))
        out = np.zeros((int(n[1]), int(n[0])), dtype=np.float32)
        self.f["spec_pha"](self.h, k, self.PHA[quants[0]], self.PHA[quants[1]], _ptr(n), _ptr(r), _ptr(out))
        return out


def _report_methods():
    def report_emf(self, field, fc):
        """The reference's emf_report (field 0..3: E, B, E_part, B_part),
        written below the current directory (reference back end only)."""
        self.f["report_emf"](self.h, int(field), int(fc))

    def report_current(self, jc):
        self.f["report_current"](self.h, int(jc))

    def report_spec(self, k, rep_type, pha_nx=(0, 0), pha_range=((0, 0), (0, 0))):
        n = np.ascontiguousarray(pha_nx, dtype=np.int32)
        r = np.ascontiguousarray(np.asarray(pha_range, dtype=np.float32).reshape(4))
        self.f["report_spec"](self.h, int(k), int(rep_type), _ptr(n), _ptr(r))

    return report_emf, report_current, report_spec


CpuSim.report_emf, CpuSim.report_current, CpuSim.report_spec = _report_methods()


def set_rand_seed(w=12345, z=67890, backend="oracle", fast=False, fresh=False):
    """Seeds the process-global generator of a back end.  ``fresh=True`` (oracle
    only) also drops the cached Box-Muller deviate, i.e. the state of a newly
    started process."""
    f = _load(backend, fast)
    f["set_rand_seed"](w, z)
    if fresh:
        if backend != "oracle":
            raise ValueError("only the oracle can reset its Box-Muller cache")
        f["rand_fresh"]()
