"""ctypes binding of libzpic_cuda (include/zpic_cuda.h).

``CudaSim`` is a thin object wrapper over the C-ABI: one handle, numpy arrays
in the reference layouts in and out.  Every failing call raises
``ZcError`` with the library's message.  There is no fallback: if the CUDA
library cannot be loaded, importing the simulation objects fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libzpic_cuda.so")

PART_DTYPE = np.dtype([("ix", "<i4"), ("iy", "<i4"), ("x", "<f4"), ("y", "<f4"),
                       ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])

STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error",
          4: "particle escaped its cell", 5: "device wait timed out", 6: "particle overflow",
          7: "invalid state"}

SMOOTH = {"none": 0, "binomial": 1, "compensated": 2}
FLD = {"none": 0, "uniform": 1, "custom": 2}
LASER = {"plane": 0, "gaussian": 1}

# every symbol include/zpic_cuda.h declares
EXPORTS = [
    "zc_sim_create", "zc_sim_destroy", "zc_species_create", "zc_species_set_particles",
    "zc_species_inject", "zc_species_get_particles", "zc_species_count", "zc_set_injector",
    "zc_set_smooth", "zc_set_moving_window", "zc_add_laser", "zc_set_ext_fld", "zc_step",
    "zc_current_zero", "zc_spec_advance", "zc_current_update", "zc_emf_advance", "zc_set_fields",
    "zc_get_fields", "zc_get_particle_fields", "zc_get_current", "zc_set_current", "zc_energy", "zc_energy_async",
    "zc_species_charge", "zc_get_info", "zc_grid_view_get", "zc_synchronize", "zc_last_step_ms", "zc_step_async", "zc_history_stream",
    "zc_last_error", "zc_status_string", "zc_set_profiling", "zc_get_profile", "zc_reset_profile",
    "zc_phase_name", "zc_field_energy_static", "zc_set_graphs", "zc_history_enable", "zc_history_get",
    "zc_history_reset", "zc_batch_create", "zc_batch_step", "zc_batch_last_ms", "zc_batch_destroy",
    "zc_batch_set_groups", "zc_batch_get_groups",
    "zc_adj_create", "zc_adj_destroy", "zc_adj_set_state", "zc_adj_forward", "zc_adj_backward",
    "zc_adj_get_state", "zc_adj_times", "zc_species_phasespace", "zc_species_create_device",
    "zc_adj_set_birth", "zc_adj_set_smooth", "zc_copy_grid_async", "zc_fence_wait", "zc_fence_destroy",
    "zc_host_alloc", "zc_host_free", "zc1_create", "zc1_destroy", "zc1_add_species", "zc1_set_smooth",
    "zc1_set_fields", "zc1_get_fields", "zc1_get_current", "zc1_step", "zc1_energy", "zc1_species_count",
    "zc1_get_particles", "zc1_get_info", "zc1_synchronize", "zc1_add_laser", "zc1_last_step_ms",
    "zc1_get_launches", "zc1_set_profile", "zc1_get_profile", "zc1_step_async", "zc1_species_pushed",
    "zc_set_device_injection", "zc_post_device_error",
]
NPHASE = 13


class ZcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class SimDesc(C.Structure):
    _fields_ = [("nx", C.c_int * 2), ("box", C.c_float * 2), ("dt", C.c_float), ("device", C.c_int),
                ("tile", C.c_int * 2), ("deterministic", C.c_int), ("tile_slack", C.c_float),
                ("fast_math", C.c_int), ("sort_every", C.c_int)]


class AdjDesc(C.Structure):
    _fields_ = [("nx", C.c_int * 2), ("box", C.c_double * 2), ("dt", C.c_double), ("q", C.c_double),
                ("m_q", C.c_double), ("np", C.c_int), ("checkpoint_every", C.c_int), ("precision", C.c_int),
                ("device", C.c_int), ("moving_window", C.c_int), ("objective", C.c_int), ("objective_row", C.c_int),
                ("objective_cells", C.c_int * 2)]


class Density(C.Structure):
    _fields_ = [("type", C.c_int), ("n", C.c_float), ("start", C.c_float), ("end", C.c_float)]


DENSITY = {"uniform": 0, "empty": 1, "step": 2, "slab": 3}


class SpeciesDesc(C.Structure):
    _fields_ = [("m_q", C.c_float), ("q", C.c_float), ("ppc", C.c_int * 2)]


class Laser(C.Structure):
    _fields_ = [("type", C.c_int), ("start", C.c_float), ("fwhm", C.c_float), ("rise", C.c_float),
                ("flat", C.c_float), ("fall", C.c_float), ("a0", C.c_float), ("omega0", C.c_float),
                ("polarization", C.c_float), ("W0", C.c_float), ("focus", C.c_float),
                ("axis", C.c_float)]


class ColumnProfile(C.Structure):
    _fields_ = [("type", C.c_int), ("start", C.c_float), ("end", C.c_float), ("ufl", C.c_float * 3)]


class Info(C.Structure):
    _fields_ = [("iter", C.c_int), ("n_move", C.c_int), ("moving_window", C.c_int),
                ("n_species", C.c_int), ("nx", C.c_int * 2), ("tile", C.c_int * 2),
                ("ntiles", C.c_int * 2), ("relayouts", C.c_int), ("captures", C.c_int)]


class GridView(C.Structure):
    _fields_ = [("E", C.c_void_p), ("B", C.c_void_p), ("J", C.c_void_p), ("plane", C.c_size_t),
                ("pitch", C.c_int), ("rows", C.c_int), ("stream", C.c_void_p)]


INJECT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p),
                        C.POINTER(C.c_int))

_lib = None


def load(path: str = LIB_PATH):
    """Loads libzpic_cuda (building it first when absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _b
        _b.build()
    lib = C.CDLL(path)
    P = C.c_void_p
    I = C.c_int
    sig = {
        "zc_sim_create": [C.POINTER(SimDesc), C.POINTER(P)],
        "zc_sim_destroy": [P],
        "zc_species_create": [P, C.POINTER(SpeciesDesc), P, I, C.POINTER(I)],
        "zc_species_set_particles": [P, I, P, I],
        "zc_species_inject": [P, I, P, I],
        "zc_species_get_particles": [P, I, P, I, C.POINTER(I)],
        "zc_species_count": [P, I, C.POINTER(I)],
        "zc_set_injector": [P, INJECT_FN, P],
        "zc_set_smooth": [P, I, I, I, I],
        "zc_set_moving_window": [P],
        "zc_add_laser": [P, C.POINTER(Laser)],
        "zc_set_ext_fld": [P, I, P, P, I, P, P],
        "zc_step": [P, I],
        "zc_post_device_error": [P, I],
        "zc_current_zero": [P],
        "zc_spec_advance": [P, I],
        "zc_current_update": [P],
        "zc_emf_advance": [P],
        "zc_set_fields": [P, P, P],
        "zc_get_fields": [P, P, P],
        "zc_get_particle_fields": [P, P, P],
        "zc_get_current": [P, P],
        "zc_set_current": [P, P],
        "zc_energy": [P, P, P],
        "zc_energy_async": [P, P, P],
        "zc_species_charge": [P, I, P],
        "zc_get_info": [P, C.POINTER(Info)],
        "zc_grid_view_get": [P, C.POINTER(GridView)],
        "zc_synchronize": [P],
        "zc_step_async": [P, I],
        "zc_history_stream": [P, P, I],
        "zc_last_step_ms": [P, C.POINTER(C.c_float)],
        "zc_set_profiling": [P, I],
        "zc_get_profile": [P, P, P],
        "zc_reset_profile": [P],
        "zc_field_energy_static": [P, P, C.c_size_t, I, I, I, C.c_float, C.c_float, P, P],
        "zc_set_graphs": [P, I],
        "zc_history_enable": [P, I],
        "zc_history_get": [P, P, I, C.POINTER(I), C.POINTER(I)],
        "zc_history_reset": [P],
        "zc_batch_create": [P, I, C.POINTER(P)],
        "zc_batch_step": [P, I],
        "zc_batch_set_groups": [P, I],
        "zc_batch_get_groups": [P, C.POINTER(I)],
        "zc_batch_last_ms": [P, C.POINTER(C.c_float)],
        "zc_batch_destroy": [P],
        "zc_adj_create": [C.POINTER(AdjDesc), C.POINTER(P)],
        "zc_adj_destroy": [P],
        "zc_adj_set_state": [P] + [P] * 10,
        "zc_adj_forward": [P, I, P, P],
        "zc_adj_backward": [P] + [P] * 8,
        "zc_adj_get_state": [P] + [P] * 10,
        "zc_adj_set_birth": [P, P],
        "zc_adj_set_smooth": [P, I, P, P],
        "zc_adj_times": [P, C.POINTER(C.c_float), C.POINTER(C.c_float)],
        "zc_species_phasespace": [P, I, I, I, P, P, P],
        "zc_species_create_device": [P, C.c_float, P, C.POINTER(Density), P, P, C.c_ulonglong, C.POINTER(I)],
        "zc_copy_grid_async": [P, I, I, P, C.POINTER(P)],
        "zc_fence_wait": [P],
        "zc_host_alloc": [C.c_size_t, C.POINTER(P)],
        "zc1_create": [P, C.POINTER(P)],
        "zc1_add_species": [P, P, P, I, C.POINTER(I)],
        "zc1_set_smooth": [P, I, I],
        "zc1_set_fields": [P, P, P],
        "zc1_get_fields": [P, P, P],
        "zc1_get_current": [P, P],
        "zc1_step": [P, I],
        "zc1_energy": [P, P, P],
        "zc1_species_count": [P, I, C.POINTER(I)],
        "zc1_get_particles": [P, I, P, I, C.POINTER(I)],
        "zc1_get_info": [P, C.POINTER(I), C.POINTER(I)],
        "zc1_synchronize": [P],
        "zc1_add_laser": [P, P],
        "zc1_last_step_ms": [P, C.POINTER(C.c_float)],
        "zc1_get_launches": [P, C.POINTER(C.c_longlong)],
        "zc1_step_async": [P, I],
        "zc_set_device_injection": [P, I, P],
        "zc1_species_pushed": [P, I, C.POINTER(C.c_longlong)],
        "zc1_set_profile": [P, I],
        "zc1_get_profile": [P, P, P],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = I
    for name in ("zc_fence_destroy", "zc_host_free", "zc1_destroy"):
        getattr(lib, name).argtypes = [P]
        getattr(lib, name).restype = None
    lib.zc_last_error.restype = C.c_char_p
    lib.zc_last_error.argtypes = []
    lib.zc_status_string.restype = C.c_char_p
    lib.zc_status_string.argtypes = [I]
    lib.zc_phase_name.restype = C.c_char_p
    lib.zc_phase_name.argtypes = [I]
    _lib = lib
    return lib


def _ck(status):
    if status != 0:
        raise ZcError(status, _lib.zc_last_error().decode())


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class CudaSim:
    """One em2d simulation on the GPU (a ``zc_sim`` handle)."""

    def __init__(self, nx, box, dt, device=0, tile=(16, 16), deterministic=False, tile_slack=0.5,
                 fast_math=False, sort_every=0):
        self.lib = load()
        d = SimDesc()
        d.nx[0], d.nx[1] = int(nx[0]), int(nx[1])
        d.box[0], d.box[1] = float(box[0]), float(box[1])
        d.dt = float(dt)
        d.device = int(device)
        d.tile[0], d.tile[1] = int(tile[0]), int(tile[1])
        d.deterministic = int(bool(deterministic))
        d.tile_slack = float(tile_slack)
        d.fast_math = int(bool(fast_math))
        d.sort_every = int(sort_every)
        h = C.c_void_p()
        _ck(self.lib.zc_sim_create(C.byref(d), C.byref(h)))
        self.h = h
        self.nx = [int(nx[0]), int(nx[1])]
        self.box = [float(box[0]), float(box[1])]
        self.dt = float(dt)
        self.n_species = 0
        self._inj = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.zc_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- species ----
    def add_species(self, m_q, q, ppc, particles: np.ndarray) -> int:
        parts = np.ascontiguousarray(particles, dtype=PART_DTYPE)
        d = SpeciesDesc(float(m_q), float(q), (C.c_int * 2)(int(ppc[0]), int(ppc[1])))
        k = C.c_int()
        _ck(self.lib.zc_species_create(self.h, C.byref(d), _p(parts), int(parts.size), C.byref(k)))
        self.n_species += 1
        return k.value

    def add_species_device(self, m_q, ppc, density="uniform", start=0.0, end=0.0, n=1.0, ufl=(0, 0, 0),
                           uth=(0, 0, 0), seed=0) -> int:
        """Loads a species on the device: the ppc lattice inside the density
        profile, thermal momenta from a counter-based generator."""
        d = Density(DENSITY[density], float(n), float(start), float(end))
        pp = np.ascontiguousarray(ppc, dtype=np.int32)
        uf = np.ascontiguousarray(ufl, dtype=np.float32)
        ut = np.ascontiguousarray(uth, dtype=np.float32)
        k = C.c_int()
        _ck(self.lib.zc_species_create_device(self.h, float(m_q), _p(pp), C.byref(d), _p(uf), _p(ut), int(seed),
                                              C.byref(k)))
        self.n_species += 1
        return k.value

    def set_particles(self, k, particles):
        parts = np.ascontiguousarray(particles, dtype=PART_DTYPE)
        _ck(self.lib.zc_species_set_particles(self.h, int(k), _p(parts), int(parts.size)))

    def inject(self, k, particles):
        parts = np.ascontiguousarray(particles, dtype=PART_DTYPE)
        _ck(self.lib.zc_species_inject(self.h, int(k), _p(parts), int(parts.size)))

    def count(self, k) -> int:
        n = C.c_int()
        _ck(self.lib.zc_species_count(self.h, int(k), C.byref(n)))
        return n.value

    def particles(self, k) -> np.ndarray:
        n = self.count(k)
        out = np.zeros(n, dtype=PART_DTYPE)
        m = C.c_int()
        _ck(self.lib.zc_species_get_particles(self.h, int(k), _p(out), n, C.byref(m)))
        return out[: m.value]

    def set_injector(self, fn):
        """``fn(species, n_move) -> structured particle array`` for the column
        injected when the window moves."""
        keep = {}

        def cb(_user, species, n_move, out_ptr, out_n):
            try:
                arr = np.ascontiguousarray(fn(species, n_move), dtype=PART_DTYPE)
                keep["a"] = arr
                out_ptr[0] = arr.ctypes.data
                out_n[0] = int(arr.size)
                return 0
            except Exception:  # pragma: no cover - reported as a status code
                import traceback
                traceback.print_exc()
                return 1

        self._inj = (INJECT_FN(cb), keep)
        _ck(self.lib.zc_set_injector(self.h, self._inj[0], None))

    def set_device_injector(self, species, density="uniform", start=0.0, end=0.0, ufl=(0.0, 0.0, 0.0)):
        """window injection drawn on the device for a cold species: density
        "uniform", "empty", "step" (start) or "slab" (start, end)"""
        types = {"uniform": 0, "empty": 1, "step": 2, "slab": 3}
        prof = ColumnProfile(types[density], float(start), float(end), (C.c_float * 3)(*ufl))
        _ck(self.lib.zc_set_device_injection(self.h, int(species), C.byref(prof)))

    # ---- configuration ----
    def set_smooth(self, xtype="none", xlevel=0, ytype="none", ylevel=0):
        _ck(self.lib.zc_set_smooth(self.h, SMOOTH[xtype], int(xlevel), SMOOTH[ytype], int(ylevel)))

    def set_moving_window(self):
        _ck(self.lib.zc_set_moving_window(self.h))

    def add_laser(self, type="plane", start=0.0, fwhm=0.0, rise=0.0, flat=0.0, fall=0.0, a0=0.0,
                  omega0=0.0, polarization=0.0, W0=0.0, focus=0.0, axis=0.0):
        L = Laser(LASER[type], start, fwhm, rise, flat, fall, a0, omega0, polarization, W0, focus, axis)
        _ck(self.lib.zc_add_laser(self.h, C.byref(L)))

    def set_ext_fld(self, E_type="none", E_0=None, E_grid=None, B_type="none", B_0=None, B_grid=None):
        args = []
        keep = []
        for t, v, g in ((E_type, E_0, E_grid), (B_type, B_0, B_grid)):
            va = None if v is None else np.ascontiguousarray(v, dtype=np.float32)
            ga = None if g is None else np.ascontiguousarray(g, dtype=np.float32)
            keep += [va, ga]
            args += [FLD[t], None if va is None else _p(va), None if ga is None else _p(ga)]
        _ck(self.lib.zc_set_ext_fld(self.h, *args))

    # ---- stepping ----
    def step(self, n=1):
        _ck(self.lib.zc_step(self.h, int(n)))

    iter = step

    def step_async(self, n=1):
        """Queues n steps and returns without waiting (errors come back from
        the next waiting call, e.g. ``synchronize()``)."""
        _ck(self.lib.zc_step_async(self.h, int(n)))

    def current_zero(self):
        _ck(self.lib.zc_current_zero(self.h))

    def spec_advance(self, k):
        _ck(self.lib.zc_spec_advance(self.h, int(k)))

    def current_update(self):
        _ck(self.lib.zc_current_update(self.h))

    def emf_advance(self):
        _ck(self.lib.zc_emf_advance(self.h))

    def synchronize(self):
        _ck(self.lib.zc_synchronize(self.h))

    def last_ms(self) -> float:
        v = C.c_float()
        _ck(self.lib.zc_last_step_ms(self.h, C.byref(v)))
        return v.value

    # ---- data (reference layouts) ----
    def _shape(self):
        return (self.nx[1] + 3, self.nx[0] + 3, 3)

    def E(self):
        a = np.zeros(self._shape(), dtype=np.float32)
        _ck(self.lib.zc_get_fields(self.h, _p(a), None))
        return a

    def B(self):
        a = np.zeros(self._shape(), dtype=np.float32)
        _ck(self.lib.zc_get_fields(self.h, None, _p(a)))
        return a

    def E_part(self):
        a = np.zeros(self._shape(), dtype=np.float32)
        _ck(self.lib.zc_get_particle_fields(self.h, _p(a), None))
        return a

    def B_part(self):
        a = np.zeros(self._shape(), dtype=np.float32)
        _ck(self.lib.zc_get_particle_fields(self.h, None, _p(a)))
        return a

    def J(self):
        a = np.zeros(self._shape(), dtype=np.float32)
        _ck(self.lib.zc_get_current(self.h, _p(a)))
        return a

    def set_fields(self, E=None, B=None):
        Ea = None if E is None else np.ascontiguousarray(E, dtype=np.float32).reshape(self._shape())
        Ba = None if B is None else np.ascontiguousarray(B, dtype=np.float32).reshape(self._shape())
        _ck(self.lib.zc_set_fields(self.h, None if Ea is None else _p(Ea), None if Ba is None else _p(Ba)))

    def set_J(self, J):
        a = np.ascontiguousarray(J, dtype=np.float32).reshape(self._shape())
        _ck(self.lib.zc_set_current(self.h, _p(a)))

    def energy(self):
        """(field energy per component [6], kinetic energy per species)."""
        emf = np.zeros(6, dtype=np.float64)
        kin = np.zeros(max(self.n_species, 1), dtype=np.float64)
        _ck(self.lib.zc_energy(self.h, _p(emf), _p(kin)))
        return emf, kin[: self.n_species]

    def energy_async(self, out):
        """Queues the energies into ``out`` (float64, 6 + n_species: the
        field components, then the kinetic energy of every species) and
        returns at once; ``out`` holds them after ``synchronize()``.  Use
        page-locked memory for ``out`` to keep the copies asynchronous."""
        if out.dtype != np.float64 or out.size < 6 + self.n_species or not out.flags.c_contiguous:
            raise ValueError("out: contiguous float64 array of 6 + n_species values")
        kin = out[6:] if self.n_species else None
        _ck(self.lib.zc_energy_async(self.h, _p(out), _p(kin) if kin is not None else None))

    def charge(self, k, out=None):
        rho = np.zeros((self.nx[1] + 1, self.nx[0] + 1), dtype=np.float32) if out is None else out
        _ck(self.lib.zc_species_charge(self.h, int(k), _p(rho)))
        return rho

    PHA = {"x1": 1, "x2": 2, "u1": 4, "u2": 5, "u3": 6}

    def phasespace(self, k, quants, pha_nx, pha_range, out=None):
        """Phase-space density [pha_nx[1], pha_nx[0]] of species k
        (quants e.g. ("x1", "u1"), pha_range ((x1min, x1max), (x2min, x2max)))."""
        n = np.ascontiguousarray(pha_nx, dtype=np.int32)
        r = np.ascontiguousarray(np.asarray(pha_range, dtype=np.float32).reshape(4))
        buf = np.zeros((int(n[1]), int(n[0])), dtype=np.float32) if out is None else out
        _ck(self.lib.zc_species_phasespace(self.h, int(k), self.PHA[quants[0]], self.PHA[quants[1]], _p(n), _p(r),
                                           _p(buf)))
        return buf

    def info(self):
        i = Info()
        _ck(self.lib.zc_get_info(self.h, C.byref(i)))
        return {"iter": i.iter, "n_move": i.n_move, "moving_window": i.moving_window,
                "n_species": i.n_species, "tile": (i.tile[0], i.tile[1]),
                "ntiles": (i.ntiles[0], i.ntiles[1]), "relayouts": i.relayouts, "captures": i.captures}

    def set_profiling(self, on=True):
        """Per-phase device timing: True (or 1) every phase, "push" (2) the
        push only (the rest of the step runs untimed), False off."""
        mode = 2 if on == "push" else int(bool(on))
        _ck(self.lib.zc_set_profiling(self.h, mode))

    def reset_profile(self):
        _ck(self.lib.zc_reset_profile(self.h))

    def profile(self):
        """{phase: (device ms, kernel launches)} summed since the last reset."""
        ms = np.zeros(NPHASE, dtype=np.float64)
        nl = np.zeros(NPHASE, dtype=np.int64)
        _ck(self.lib.zc_get_profile(self.h, _p(ms), _p(nl)))
        return {self.lib.zc_phase_name(k).decode(): (float(ms[k]), int(nl[k])) for k in range(NPHASE)}

    def grid_view(self):
        v = GridView()
        _ck(self.lib.zc_grid_view_get(self.h, C.byref(v)))
        return v

    def set_graphs(self, on=True):
        """Replays whole blocks of steps as one captured CUDA graph."""
        _ck(self.lib.zc_set_graphs(self.h, int(bool(on))))

    def history_enable(self, max_steps):
        """Records the field and kinetic energies after every step on the
        device (up to ``max_steps`` rows)."""
        _ck(self.lib.zc_history_enable(self.h, int(max_steps)))

    def history_stream(self, rows):
        """Every step writes its energy row (6 field components, then the
        kinetic energy of every species) into ``rows``: page-locked float64
        host memory of shape (max_steps, 6 + n_species), e.g. from
        ``torch.empty(..., pin_memory=True)``.  ``None`` turns it off."""
        if rows is None:
            _ck(self.lib.zc_history_stream(self.h, None, 0))
            return
        if rows.dtype != np.float64 or rows.ndim != 2 or rows.shape[1] != 6 + self.n_species \
                or not rows.flags.c_contiguous:
            raise ValueError("rows: contiguous float64 (max_steps, 6 + n_species)")
        self._stream_rows = rows  # kept alive while the device writes into it
        _ck(self.lib.zc_history_stream(self.h, _p(rows), rows.shape[0]))

    def history_reset(self):
        _ck(self.lib.zc_history_reset(self.h))

    def history(self) -> np.ndarray:
        """[steps, 6 + n_species]: field energy per component, then the
        kinetic energy of each species, one row per step."""
        n, c = C.c_int(), C.c_int()
        _ck(self.lib.zc_history_get(self.h, None, 0, C.byref(n), C.byref(c)))
        out = np.zeros((n.value, c.value), dtype=np.float64)
        if n.value:
            _ck(self.lib.zc_history_get(self.h, _p(out), n.value, C.byref(n), C.byref(c)))
        return out


class CudaBatch:
    """Independent simulations advanced together (a ``zc_batch`` handle):
    one CUDA graph per group of members runs a block of steps of each of
    them as parallel branches.  ``groups`` sets the group count (None: one
    per 32 members, 1 to 8).  The members stay usable on their own."""

    def __init__(self, sims, groups=None):
        self.lib = load()
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s.h.value for s in self.sims])
        h = C.c_void_p()
        _ck(self.lib.zc_batch_create(arr, len(self.sims), C.byref(h)))
        self.h = h
        if groups is not None:
            self.set_groups(groups)

    def set_groups(self, n):
        _ck(self.lib.zc_batch_set_groups(self.h, int(n)))

    @property
    def groups(self) -> int:
        v = C.c_int()
        _ck(self.lib.zc_batch_get_groups(self.h, C.byref(v)))
        return v.value

    def step(self, n=1):
        _ck(self.lib.zc_batch_step(self.h, int(n)))

    def last_ms(self) -> float:
        v = C.c_float()
        _ck(self.lib.zc_batch_last_ms(self.h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.zc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
