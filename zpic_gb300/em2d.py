"""em2d -- ZPIC's 2D electromagnetic PIC code on GB300, with the class
interface of the reference's Cython module (python/source/em2d.pyx):
``Density``, ``Species``, ``ExternalField``, ``InitialField``, ``EMF``,
``Laser``, ``Current``, ``Smooth`` and ``Simulation``.

Like the Cython module sits on the em2d C API, this module sits on
``libzpic_em2d`` (the same C API, include/em2d/*.h) through ctypes; the time
step runs on the GPU through ``libzpic_cuda``.  Particle loading uses the same
generator, seeded like the reference (``set_rand_seed(12345, 67890)`` in
``Simulation.__init__``, em2d.pyx:1781).

Data access follows the reference: ``Species.particles``, ``EMF.Ex`` ...
``Current.Jz`` are numpy views of host buffers in the reference layout.  Here
those buffers mirror the device state: a view is refreshed from the GPU when
it is taken, and writes made through the particle view (or ``Species.add``)
are sent back to the GPU before the next step.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

from . import _zc

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libzpic_em2d.so")


# ---------------------------------------------------------------------------
# C structures (include/em2d/*.h, same layout as the reference's headers)
# ---------------------------------------------------------------------------
class float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


DENS_FN = C.CFUNCTYPE(C.c_float, C.c_float, C.c_void_p)


class t_density(C.Structure):
    _fields_ = [("n", C.c_float), ("type", C.c_int), ("start", C.c_float), ("end", C.c_float),
                ("custom_x", DENS_FN), ("custom_data_x", C.c_void_p),
                ("custom_y", DENS_FN), ("custom_data_y", C.c_void_p),
                ("custom_x_total_part", C.c_ulong), ("custom_x_total_q", C.c_double)]


class t_part(C.Structure):
    _fields_ = [("ix", C.c_int), ("iy", C.c_int), ("x", C.c_float), ("y", C.c_float),
                ("ux", C.c_float), ("uy", C.c_float), ("uz", C.c_float)]


class t_species(C.Structure):
    _fields_ = [("name", C.c_char * 33), ("part", C.POINTER(t_part)), ("np", C.c_int), ("np_max", C.c_int),
                ("m_q", C.c_float), ("energy", C.c_double), ("q", C.c_float), ("ppc", C.c_int * 2),
                ("density", t_density), ("ufl", C.c_float * 3), ("uth", C.c_float * 3),
                ("nx", C.c_int * 2), ("dx", C.c_float * 2), ("box", C.c_float * 2), ("dt", C.c_float),
                ("iter", C.c_int), ("moving_window", C.c_int), ("n_move", C.c_int), ("n_sort", C.c_int)]


class t_smooth(C.Structure):
    _fields_ = [("xtype", C.c_int), ("ytype", C.c_int), ("xlevel", C.c_int), ("ylevel", C.c_int)]


class t_current(C.Structure):
    _fields_ = [("J", C.POINTER(float3)), ("J_buf", C.POINTER(float3)), ("nx", C.c_int * 2), ("nrow", C.c_int),
                ("gc", (C.c_int * 2) * 2), ("box", C.c_float * 2), ("dx", C.c_float * 2), ("smooth", t_smooth),
                ("dt", C.c_float), ("iter", C.c_int), ("moving_window", C.c_int)]


class t_emf_ext_fld(C.Structure):
    _fields_ = [("E_type", C.c_int), ("B_type", C.c_int), ("E_0", float3), ("B_0", float3),
                ("E_custom", C.c_void_p), ("B_custom", C.c_void_p), ("E_custom_data", C.c_void_p),
                ("B_custom_data", C.c_void_p), ("E_part_buf", C.POINTER(float3)),
                ("B_part_buf", C.POINTER(float3))]


class t_emf(C.Structure):
    _fields_ = [("E", C.POINTER(float3)), ("B", C.POINTER(float3)), ("E_buf", C.POINTER(float3)),
                ("B_buf", C.POINTER(float3)), ("E_part", C.POINTER(float3)), ("B_part", C.POINTER(float3)),
                ("nx", C.c_int * 2), ("nrow", C.c_int), ("gc", (C.c_int * 2) * 2), ("box", C.c_float * 2),
                ("dx", C.c_float * 2), ("dt", C.c_float), ("iter", C.c_int), ("moving_window", C.c_int),
                ("n_move", C.c_int), ("ext_fld", t_emf_ext_fld)]


class t_emf_laser(C.Structure):
    _fields_ = [("type", C.c_int), ("start", C.c_float), ("fwhm", C.c_float), ("rise", C.c_float),
                ("flat", C.c_float), ("fall", C.c_float), ("a0", C.c_float), ("omega0", C.c_float),
                ("polarization", C.c_float), ("W0", C.c_float), ("focus", C.c_float), ("axis", C.c_float)]


class t_simulation(C.Structure):
    _fields_ = [("dt", C.c_float), ("tmax", C.c_float), ("ndump", C.c_int), ("n_species", C.c_int),
                ("species", C.POINTER(t_species)), ("emf", t_emf), ("current", t_current),
                ("moving_window", C.c_int)]


PART_DTYPE = np.dtype([("ix", "<i4"), ("iy", "<i4"), ("x", "<f4"), ("y", "<f4"),
                       ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])

_lib = None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    _zc.load()  # builds the libraries when absent; fails loudly without CUDA
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sigs = {
        "set_rand_seed": (None, [C.c_uint32, C.c_uint32]),
        "rand_seed_fresh": (None, [C.c_uint32, C.c_uint32]),
        "spec_new": (None, [C.POINTER(t_species), C.c_char_p, C.c_float, P, P, P, P, P, C.c_float,
                            C.POINTER(t_density)]),
        "spec_grow_buffer": (None, [C.POINTER(t_species), C.c_int]),
        "spec_delete": (None, [C.POINTER(t_species)]),
        "sim_new": (None, [C.POINTER(t_simulation), P, P, C.c_float, C.c_float, C.c_int,
                           C.POINTER(t_species), C.c_int]),
        "sim_delete": (None, [C.POINTER(t_simulation)]),
        "sim_iter": (None, [C.POINTER(t_simulation)]),
        "sim_set_moving_window": (None, [C.POINTER(t_simulation)]),
        "sim_set_smooth": (None, [C.POINTER(t_simulation), C.POINTER(t_smooth)]),
        "sim_add_laser": (None, [C.POINTER(t_simulation), C.POINTER(t_emf_laser)]),
        "sim_sync_host": (None, [C.POINTER(t_simulation)]),
        "sim_set_mirrors": (None, [C.POINTER(t_simulation), C.c_int]),
        "sim_gpu_handle": (P, [C.POINTER(t_simulation)]),
        "sim_sync_device": (None, [C.POINTER(t_simulation)]),
        "sim_set_gpu_options": (None, [C.c_int, C.c_int, C.c_int, C.c_int]),
        "emf_get_energy": (None, [C.POINTER(t_emf), P]),
        "emf_set_ext_fld_grid": (None, [C.POINTER(t_emf), C.c_int, P, P, C.c_int, P, P]),
        "emf_init_fld_grid": (None, [C.POINTER(t_emf), P, P]),
        "spec_deposit_charge": (None, [C.POINTER(t_species), P]),
        "spec_deposit_pha": (None, [C.POINTER(t_species), C.c_int, P, P, P]),
        "spec_report": (None, [C.POINTER(t_species), C.c_int, P, P]),
        "emf_report": (None, [C.POINTER(t_emf), C.c_char, C.c_int]),
        "current_report": (None, [C.POINTER(t_current), C.c_int]),
        "zdf_flush": (C.c_int, []),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def zdf_flush():
    """Waits until every report file queued so far is written (the reports
    write ZDF files on a background thread); returns how many failed."""
    return int(_load().zdf_flush())


def gpu_options(device=0, tile=(16, 16), fast_math=False):
    """GPU, particle tile and push build used by the next Simulation."""
    _load().sim_set_gpu_options(int(device), int(tile[0]), int(tile[1]), int(bool(fast_math)))


def _arr(values, dtype):
    return np.ascontiguousarray(values, dtype=dtype)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------------------
# Density (em2d.pyx:25-168)
# ---------------------------------------------------------------------------
class Density:
    """Density(type='uniform', start=0.0, end=0.0, n=1.0, custom_x=None, custom_y=None)

    Charge density profile used to load a particle species: "uniform",
    "empty", "step", "slab" or "custom" (custom_x / custom_y are functions of
    position)."""

    _density_types = {"uniform": 0, "empty": 1, "step": 2, "slab": 3, "custom": 4}

    def __init__(self, *, type="uniform", start=0.0, end=0.0, n=1.0, custom_x=None, custom_y=None):
        self._d = t_density()
        self._d.type = self._density_types[type]
        self._d.n = n
        self._d.start = start
        self._d.end = end
        self.custom_func_x = None
        self.custom_func_y = None
        self._cb = []
        if custom_x:
            self.custom_func_x = custom_x
        if custom_y:
            self.custom_func_y = custom_y
        self._bind()

    def _bind(self):
        self._cb = []
        if self.custom_func_x:
            cb = DENS_FN(lambda x, _d, f=self.custom_func_x: float(f(x)))
            self._cb.append(cb)
            self._d.custom_x = cb
        if self.custom_func_y:
            cb = DENS_FN(lambda y, _d, f=self.custom_func_y: float(f(y)))
            self._cb.append(cb)
            self._d.custom_y = cb

    def copy(self):
        new = Density()
        C.memmove(C.byref(new._d), C.byref(self._d), C.sizeof(t_density))
        new.custom_func_x = self.custom_func_x
        new.custom_func_y = self.custom_func_y
        new._bind()
        return new

    @property
    def n(self):
        return self._d.n

    @n.setter
    def n(self, value):
        self._d.n = value

    @property
    def type(self):
        return {v: k for k, v in self._density_types.items()}[self._d.type]

    @type.setter
    def type(self, value):
        self._d.type = self._density_types[value]

    @property
    def start(self):
        return self._d.start

    @start.setter
    def start(self, value):
        self._d.start = value

    @property
    def end(self):
        return self._d.end

    @end.setter
    def end(self, value):
        self._d.end = value


# ---------------------------------------------------------------------------
# Species (em2d.pyx:171-458)
# ---------------------------------------------------------------------------
def load_particles(m_q, ppc, nx, box, dt, *, ufl=(0.0, 0.0, 0.0), uth=(0.0, 0.0, 0.0), density=None,
                   name="species"):
    """Loads one species on the host exactly as spec_new does
    (em2d/particles.c:535-612), from the current state of the global random
    generator (set_rand_seed), and returns (particles, q): the records as a
    structured array and the charge of one simulation particle."""
    lib = _load()
    sp = t_species()
    nx_a, box_a = _arr(nx, np.int32), _arr(box, np.float32)
    ppc_a, ufl_a, uth_a = _arr(ppc, np.int32), _arr(ufl, np.float32), _arr(uth, np.float32)
    dens = density if density is not None else Density()
    lib.spec_new(C.byref(sp), name.encode(), float(m_q), _ptr(ppc_a), _ptr(ufl_a), _ptr(uth_a), _ptr(nx_a),
                 _ptr(box_a), float(dt), C.byref(dens._d))
    try:
        if sp.np > 0:
            buf = (t_part * sp.np).from_address(C.addressof(sp.part.contents))
            parts = np.frombuffer(buf, dtype=PART_DTYPE).copy()
        else:
            parts = np.zeros(0, dtype=PART_DTYPE)
        return parts, float(sp.q)
    finally:
        lib.spec_delete(C.byref(sp))


def set_rand_seed(w, z, fresh=False):
    """Seeds the generator used by species loading (em2d/random.c:48-53).
    The generator is per host thread.  ``fresh`` also drops the cached
    normal deviate, giving the state of a newly started process."""
    if fresh:
        _load().rand_seed_fresh(int(w), int(z))
    else:
        _load().set_rand_seed(int(w), int(z))


class Species:
    """Species(name, m_q, ppc=[1,1], ufl=[0,0,0], uth=[0,0,0], density=None, n_sort=16)

    A particle species.  ``particles`` gives read/write access to the
    particle records (ix, iy, x, y, ux, uy, uz)."""

    _diag_types = {"charge": 0x1000, "pha": 0x2000, "particles": 0x3000}
    _pha_quants = {"x1": 1, "x2": 2, "u1": 4, "u2": 5, "u3": 6}

    def __init__(self, name, m_q, ppc=(1, 1), *, ufl=(0.0, 0.0, 0.0), uth=(0.0, 0.0, 0.0), density=None,
                 n_sort=16):
        self._name = name
        self._m_q = float(m_q)
        self._ppc = _arr(ppc, np.int32)
        self._ufl = _arr(ufl, np.float32)
        self._uth = _arr(uth, np.float32)
        self._n_sort = int(n_sort)
        self._density = density.copy() if density else Density()
        self._sp = None    # pointer to the t_species inside the simulation
        self._sim = None

    def _new(self, ptr, nx, box, dt):
        self._sp = ptr
        _load().spec_new(ptr, self._name.encode(), self._m_q, _ptr(self._ppc), _ptr(self._ufl),
                         _ptr(self._uth), _ptr(nx), _ptr(box), float(dt), C.byref(self._density._d))
        ptr.contents.n_sort = self._n_sort

    def _s(self):
        if self._sp is None:
            raise RuntimeError("species is not part of a simulation yet")
        return self._sp.contents

    def add(self, ix, x, u):
        """add(ix, x, u): appends one particle (sent to the GPU before the
        next step)."""
        self._sim._pull()
        s = self._s()
        _load().spec_grow_buffer(self._sp, s.np + 1)
        s.part[s.np] = t_part(int(ix[0]), int(ix[1]), float(x[0]), float(x[1]), float(u[0]), float(u[1]),
                              float(u[2]))
        s.np += 1
        self._sim._dirty_host = True

    def report(self, type, *, quants=(), pha_nx=(), pha_range=()):
        rep = self._diag_types[type]
        if rep == 0x2000:
            nx = _arr(pha_nx, np.int32)
            rg = _arr(pha_range, np.float32)
            rep = self._pha_quants[quants[0]] + self._pha_quants[quants[1]] * 16 + 0x2000
            _load().spec_report(self._sp, rep, _ptr(nx), _ptr(rg))
        else:
            _load().spec_report(self._sp, rep, None, None)

    @property
    def particles(self):
        """ndarray of particle data (read/write)."""
        self._sim._pull()
        s = self._s()
        self._sim._dirty_host = True  # the caller may edit the records
        if s.np == 0:
            return np.zeros(0, dtype=PART_DTYPE)
        buf = (t_part * s.np).from_address(C.addressof(s.part.contents))
        return np.frombuffer(buf, dtype=PART_DTYPE)

    def charge(self):
        """Charge density of the species on the simulation grid (nx[1], nx[0])."""
        s = self._s()
        rho = np.zeros((s.nx[1] + 1, s.nx[0] + 1), dtype=np.float32)
        self._sim._push()
        _load().spec_deposit_charge(self._sp, _ptr(rho))
        return rho[: s.nx[1], : s.nx[0]]

    def phasespace(self, quants, pha_nx, pha_range):
        self._sim._push()
        nx = _arr(pha_nx, np.int32)
        rg = _arr(pha_range, np.float32)
        rep = self._pha_quants[quants[0]] + self._pha_quants[quants[1]] * 16 + 0x2000
        pha = np.zeros((nx[1], nx[0]), dtype=np.float32)
        _load().spec_deposit_pha(self._sp, rep, _ptr(nx), _ptr(rg), _ptr(pha))
        return pha

    @property
    def energy(self):
        """Time-centred kinetic energy after the last step (0 before the
        first)."""
        self._sim._refresh_energy()
        return self._s().energy

    @property
    def dx(self):
        return np.array(self._s().dx[:], dtype=np.float32)

    @property
    def dt(self):
        return self._s().dt

    @property
    def iter(self):
        return self._s().iter

    @property
    def ppc(self):
        return np.array(self._s().ppc[:], dtype=np.int32)

    @property
    def n_sort(self):
        return self._s().n_sort if self._sp is not None else self._n_sort

    @n_sort.setter
    def n_sort(self, value):
        if value < 0:
            print("(*error*) Invalid value for n_sort, must be >= 0.", file=sys.stderr)
            return
        if self._sp is not None:
            self._s().n_sort = int(value)
        self._n_sort = int(value)

    @property
    def n_move(self):
        self._sim._pull()
        return self._s().n_move


# ---------------------------------------------------------------------------
# external / initial fields (em2d.pyx:461-876)
# ---------------------------------------------------------------------------
_FLD = {"none": 0, "uniform": 1, "custom": 2}


class _FieldSpec:
    def __init__(self, *, E_type="none", B_type="none", E_0=None, B_0=None, E_custom=None, B_custom=None):
        self._E_type = E_type
        self._B_type = B_type
        self._E_0 = list(E_0) if E_0 is not None else [0.0, 0.0, 0.0]
        self._B_0 = list(B_0) if B_0 is not None else [0.0, 0.0, 0.0]
        self.custom_func_E = E_custom
        self.custom_func_B = B_custom

    def copy(self):
        return type(self)(E_type=self._E_type, B_type=self._B_type, E_0=self._E_0, B_0=self._B_0,
                          E_custom=self.custom_func_E, B_custom=self.custom_func_B)

    E_type = property(lambda s: s._E_type, lambda s, v: setattr(s, "_E_type", v))
    B_type = property(lambda s: s._B_type, lambda s, v: setattr(s, "_B_type", v))
    E_0 = property(lambda s: s._E_0, lambda s, v: setattr(s, "_E_0", list(v)))
    B_0 = property(lambda s: s._B_0, lambda s, v: setattr(s, "_B_0", list(v)))
    E_custom = property(lambda s: s.custom_func_E, lambda s, v: setattr(s, "custom_func_E", v))
    B_custom = property(lambda s: s.custom_func_B, lambda s, v: setattr(s, "custom_func_B", v))

    def _grid(self, fn, emf):
        """Evaluates fn(ix, dx, iy, dy) on every buffer cell, reference layout."""
        e = emf._e()
        nx, ny = e.nx[0], e.nx[1]
        dx, dy = float(e.dx[0]), float(e.dx[1])
        g = np.zeros((ny + 3, nx + 3, 3), dtype=np.float32)
        for j in range(-1, ny + 2):
            for i in range(-1, nx + 2):
                g[j + 1, i + 1] = fn(i, dx, j, dy)
        return g


class ExternalField(_FieldSpec):
    """ExternalField(E_type='none', B_type='none', E_0=None, B_0=None, E_custom=None, B_custom=None)

    External E/B fields seen by the particles (added to the self-consistent
    fields); custom fields are functions f(ix, dx, iy, dy) -> (fx, fy, fz)."""


class InitialField(_FieldSpec):
    """InitialField(E_type='none', B_type='none', E_0=None, B_0=None, E_custom=None, B_custom=None)

    Initial E/B field values."""


# ---------------------------------------------------------------------------
# EMF (em2d.pyx:879-1294)
# ---------------------------------------------------------------------------
class EMF:
    """The simulation's electromagnetic fields (created by Simulation)."""

    _diag_types = {"E": 0, "B": 1, "Epart": 2, "Bpart": 3}

    def __init__(self, sim):
        self._sim = sim

    def _e(self):
        return self._sim._s.contents.emf

    def _eptr(self):
        return C.pointer(self._e())

    def report(self, type, fc):
        self._sim._push()
        _load().emf_report(self._eptr(), bytes([self._diag_types[type]]), int(fc))

    def set_ext_fld(self, ext):
        t = (_FLD[ext.E_type], _FLD[ext.B_type])
        E0 = _arr(ext.E_0, np.float32)
        B0 = _arr(ext.B_0, np.float32)
        Eg = ext._grid(ext.custom_func_E, self) if t[0] == 2 else None
        Bg = ext._grid(ext.custom_func_B, self) if t[1] == 2 else None
        self._sim._push()
        _load().emf_set_ext_fld_grid(self._eptr(), t[0], _ptr(E0), None if Eg is None else _ptr(Eg),
                                     t[1], _ptr(B0), None if Bg is None else _ptr(Bg))
        self._sim._synced = False

    def init_fld(self, init):
        if self._e().iter != 0:
            raise RuntimeError("emf_init_fld should only be called at initialization")
        self._sim._pull()
        e = self._e()
        shape = (e.nx[1] + 3, e.nx[0] + 3, 3)
        E = np.ctypeslib.as_array(C.cast(e.E_buf, C.POINTER(C.c_float)), shape=shape).copy()
        B = np.ctypeslib.as_array(C.cast(e.B_buf, C.POINTER(C.c_float)), shape=shape).copy()
        for F, t, v0, fn in ((E, init.E_type, init.E_0, init.custom_func_E),
                             (B, init.B_type, init.B_0, init.custom_func_B)):
            if t == "uniform":
                F[:] = np.asarray(v0, dtype=np.float32)
            elif t == "custom":
                F[:] = init._grid(fn, self)
        _load().emf_init_fld_grid(self._eptr(), _ptr(E), _ptr(B))
        self._sim._synced = False

    @property
    def nx(self):
        return np.array(self._e().nx[:], dtype=np.int32)

    @property
    def dx(self):
        return np.array(self._e().dx[:], dtype=np.float32)

    @property
    def box(self):
        return np.array(self._e().box[:], dtype=np.float32)

    @property
    def n_move(self):
        return self._e().n_move

    @property
    def energy(self):
        """Field energy per component [Ex, Ey, Ez, Bx, By, Bz]."""
        self._sim._push()
        out = np.zeros(6, dtype=np.float64)
        _load().emf_get_energy(self._eptr(), _ptr(out))
        return out

    @property
    def solver_type(self):
        return "Yee"

    def _component(self, which, comp):
        self._sim._pull()
        e = self._e()
        gx, gy = e.nx[0] + 3, e.nx[1] + 3
        ptr = {"E": e.E_buf, "B": e.B_buf,
               "Epart": e.ext_fld.E_part_buf if e.ext_fld.E_type else e.E_buf,
               "Bpart": e.ext_fld.B_part_buf if e.ext_fld.B_type else e.B_buf}[which]
        full = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float)), shape=(gy, gx, 3))
        # the same slice as the reference (em2d.pyx:1061)
        return full[1: 1 + e.nx[1], 1: 1 + e.nx[0], comp]

    Ex = property(lambda s: s._component("E", 0))
    Ey = property(lambda s: s._component("E", 1))
    Ez = property(lambda s: s._component("E", 2))
    Bx = property(lambda s: s._component("B", 0))
    By = property(lambda s: s._component("B", 1))
    Bz = property(lambda s: s._component("B", 2))
    Ex_part = property(lambda s: s._component("Epart", 0))
    Ey_part = property(lambda s: s._component("Epart", 1))
    Ez_part = property(lambda s: s._component("Epart", 2))
    Bx_part = property(lambda s: s._component("Bpart", 0))
    By_part = property(lambda s: s._component("Bpart", 1))
    Bz_part = property(lambda s: s._component("Bpart", 2))


# ---------------------------------------------------------------------------
# Laser (em2d.pyx:1297-1531)
# ---------------------------------------------------------------------------
class Laser:
    """Laser(type='plane', start=0.0, fwhm=0.0, rise=0.0, flat=0.0, fall=0.0, a0=0.0, omega0=0.0,
    polarization=0.0, W0=0.0, focus=0.0, axis=0.0)"""

    _laser_types = {"plane": 0, "gaussian": 1}

    def __init__(self, *, type="plane", start=0.0, fwhm=0.0, rise=0.0, flat=0.0, fall=0.0, a0=0.0,
                 omega0=0.0, polarization=0.0, W0=0.0, focus=0.0, axis=0.0):
        self._l = t_emf_laser(self._laser_types[type], start, fwhm, rise, flat, fall, a0, omega0,
                              polarization, W0, focus, axis)

    def __getattr__(self, name):
        if name in ("start", "fwhm", "rise", "flat", "fall", "a0", "omega0", "polarization", "W0",
                    "focus", "axis"):
            return getattr(self.__dict__["_l"], name)
        if name == "type":
            return {v: k for k, v in self._laser_types.items()}[self.__dict__["_l"].type]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name == "_l":
            self.__dict__["_l"] = value
        elif name == "type":
            self._l.type = self._laser_types[value]
        else:
            setattr(self._l, name, value)


# ---------------------------------------------------------------------------
# Current (em2d.pyx:1535-1620)
# ---------------------------------------------------------------------------
class Current:
    """The simulation's electric current density (created by Simulation)."""

    def __init__(self, sim):
        self._sim = sim

    def _c(self):
        return self._sim._s.contents.current

    def report(self, jc):
        _load().current_report(C.pointer(self._c()), int(jc))

    def _component(self, comp):
        self._sim._pull()
        c = self._c()
        full = np.ctypeslib.as_array(C.cast(c.J_buf, C.POINTER(C.c_float)),
                                     shape=(c.nx[1] + 3, c.nx[0] + 3, 3))
        return full[1: 1 + c.nx[1], 1: 1 + c.nx[0], comp]

    Jx = property(lambda s: s._component(0))
    Jy = property(lambda s: s._component(1))
    Jz = property(lambda s: s._component(2))


# ---------------------------------------------------------------------------
# Smooth (em2d.pyx:1622-1723)
# ---------------------------------------------------------------------------
class Smooth:
    """Smooth(xtype='none', ytype='none', xlevel=0, ylevel=0)"""

    _filter_types = {"none": 0, "binomial": 1, "compensated": 2}

    def __init__(self, *, xtype="none", ytype="none", xlevel=0, ylevel=0):
        self._s = t_smooth(self._filter_types[xtype], self._filter_types[ytype], int(xlevel), int(ylevel))

    def _name(self, v):
        return {v_: k for k, v_ in self._filter_types.items()}[v]

    xtype = property(lambda s: s._name(s._s.xtype), lambda s, v: setattr(s._s, "xtype", s._filter_types[v]))
    ytype = property(lambda s: s._name(s._s.ytype), lambda s, v: setattr(s._s, "ytype", s._filter_types[v]))
    xlevel = property(lambda s: s._s.xlevel, lambda s, v: setattr(s._s, "xlevel", int(v)))
    # the reference's getter returns xlevel (em2d.pyx:1720); kept
    ylevel = property(lambda s: s._s.xlevel, lambda s, v: setattr(s._s, "ylevel", int(v)))


# ---------------------------------------------------------------------------
# Simulation (em2d.pyx:1726-2074)
# ---------------------------------------------------------------------------
class Simulation:
    """Simulation(nx, box, dt, species=None, report=None, mov_window=False, smooth=None,
    init_fld=None, ext_fld=None)"""

    def __init__(self, nx, box, dt, *, species=None, report=None, mov_window=False, smooth=None,
                 init_fld=None, ext_fld=None):
        lib = _load()
        self._s = C.pointer(t_simulation())
        # the seeds of a new C simulation (em2d.pyx:1781)
        lib.set_rand_seed(12345, 67890)
        self._nx = _arr(nx, np.int32)
        self._box = _arr(box, np.float32)
        self._dirty_host = False   # host mirrors edited: upload before the next step
        self._synced = True        # host mirrors match the device
        self._energy_ok = True
        if isinstance(species, Species):
            species = [species]
        elif species is None:
            species = []
        self.species = list(species)
        n = len(self.species)
        # the C library owns (and frees in sim_delete) the species array
        libc = C.CDLL(None)
        libc.calloc.restype = C.c_void_p
        libc.calloc.argtypes = [C.c_size_t, C.c_size_t]
        raw = libc.calloc(max(n, 1), C.sizeof(t_species))
        self._spec = C.cast(raw, C.POINTER(t_species))
        for k, sp in enumerate(self.species):
            sp._sim = self
            sp._new(C.pointer(self._spec[k]), self._nx, self._box, float(dt))
        self.report = report
        lib.sim_new(self._s, _ptr(self._nx), _ptr(self._box), float(dt), 0.0, 0, self._spec if n else None, n)
        self._alive = True
        # this class refreshes the mirrors when a view is taken and uploads
        # edits before a step itself, so the library's per-step copies are off
        lib.sim_set_mirrors(self._s, 0)
        self.n = 0
        self.t = 0.0
        self.emf = EMF(self)
        self.current = Current(self)
        if mov_window:
            lib.sim_set_moving_window(self._s)
        if smooth:
            lib.sim_set_smooth(self._s, C.byref(smooth._s))
        if init_fld:
            self.emf.init_fld(init_fld)
        if ext_fld:
            self.emf.set_ext_fld(ext_fld)

    def __del__(self):
        if getattr(self, "_alive", False):
            _load().sim_delete(self._s)
            self._alive = False

    # ---- host mirrors ----
    def _pull(self):
        """Refreshes the host mirrors from the GPU when they are stale."""
        if not self._synced:
            _load().sim_sync_host(self._s)
            self._synced = True
            self._energy_ok = True

    def _push(self):
        """Sends host edits to the GPU (before a step or a device query)."""
        if self._dirty_host:
            _load().sim_sync_device(self._s)
            self._dirty_host = False

    def _refresh_energy(self):
        if not self._energy_ok:
            self._pull()

    def _stepped(self):
        self._synced = False
        self._energy_ok = False

    # ---- API ----
    def set_moving_window(self):
        _load().sim_set_moving_window(self._s)

    def set_smooth(self, smooth):
        _load().sim_set_smooth(self._s, C.byref(smooth._s))

    def add_laser(self, laser):
        self._push()
        _load().sim_add_laser(self._s, C.byref(laser._l))
        self._synced = False

    def iter(self):
        """Advance the simulation one iteration."""
        self._push()
        _load().sim_iter(self._s)
        self._stepped()
        self.n = self.n + 1
        self.t = self.n * self._s.contents.dt

    def run(self, tmax):
        """Advance the simulation up to time tmax, calling the report
        function (if any) before every iteration."""
        if tmax < self.t:
            print("Simulation is already at t = {:g}".format(self.t))
            return
        print("\nRunning simulation up to t = {:g} ...".format(tmax))
        while self.t <= tmax:
            print("n = {:d}, t = {:g}".format(self.n, self.t), end="\r")
            if self.report:
                self.report(self)
            self.iter()
        print("n = {:d}, t = {:g}".format(self.n, self.t), end="\r")
        print("\nDone.")

    @property
    def dt(self):
        return self._s.contents.dt

    @property
    def dx(self):
        return self.emf.dx

    @property
    def nx(self):
        return self.emf.nx

    @property
    def box(self):
        return self.emf.box

    @property
    def n_move(self):
        return self.emf.n_move
