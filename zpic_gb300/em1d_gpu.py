"""The em1d step on the GPU (C-ABI zc1_* of libzpic_cuda).

    sim = CudaSim1D(nx, box, dt, open_fields=False, open_particles=False,
                    moving_window=False)
    sim.add_species(m_q, q, ppc, particles, ufl=..., density=("step", start, end))
    sim.set_smooth("compensated", 1)
    sim.set_fields(E, B)         # (nx + 3, 3) float32 buffers, reference layout
    sim.add_laser(start, a0, omega0, fwhm=..., polarization=...)
    sim.step(n)
    sim.E(), sim.B(), sim.J(), sim.energy(), sim.particles(k)

Particles are the reference's 20-byte records (PART_DTYPE), e.g. as its
spec_new loads them (em1d/particles.c:511-592).  There is no CPU fallback:
without the CUDA library the constructor raises.
"""
import ctypes as C

import numpy as np

from . import _zc

PART_DTYPE = np.dtype([("ix", "<i4"), ("x", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])
DENSITY = {"uniform": 0, "empty": 1, "step": 2, "slab": 3}
SMOOTH = {"none": 0, "binomial": 1, "compensated": 2}


class Desc1(C.Structure):
    _fields_ = [("nx", C.c_int), ("box", C.c_float), ("dt", C.c_float), ("device", C.c_int),
                ("open_fields", C.c_int), ("open_particles", C.c_int), ("moving_window", C.c_int),
                ("sort_every", C.c_int), ("push_ctas", C.c_int)]


class SpeciesDesc1(C.Structure):
    _fields_ = [("m_q", C.c_float), ("q", C.c_float), ("ppc", C.c_int), ("ufl", C.c_float * 3),
                ("uth", C.c_float * 3), ("density", C.c_int), ("start", C.c_float), ("end", C.c_float)]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class CudaSim1D:
    def __init__(self, nx, box, dt, *, device=0, open_fields=False, open_particles=False, moving_window=False,
                 sort_every=0, push_ctas=0):
        self.lib = _zc.load()
        self.nx = int(nx)
        d = Desc1(self.nx, float(box), float(dt), int(device), int(bool(open_fields)), int(bool(open_particles)),
                  int(bool(moving_window)), int(sort_every), int(push_ctas))
        h = C.c_void_p()
        _zc._ck(self.lib.zc1_create(C.byref(d), C.byref(h)))
        self.h = h
        self.nspec = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.zc1_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_species(self, m_q, q, ppc, particles, *, ufl=(0, 0, 0), uth=(0, 0, 0), density=("uniform", 0.0, 0.0)):
        parts = np.ascontiguousarray(particles, dtype=PART_DTYPE)
        sd = SpeciesDesc1(float(m_q), float(q), int(ppc), (C.c_float * 3)(*ufl), (C.c_float * 3)(*uth),
                          DENSITY[density[0]], float(density[1]), float(density[2]))
        k = C.c_int()
        _zc._ck(self.lib.zc1_add_species(self.h, C.byref(sd), _p(parts), len(parts), C.byref(k)))
        self.nspec += 1
        return k.value

    def set_smooth(self, type="none", level=0):
        _zc._ck(self.lib.zc1_set_smooth(self.h, SMOOTH[type], int(level)))

    def set_fields(self, E=None, B=None):
        e = None if E is None else np.ascontiguousarray(E, dtype=np.float32)
        b = None if B is None else np.ascontiguousarray(B, dtype=np.float32)
        _zc._ck(self.lib.zc1_set_fields(self.h, None if e is None else _p(e), None if b is None else _p(b)))

    def _grid(self):
        return np.zeros((self.nx + 3, 3), dtype=np.float32)

    def E(self):
        out = self._grid()
        _zc._ck(self.lib.zc1_get_fields(self.h, _p(out), None))
        return out

    def B(self):
        out = self._grid()
        _zc._ck(self.lib.zc1_get_fields(self.h, None, _p(out)))
        return out

    def J(self):
        out = self._grid()
        _zc._ck(self.lib.zc1_get_current(self.h, _p(out)))
        return out

    def add_laser(self, start, a0, omega0, *, fwhm=0.0, rise=0.0, flat=0.0, fall=0.0, polarization=0.0):
        """emf_add_laser (em1d/emf.c:191-260): a plane-wave pulse ending at
        `start`; `fwhm`, when set, overrides rise/flat/fall"""
        L = _zc.Laser(type=0, start=float(start), fwhm=float(fwhm), rise=float(rise), flat=float(flat),
                      fall=float(fall), a0=float(a0), omega0=float(omega0), polarization=float(polarization))
        _zc._ck(self.lib.zc1_add_laser(self.h, C.byref(L)))

    def step(self, n=1, wait=True):
        """n steps; with wait=False they are only enqueued (simulations then
        overlap on the GPU) until synchronize()"""
        if wait:
            _zc._ck(self.lib.zc1_step(self.h, int(n)))
        else:
            _zc._ck(self.lib.zc1_step_async(self.h, int(n)))

    def synchronize(self):
        _zc._ck(self.lib.zc1_synchronize(self.h))

    def pushed(self, k):
        """particles species k has pushed so far (particle-steps)"""
        v = C.c_longlong()
        _zc._ck(self.lib.zc1_species_pushed(self.h, int(k), C.byref(v)))
        return v.value

    def launches(self):
        """kernels launched by the steps so far"""
        v = C.c_longlong()
        _zc._ck(self.lib.zc1_get_launches(self.h, C.byref(v)))
        return v.value

    KINDS = ("push", "sort", "fields")

    def set_profile(self, on=True):
        _zc._ck(self.lib.zc1_set_profile(self.h, int(bool(on))))

    def profile(self):
        """{kind: (device ms, launches)} since set_profile(True)"""
        ms = np.zeros(len(self.KINDS))
        n = np.zeros(len(self.KINDS), dtype=np.int64)
        _zc._ck(self.lib.zc1_get_profile(self.h, _p(ms), _p(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.KINDS)}

    def last_ms(self):
        """device time of the last step() call, CUDA events on the simulation's stream"""
        v = C.c_float()
        _zc._ck(self.lib.zc1_last_step_ms(self.h, C.byref(v)))
        return v.value

    def energy(self):
        """(field energy per component [6], kinetic energy per species)"""
        emf = np.zeros(6)
        kin = np.zeros(max(self.nspec, 1))
        _zc._ck(self.lib.zc1_energy(self.h, _p(emf), _p(kin)))
        return emf, kin[:self.nspec]

    def count(self, k):
        n = C.c_int()
        _zc._ck(self.lib.zc1_species_count(self.h, int(k), C.byref(n)))
        return n.value

    def particles(self, k):
        n = self.count(k)
        out = np.zeros(n, dtype=PART_DTYPE)
        got = C.c_int()
        _zc._ck(self.lib.zc1_get_particles(self.h, int(k), _p(out), n, C.byref(got)))
        return out[:got.value]

    def info(self):
        it, nm = C.c_int(), C.c_int()
        _zc._ck(self.lib.zc1_get_info(self.h, C.byref(it), C.byref(nm)))
        return {"iter": it.value, "n_move": nm.value}
