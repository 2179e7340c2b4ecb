"""Writer-level ZDF cases shared by the fixture generator
(tests/golden/make_zdf_golden.py, run against the reference's em2d/zdf.c)
and the tests (run against libzpic_em2d): the same calls with the same
inputs must give byte-identical files.

The ctypes structs follow the ZDF interface (include/em2d/zdf.h, the
reference's em2d/zdf.h:93-203)."""
import ctypes as C
import os

import numpy as np


class GridAxis(C.Structure):
    _fields_ = [("name", C.c_char_p), ("type", C.c_int), ("min", C.c_double), ("max", C.c_double),
                ("label", C.c_char_p), ("units", C.c_char_p)]


class GridInfo(C.Structure):
    _fields_ = [("name", C.c_char_p), ("ndims", C.c_uint32), ("count", C.c_uint64 * 3), ("label", C.c_char_p),
                ("units", C.c_char_p), ("axis", C.POINTER(GridAxis))]


class Iteration(C.Structure):
    _fields_ = [("name", C.c_char_p), ("n", C.c_int32), ("t", C.c_double), ("time_units", C.c_char_p)]


class PartInfo(C.Structure):
    _fields_ = [("name", C.c_char_p), ("label", C.c_char_p), ("np", C.c_uint64), ("nquants", C.c_uint32),
                ("quants", C.POINTER(C.c_char_p)), ("qlabels", C.POINTER(C.c_char_p)),
                ("qunits", C.POINTER(C.c_char_p))]


class File(C.Structure):
    _fields_ = [("fp", C.c_void_p), ("mode", C.c_int), ("ndatasets", C.c_uint32)]


class Dataset(C.Structure):
    _fields_ = [("name", C.c_char_p), ("data_type", C.c_int), ("ndims", C.c_uint32), ("count", C.c_uint64 * 3),
                ("data", C.c_void_p), ("id", C.c_uint64), ("offset", C.c_uint64)]


class Chunk(C.Structure):
    _fields_ = [("count", C.c_uint64 * 3), ("start", C.c_uint64 * 3), ("stride", C.c_uint64 * 3),
                ("data", C.c_void_p)]


# the simulation of the report fixtures: a plasma with a moving window and
# a laser, so that the window offset shows in the charge axis
REPORT_DECK = dict(
    nx=[64, 8], box=[1.28, 1.6], dt=0.014,
    species=[dict(name="electrons", m_q=-1.0, ppc=[2, 2], uth=[0.02, 0.02, 0.02],
                  density=dict(type="step", start=0.6))],
    laser=dict(type="gaussian", start=0.5, fwhm=0.3, a0=1.0, omega0=10.0, W0=0.8, focus=0.6, axis=0.8,
               polarization=0.0),
    moving_window=True,
    smooth=dict(xtype="binomial", xlevel=1),
    steps=30)
REPORT_STEPS = 30
PHA_NX = (32, 16)
PHA_RANGE = ((0.0, 1.6), (-0.2, 0.2))
PHA_TYPE = 0x2000 + 1 + 4 * 16  # PHASESPACE(X1, U1)


def bind(lib):
    """Sets the signatures of the ZDF entry points of `lib` (either library)."""
    P = C.c_void_p
    sig = {
        "zdf_save_grid": (C.c_int, [P, C.c_int, C.POINTER(GridInfo), C.POINTER(Iteration), C.c_char_p]),
        "zdf_open_part_file": (C.c_int, [C.POINTER(File), C.POINTER(PartInfo), C.POINTER(Iteration), C.c_char_p]),
        "zdf_add_quant_part_file": (C.c_int, [C.POINTER(File), C.c_char_p, P, C.c_uint64]),
        "zdf_open_file": (C.c_int, [C.POINTER(File), C.c_char_p, C.c_int]),
        "zdf_close_file": (C.c_int, [C.POINTER(File)]),
        "zdf_add_string": (C.c_size_t, [C.POINTER(File), C.c_char_p, C.c_char_p]),
        "zdf_add_int32": (C.c_size_t, [C.POINTER(File), C.c_char_p, C.c_int32]),
        "zdf_add_double": (C.c_size_t, [C.POINTER(File), C.c_char_p, C.c_double]),
        "zdf_add_iteration": (C.c_size_t, [C.POINTER(File), C.POINTER(Iteration)]),
        "zdf_start_cdset": (C.c_size_t, [C.POINTER(File), C.POINTER(Dataset)]),
        "zdf_write_cdset": (C.c_size_t, [C.POINTER(File), C.POINTER(Dataset), C.POINTER(Chunk)]),
        "zdf_end_cdset": (C.c_size_t, [C.POINTER(File), C.POINTER(Dataset)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def _b(s):
    return s.encode() if s is not None else None


def _iteration(n, t, units="1/\\omega_p"):
    return Iteration(b"ITERATION", n, t, _b(units))


def case_grid2d(lib, root):
    data = (np.arange(24 * 10, dtype=np.float32).reshape(10, 24) * np.float32(0.37) - np.float32(7.5)) ** 2
    axis = (GridAxis * 2)(GridAxis(b"x", 0, 0.0, 2.4, b"x", b"c/\\omega_p"),
                          GridAxis(b"y", 0, -0.5, 0.5, b"y", b"c/\\omega_p"))
    info = GridInfo(b"E1", 2, (C.c_uint64 * 3)(24, 10, 0), b"E_y", b"m_e c \\omega_p e^{-1}", axis)
    it = _iteration(120, float(np.float32(120) * np.float32(0.07)))
    assert lib.zdf_save_grid(data.ctypes.data_as(C.c_void_p), 9, C.byref(info), C.byref(it),
                             os.path.join(root, "EMF").encode())
    return os.path.join("EMF", "E1-000120.zdf")


def case_grid1d_f64_noaxis(lib, root):
    data = np.linspace(-1.0, 3.0, 13)
    info = GridInfo(b"line", 1, (C.c_uint64 * 3)(13, 0, 0), b"a line", None, None)
    it = _iteration(7, 0.125, None)
    assert lib.zdf_save_grid(data.ctypes.data_as(C.c_void_p), 10, C.byref(info), C.byref(it),
                             os.path.join(root, "deep", "er", "path").encode())
    return os.path.join("deep", "er", "path", "line-000007.zdf")


def case_grid3d_int(lib, root):
    data = (np.arange(3 * 4 * 5) - 17).astype(np.int16).reshape(5, 4, 3)
    axis = (GridAxis * 3)(GridAxis(b"a", 1, 1.0, 10.0, b"A", b""), GridAxis(b"b", 2, 0.0, 1.0, b"B", b"u"),
                          GridAxis(b"c", 0, -3.0, 3.0, b"C", b"units c"))
    info = GridInfo(b"cube", 3, (C.c_uint64 * 3)(3, 4, 5), b"cube label", b"cu", axis)
    it = _iteration(0, 0.0)
    assert lib.zdf_save_grid(data.ctypes.data_as(C.c_void_p), 3, C.byref(info), C.byref(it), root.encode())
    bytes8 = np.arange(7, dtype=np.uint8) * 31
    info8 = GridInfo(b"bytes", 1, (C.c_uint64 * 3)(7, 0, 0), b"odd length", b"", None)
    assert lib.zdf_save_grid(bytes8.ctypes.data_as(C.c_void_p), 2, C.byref(info8), C.byref(it), root.encode())
    return [os.path.join("cube-000000.zdf"), os.path.join("bytes-000000.zdf")]


def case_particles(lib, root):
    n = 37
    rng = np.random.default_rng(3)
    cols = [rng.standard_normal(n).astype(np.float32) for _ in range(5)]
    q = (C.c_char_p * 5)(b"x", b"y", b"ux", b"uy", b"uz")
    ql = (C.c_char_p * 5)(b"x", b"y", b"u_x", b"u_y", b"u_z")
    qu = (C.c_char_p * 5)(b"c/\\omega_p", b"c/\\omega_p", b"c", b"c", b"c")
    info = PartInfo(b"electrons", b"electrons", n, 5, q, ql, qu)
    it = _iteration(33, 1.65)
    f = File()
    assert lib.zdf_open_part_file(C.byref(f), C.byref(info), C.byref(it),
                                  os.path.join(root, "PARTICLES", "electrons").encode())
    for name, col in zip([b"x", b"y", b"ux", b"uy", b"uz"], cols):
        assert lib.zdf_add_quant_part_file(C.byref(f), name, col.ctypes.data_as(C.c_void_p), n)
    assert lib.zdf_close_file(C.byref(f))
    return os.path.join("PARTICLES", "electrons", "particles-electrons-000033.zdf")


def case_records_chunked(lib, root):
    fn = os.path.join(root, "records.zdf")
    f = File()
    assert lib.zdf_open_file(C.byref(f), fn.encode(), 0)
    assert lib.zdf_add_string(C.byref(f), b"TYPE", b"chunked test")
    assert lib.zdf_add_string(C.byref(f), b"EMPTY", None)
    assert lib.zdf_add_int32(C.byref(f), b"an int", -123456)
    assert lib.zdf_add_double(C.byref(f), b"a double", 2.718281828459045)
    it = _iteration(9, 0.9)
    assert lib.zdf_add_iteration(C.byref(f), C.byref(it))
    ds = Dataset(b"DATA", 9, 2, (C.c_uint64 * 3)(8, 6, 0), None, 0, 0)
    assert lib.zdf_start_cdset(C.byref(f), C.byref(ds))
    full = np.arange(48, dtype=np.float32).reshape(6, 8) / np.float32(3)
    keep = []
    for r0 in (0, 2, 4):
        part = np.ascontiguousarray(full[r0:r0 + 2])
        keep.append(part)
        ch = Chunk((C.c_uint64 * 3)(8, 2, 0), (C.c_uint64 * 3)(0, r0, 0), (C.c_uint64 * 3)(1, 1, 0),
                   part.ctypes.data_as(C.c_void_p))
        assert lib.zdf_write_cdset(C.byref(f), C.byref(ds), C.byref(ch))
    assert lib.zdf_end_cdset(C.byref(f), C.byref(ds))
    assert lib.zdf_close_file(C.byref(f))
    return "records.zdf"


CASES = [case_grid2d, case_grid1d_f64_noaxis, case_grid3d_int, case_particles, case_records_chunked]


def write_all(lib, root):
    """Runs every case below `root`; returns the files written (relative)."""
    out = []
    for case in CASES:
        r = case(lib, root)
        out += r if isinstance(r, list) else [r]
    return out
