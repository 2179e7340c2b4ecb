"""Builds libzpic_cuda.so (sm_103a) in-tree with nvcc.

    python -m zpic_gb300.build          # or zpic_gb300.build.build()

The translation units are compiled in parallel and linked into
``zpic_gb300/lib/libzpic_cuda.so``.  The physics kernels (exact push,
particles, fields) are compiled with ``--fmad=false`` so that every float32
operation rounds as in the reference C code; the fast push build allows FMA
contraction and approximate float32 division / square root; the host runtime
uses the defaults.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = [
    ("zc_push_exact.cu", ["--fmad=false"]),
    ("zc_push_fast.cu", ["--fmad=true", "--prec-div=false", "--prec-sqrt=false"]),
    ("zc_push_exact_det.cu", ["--fmad=false"]),
    ("zc_push_fast_det.cu", ["--fmad=true", "--prec-div=false", "--prec-sqrt=false"]),
    ("zc_particles.cu", ["--fmad=false"]),
    ("zc_fields.cu", ["--fmad=false"]),
    ("zc_api.cu", []),
    ("zc_noalloc.cu", []),
    ("zc_adjoint.cu", ["--fmad=false"]),
    ("zc_em1d.cu", ["--fmad=false"]),
]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles and links the library; returns its path."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                     "-I", os.path.join(os.path.dirname(HERE), "include")]
    if ptxas_info:
        common += ["-Xptxas", "-v"]

    def one(unit):
        src, extra = unit
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        out = _run([cc, "-c", os.path.join(CSRC, src), "-o", obj] + common + extra)
        return obj, out

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(one, UNITS))
    objs = [o for o, _ in results]
    if verbose or ptxas_info:
        for _, out in results:
            if out.strip():
                print(out)
    lib = os.path.join(LIBDIR, "libzpic_cuda.so")
    tmp = lib + ".tmp"
    _run([cc] + ARCH + ["-shared", "-o", tmp] + objs)
    os.replace(tmp, lib)
    # the em2d drop-in C API (plain C host code over the C-ABI)
    em2d = os.path.join(LIBDIR, "libzpic_em2d.so")
    _run([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-D_DEFAULT_SOURCE", "-fPIC", "-shared", "-pthread",
          "-fvisibility=hidden", os.path.join(CSRC, "em2d", "em2d_host.c"), os.path.join(CSRC, "em2d", "zdf_io.c"),
          "-o", em2d + ".tmp", "-L", LIBDIR, "-lzpic_cuda", "-Wl,-rpath,$ORIGIN", "-lm"])
    os.replace(em2d + ".tmp", em2d)
    # the em1d drop-in C API over the 1-D step (zc1_*)
    em1d = os.path.join(LIBDIR, "libzpic_em1d.so")
    _run([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-D_DEFAULT_SOURCE", "-fPIC", "-shared", "-pthread",
          "-fvisibility=hidden", os.path.join(CSRC, "em1d", "em1d_host.c"), os.path.join(CSRC, "em2d", "zdf_io.c"),
          "-o", em1d + ".tmp", "-L", LIBDIR, "-lzpic_cuda", "-Wl,-rpath,$ORIGIN", "-lm"])
    os.replace(em1d + ".tmp", em1d)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
