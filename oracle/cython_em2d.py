"""The reference's own Cython em2d module built against the em2d drop-in
(TEST INFRASTRUCTURE ONLY).

The reference's Python layer (``python/source/em2d.pyx`` with its
``em2d.pxd``) is a caller of the em2d C API.  Here it is built unmodified
against the drop-in's headers (``include/em2d``) and library
(``libzpic_em2d``) in place of the reference's C sources, so that tests can
drive the drop-in exactly as the reference's Python users do.

* ``generate()`` -- where the reference tree and Cython are present,
  translates the ``.pyx`` to C with the directive
  ``legacy_implicit_noexcept`` (Cython 3 rejects the module's callbacks
  without it; the reference pins Cython 0.29) into
  ``oracle/_ref/em2d_cython/python/source/em2d.c``.  ``oracle/_ref`` holds
  only build outputs of the reference and stays out of version control.
* ``compile()`` -- wherever that C file exists, compiles it with the Python
  headers and links it to ``libzpic_em2d``.  The module's
  ``#include "../../em2d/<header>"`` lines resolve through a link
  ``oracle/_ref/em2d_cython/em2d`` to ``include/em2d``.
* ``load()`` -- imports the built module (``em2d_ref``) or returns None.
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sysconfig

from oracle.pyoracle import REFERENCE_ROOT

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref", "em2d_cython")
SRC_DIR = os.path.join(OUT, "python", "source")
C_FILE = os.path.join(SRC_DIR, "em2d.c")
LIBDIR = os.path.join(ROOT, "zpic_gb300", "lib")


def _module_path() -> str:
    return os.path.join(OUT, "em2d" + sysconfig.get_config_var("EXT_SUFFIX"))


def generate() -> bool:
    """Translates the reference's module to C; False where the reference
    tree or Cython is missing."""
    src = os.path.join(REFERENCE_ROOT, "python", "source")
    if not os.path.isfile(os.path.join(src, "em2d.pyx")):
        return False
    try:
        from Cython.Build import cythonize
        from Cython.Compiler import Options  # noqa: F401
    except ImportError:
        return False
    os.makedirs(SRC_DIR, exist_ok=True)
    for f in ("em2d.pyx", "em2d.pxd"):
        dst = os.path.join(SRC_DIR, f)
        if not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(os.path.join(src, f)):
            shutil.copyfile(os.path.join(src, f), dst)
    cythonize([os.path.join(SRC_DIR, "em2d.pyx")], quiet=True, language_level="3str",
              compiler_directives={"legacy_implicit_noexcept": True})
    return os.path.isfile(C_FILE)


def compile() -> str | None:
    """Builds the extension module from the translated C file; returns its
    path, or None when there is no C file."""
    if not os.path.isfile(C_FILE):
        return None
    link = os.path.join(OUT, "em2d")
    if not os.path.islink(link):
        if os.path.lexists(link):
            os.remove(link)
        os.symlink(os.path.join(ROOT, "include", "em2d"), link)
    out = _module_path()
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(C_FILE),
                                                           os.path.getmtime(os.path.join(LIBDIR,
                                                                                         "libzpic_em2d.so"))):
        return out
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", "-I", sysconfig.get_paths()["include"], C_FILE,
           "-L", LIBDIR, "-lzpic_em2d", "-Wl,-rpath," + LIBDIR, "-lm", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference's em2d module against the drop-in failed:\n" + r.stderr[-4000:])
    return out


def load():
    """The reference's em2d module linked to the drop-in, or None."""
    path = _module_path()
    if not os.path.exists(path):
        return None
    spec = importlib.util.spec_from_file_location("em2d", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod
