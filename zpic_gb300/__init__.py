"""zpic_gb300 -- the ZPIC em2d electromagnetic PIC step on GB300 (sm_103a).

Layers:
  libzpic_cuda (zpic_gb300/lib, built from zpic_gb300/csrc): the C-ABI of
      include/zpic_cuda.h over hand-written CUDA kernels;
  zpic_gb300._zc.CudaSim: ctypes binding of that ABI.
"""
__all__ = ["CudaSim", "ZcError"]


def __getattr__(name):
    if name in ("CudaSim", "ZcError"):
        from . import _zc

        return getattr(_zc, name)
    raise AttributeError(name)
