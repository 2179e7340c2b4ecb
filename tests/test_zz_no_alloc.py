"""zc_field_energy_static -- the field-energy entry point that allocates no
device memory -- against zc_energy on the same fields, through the C-ABI.

It is meant for callers whose time loop must not call cudaMalloc/cudaFree:
their device memory is already owned by another allocator, or they cannot
afford the device synchronisation those calls bring.  The caller owns the
field planes and the 6-double output; the library's scratch is a fixed device
array shared by every call.

Tolerance: relative 1e-6 per component, the energy tolerance of the other GPU
tests (both reductions use float Kahan partials and FP64 sums, grouped
differently).  This file is collected last so that a stop at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(nx, ny, seed):
    rng = np.random.default_rng(seed)
    shape = (ny + 3, nx + 3, 3)
    return (rng.standard_normal(shape).astype(np.float32),
            (0.5 * rng.standard_normal(shape)).astype(np.float32))


def _call_static(g, nx, ny, out, plane=None):
    v = g.grid_view()
    dx = np.float32(g.box[0]) / np.float32(nx)
    dy = np.float32(g.box[1]) / np.float32(ny)
    return g.lib.zc_field_energy_static(ctypes.c_void_p(v.E), ctypes.c_void_p(v.B),
                                        v.plane if plane is None else plane, v.pitch, nx, ny,
                                        float(dx), float(dy), ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(v.stream))


def test_static_energy_matches_zc_energy_on_two_calls():
    torch = pytest.importorskip("torch")
    from zpic_gb300._zc import CudaSim

    out = torch.zeros(6, dtype=torch.float64, device="cuda:0")  # caller-owned output
    # torch zero-fills `out` on its own stream; the library writes it on the
    # simulation's stream, so the fill must be finished first
    torch.cuda.synchronize()
    # the second grid is smaller: rows left in the shared scratch by the first
    # call must not leak into the second result
    for call, (nx, ny, seed) in enumerate(((96, 64, 1), (40, 24, 2))):
        g = CudaSim([nx, ny], [nx * 0.1, ny * 0.1], 0.05)
        E, B = _fields(nx, ny, seed)
        g.set_fields(E=E, B=B)
        ref, _ = g.energy()
        g.synchronize()
        free_before = torch.cuda.mem_get_info(0)[0]
        st = _call_static(g, nx, ny, out)
        assert st == 0, g.lib.zc_last_error().decode()
        g.synchronize()
        if call:  # after the first call's one-time set-up: no device memory taken
            assert torch.cuda.mem_get_info(0)[0] == free_before
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-6)
        g.close()


def test_static_energy_rejects_grid_beyond_fixed_scratch():
    torch = pytest.importorskip("torch")
    from zpic_gb300._zc import CudaSim

    out = torch.zeros(6, dtype=torch.float64, device="cuda:0")
    g = CudaSim([16, 16], [1.6, 1.6], 0.05)
    v = g.grid_view()
    ny = 8193  # one row beyond ZC_STATIC_MAX_ROWS; rejected before any launch
    st = _call_static(g, 16, ny, out, plane=v.pitch * (ny + 3))
    assert st == 1
    assert b"8192" in g.lib.zc_last_error()
    g.close()
