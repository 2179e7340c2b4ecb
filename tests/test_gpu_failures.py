"""Failure statuses of the C-ABI, made on the host.

The kernels report a failed check (a particle moved more than one cell or
left its tile; a bounded barrier wait gave up; the spill list overflowed) by
setting bits of a device error word, which the host reads between steps.
These tests write that word from the host between steps
(``zc_post_device_error``) -- no kernel is made to fail -- and check that:

* ``zc_step`` returns the matching status with a message, eagerly and under
  graph replay;
* the simulation stays usable: the word is cleared, and the next steps still
  follow the oracle;
* an impossible capacity request returns ``ZC_ENOMEM`` before any
  allocation;
* the em2d drop-in turns a failed step into the reference's convention, a
  message on stderr and ``exit(-1)`` (``em2d/simulation.c:106-110``), not a
  crash.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from gpu_util import field_err, mirror

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ESCAPE, TIMEOUT, OVERFLOW = 4, 5, 6
MESSAGES = {ESCAPE: "moved more than one cell", TIMEOUT: "timed out", OVERFLOW: "particles were lost"}


@pytest.mark.parametrize("graphs", [False, True], ids=["eager", "graphs"])
@pytest.mark.parametrize("status", [ESCAPE, TIMEOUT, OVERFLOW], ids=["escape", "timeout", "overflow"])
def test_posted_device_error_is_reported_and_cleared(status, graphs):
    from zpic_gb300._zc import ZcError

    cpu, g = mirror("weibel_smooth")
    try:
        g.set_graphs(graphs)
        n = 16 if graphs else 1  # a whole block under replay
        cpu.iter(n)
        g.step(n)
        assert g.lib.zc_post_device_error(g.h, status) == 0
        with pytest.raises(ZcError) as exc:
            g.step(n)
        assert exc.value.status == status
        assert MESSAGES[status] in g.lib.zc_last_error().decode()
        cpu.iter(n)  # the failed call still ran its steps
        # the word was cleared: the run goes on, on the oracle's track
        for _ in range(2):
            cpu.iter(n)
            g.step(n)
        for f in ("E", "B", "J"):
            assert field_err(getattr(g, f)(), getattr(cpu, f)()) <= 1e-5, f
        assert g.count(0) == cpu.np_(0)
    finally:
        g.close()


def test_post_rejects_host_side_statuses():
    _, g = mirror("thermal")
    try:
        assert g.lib.zc_post_device_error(g.h, 1) == 1  # ZC_EINVAL cannot be posted
        assert g.lib.zc_post_device_error(None, ESCAPE) == 1
        g.step(1)  # nothing was posted
    finally:
        g.close()


def test_impossible_capacity_is_enomem():
    from zpic_gb300._zc import CudaSim, ZcError

    from decks import build_cpu

    cpu = build_cpu("thermal")
    # a tile slack of 1e9 asks for tiles of about 10^11 particles: refused on
    # the host before anything is allocated
    g = CudaSim(cpu.nx, cpu.box, cpu.dt, tile_slack=1e9)
    try:
        with pytest.raises(ZcError) as exc:
            g.add_species(-1.0, cpu.q(0), (4, 4), cpu.particles(0))
        assert exc.value.status == 2
        assert "too large" in g.lib.zc_last_error().decode()
    finally:
        g.close()


_CHILD = r"""
import ctypes, sys
sys.path.insert(0, {root!r})
from zpic_gb300 import em2d
sim = em2d.Simulation([32, 24], [3.2, 2.4], 0.07,
                      species=[em2d.Species("e", -1.0, [2, 2], uth=[0.1, 0.1, 0.1])])
sim.iter()
lib = em2d._load()
print("stepped", flush=True)
# the simulation's C-ABI handle, as the drop-in keeps it
cuda = ctypes.CDLL(em2d._zc.LIB_PATH)
h = lib.sim_gpu_handle(sim._s)
cuda.zc_post_device_error.argtypes = [ctypes.c_void_p, ctypes.c_int]
assert cuda.zc_post_device_error(h, {status}) == 0
lib.sim_iter(sim._s)
print("not reached", flush=True)
"""


def test_em2d_drop_in_exits_like_the_reference():
    code = _CHILD.format(root=ROOT, status=ESCAPE)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert "stepped" in r.stdout, r.stderr
    assert "not reached" not in r.stdout
    assert r.returncode == 255, (r.returncode, r.stderr[-2000:])  # exit(-1)
    assert "(*error*) sim_iter" in r.stderr and "moved more than one cell" in r.stderr


def test_queued_steps_report_errors_at_the_next_wait():
    """zc_step_async returns without waiting: a device error of a queued step
    comes back from the next waiting call, and the run goes on."""
    from zpic_gb300._zc import ZcError

    cpu, g = mirror("weibel_smooth")
    try:
        cpu.iter(2)
        g.step_async(2)
        assert g.lib.zc_post_device_error(g.h, ESCAPE) == 0
        g.step_async(1)  # queued: no status yet
        cpu.iter(1)
        with pytest.raises(ZcError) as exc:
            g.synchronize()
        assert exc.value.status == ESCAPE
        cpu.iter(3)
        g.step_async(3)
        g.synchronize()
        for f in ("E", "B", "J"):
            assert field_err(getattr(g, f)(), getattr(cpu, f)()) <= 1e-5, f
    finally:
        g.close()
