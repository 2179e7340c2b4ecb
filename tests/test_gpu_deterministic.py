"""Deterministic mode (zc_sim_desc.deterministic): currents and kinetic
energies are summed as 64-bit fixed-point integers, so runs are
bit-reproducible -- run to run, with or without graph replay, and (exact
push) whatever the tile shape -- and still match the oracle within the
forward tolerance."""
import numpy as np
import pytest

from decks import DECKS
from gpu_util import canon, field_err, mirror

pytestmark = pytest.mark.gpu


def _state(g, n_species):
    emf, kin = g.energy()
    return {"E": g.E(), "B": g.B(), "J": g.J(), "emf": emf, "kin": kin,
            "parts": [canon(g.particles(k)) for k in range(n_species)]}


def _same(a, b):
    for f in ("E", "B", "J", "emf", "kin"):
        assert np.array_equal(a[f], b[f]), f
    for pa, pb in zip(a["parts"], b["parts"]):
        assert pa.tobytes() == pb.tobytes()


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
@pytest.mark.parametrize("name", ["weibel_smooth", "thermal", "lwfa_window"])
def test_runs_are_bit_identical(name, fast):
    n = len(DECKS[name]["species"])
    runs = []
    for _ in range(2):
        cpu, g = mirror(name, deterministic=True, fast_math=fast)
        g.step(12)
        runs.append(_state(g, n))
    _same(runs[0], runs[1])


def test_tile_shape_and_graphs_do_not_change_bits():
    n = 2
    ref = None
    for tile, graphs in (((16, 16), False), ((8, 8), False), ((32, 16), True), ((16, 8), True)):
        cpu, g = mirror("weibel_smooth", tile=tile, deterministic=True, sort_every=2)
        g.set_graphs(graphs)
        g.step(13)
        st = _state(g, n)
        if ref is None:
            ref = st
        else:
            _same(ref, st)


@pytest.mark.parametrize("name", ["weibel_smooth", "thermal", "custom_ext", "lwfa_window", "window_smooth_xy"])
def test_deterministic_matches_oracle(name):
    cpu, g = mirror(name, deterministic=True)
    for step in range(10):
        cpu.iter()
        g.step(1)
        for f in ("E", "B"):
            err = field_err(getattr(g, f)(), getattr(cpu, f)())
            assert err <= 1e-5, f"{f} relative error {err:.2e} at step {step}"
        # J: every contribution is rounded to a multiple of 2^-40, an
        # absolute resolution that shows where the whole current is tiny
        # (a cold plasma the laser has only begun to reach)
        jg, jc = g.J(), cpu.J()
        assert np.abs(jg - jc).max() <= 1e-5 * np.abs(jc).max() + 1e-9, f"J at step {step}"
    emf_g, kin_g = g.energy()
    for k in range(cpu.n_species):
        assert abs(kin_g[k] - cpu.energy(k)) <= 1e-5 * abs(cpu.energy(k))


def test_queued_steps_and_energies_match_waiting_ones():
    """zc_step_async + zc_energy_async (one wait at the end) give the bits
    of zc_step + zc_energy, energies of every step included; 20 queued
    steps cross the wait every 16 steps."""
    import torch

    name = "thermal"
    rows = []
    for queued in (False, True):
        cpu, g = mirror(name, deterministic=True)
        out = torch.zeros((20, 7), dtype=torch.float64, pin_memory=True).numpy()
        for i in range(20):
            if queued:
                g.step_async(1)
                g.energy_async(out[i])
            else:
                g.step(1)
                emf, kin = g.energy()
                out[i, :6], out[i, 6] = emf, kin[0]
        g.synchronize()
        rows.append((out.copy(), g.E(), g.B()))
        g.close()
    for a, b in zip(rows[0], rows[1]):
        assert np.array_equal(a, b)


def test_graphs_with_timed_push_keep_bits_and_time_every_push():
    """Push-only profiling under graph replay: the blocks carry event-record
    nodes around every push.  The run keeps the bits of an eager untimed run,
    and every push of the call is timed (eager steps before the first block
    boundary and after the last, nodes in between)."""
    name = "weibel_smooth"
    n = len(DECKS[name]["species"])
    states = []
    for graphs, prof in ((False, False), (True, "push")):
        cpu, g = mirror(name, deterministic=True, sort_every=2)
        g.set_graphs(graphs)
        g.step(3)
        g.set_profiling(prof)
        g.reset_profile()
        g.step(22)  # 1 eager step, 5 blocks of 4 steps, 1 eager step
        p = g.profile()
        if prof:
            ms, launches = p["push"]
            assert launches == 22 * n
            assert ms > 0
        states.append(_state(g, n))
        g.close()
    _same(states[0], states[1])


def test_history_streamed_to_host_rows_matches_device_history():
    """zc_history_stream: every step writes its energy row into page-locked
    host rows, also inside replayed graphs and queued steps; the rows equal
    the device-side history's bits (and zc_energy's values to 1e-6: that sums
    the field energy over more blocks).  Pageable rows are refused."""
    import torch
    from zpic_gb300._zc import ZcError

    name, steps = "weibel_smooth", 21
    n = len(DECKS[name]["species"])
    out = []
    for stream in (False, True):
        cpu, g = mirror(name, deterministic=True, sort_every=2)
        g.set_graphs(True)
        if stream:
            rows = torch.zeros((steps, 6 + n), dtype=torch.float64, pin_memory=True).numpy()
            with pytest.raises(ZcError):
                g.history_stream(np.zeros((steps, 6 + n)))
            g.history_stream(rows)
            g.step_async(steps)
            g.synchronize()
            assert len(g.history()) == steps
            hist = rows.copy()
        else:
            g.history_enable(steps)
            g.step(steps)
            hist = g.history()
        emf, kin = g.energy()
        # (the history sums the field energy over fewer blocks than zc_energy)
        assert np.allclose(hist[-1], np.concatenate([emf, kin]), rtol=1e-6, atol=0)
        out.append(hist)
        g.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("groups", [1, 2, 3])
def test_batch_gives_the_bits_of_runs_alone(groups):
    """Three different runs batched (in one, two or three groups on their own
    streams; 13 steps: three 4-step blocks and a 1-step tail) end with the
    bits of the same runs stepped alone."""
    from zpic_gb300._zc import CudaBatch

    names = ("weibel_smooth", "thermal", "custom_ext")
    alone = []
    for name in names:
        _, g = mirror(name, deterministic=True, sort_every=2)
        g.step(13)
        alone.append(_state(g, len(DECKS[name]["species"])))
        g.close()
    sims = [mirror(name, deterministic=True, sort_every=2)[1] for name in names]
    b = CudaBatch(sims, groups=groups)
    b.step(13)
    for name, g, ref in zip(names, sims, alone):
        _same(ref, _state(g, len(DECKS[name]["species"])))
    b.close()
