"""Graph replay, the per-step energy history and batched runs against the
oracle: captured blocks of steps and batches of runs must give the results
of eager steps of each run alone."""
import numpy as np
import pytest

from decks import DECKS, build_cpu
from gpu_util import field_err, mirror

pytestmark = pytest.mark.gpu


def _check(cpu, g, tol=1e-5):
    for f in ("E", "B", "J"):
        err = field_err(getattr(g, f)(), getattr(cpu, f)())
        assert err <= tol, f"{f} relative error {err:.2e}"
    emf_g, kin_g = g.energy()
    emf_c = cpu.emf_energy()
    assert np.all(np.abs(emf_g - emf_c) <= tol * np.abs(emf_c).max() + 1e-30)
    for k in range(cpu.n_species):
        assert abs(kin_g[k] - cpu.energy(k)) <= tol * abs(cpu.energy(k))
        assert g.count(k) == cpu.np_(k)


@pytest.mark.parametrize("name", ["thermal", "weibel_smooth", "custom_ext"])
def test_graph_steps_match_oracle(name):
    """Blocks of 4 steps (sort every 2) replayed as graphs; the calls start
    on and off a block boundary and end with eager steps."""
    cpu, g = mirror(name, sort_every=2)
    g.set_graphs(True)
    done = 0
    for n in (9, 6, 1, 4):
        g.step(n)
        cpu.iter(n)
        done += n
        assert g.info()["iter"] == done
        _check(cpu, g)


def test_graph_recaptures_after_reconfiguration():
    cpu, g = mirror("thermal", sort_every=1)
    g.set_graphs(True)
    g.step(4)
    cpu.iter(4)
    # new particle layout and new smoothing: the captured block is stale
    parts = cpu.particles(0)
    g.set_particles(0, parts)
    cpu.set_smooth("binomial", 2, "none", 0)
    g.set_smooth("binomial", 2, "none", 0)
    g.step(6)
    cpu.iter(6)
    _check(cpu, g)


def test_history_matches_oracle_energies():
    cpu, g = mirror("weibel_smooth")
    g.history_enable(12)
    rows = []
    for _ in range(10):
        cpu.iter()
        rows.append(np.concatenate([cpu.emf_energy(), [cpu.energy(k) for k in range(cpu.n_species)]]))
    g.step(10)
    h = g.history()
    assert h.shape == (10, 6 + 2)
    want = np.array(rows)
    scale = np.abs(want).max(axis=0) + 1e-30
    assert np.all(np.abs(h - want) <= 1e-5 * scale)
    # rows past the capacity are dropped, reset starts over
    g.step(5)
    assert g.history().shape[0] == 12
    g.history_reset()
    g.step(1)
    assert g.history().shape[0] == 1


def test_history_under_graphs():
    cpu, g = mirror("thermal", sort_every=2)
    g.set_graphs(True)
    g.history_enable(16)
    g.step(13)
    e = []
    for _ in range(13):
        cpu.iter()
        e.append(cpu.emf_energy().sum())
    h = g.history()
    assert h.shape[0] == 13
    assert np.allclose(h[:, :6].sum(axis=1), e, rtol=1e-5, atol=1e-30)


@pytest.mark.parametrize("groups", [None, 2, 3])
def test_batch_matches_runs_alone(groups):
    """Three different runs in one batch (one group, or the members dealt
    into two or three groups on their own streams), one of them started off
    a block boundary, each checked against its own oracle run."""
    from zpic_gb300._zc import CudaBatch

    pairs = [mirror(n, sort_every=2) for n in ("thermal", "weibel_smooth", "custom_ext")]
    cpu1, g1 = pairs[1]
    g1.step(3)
    cpu1.iter(3)
    for cpu, g in pairs:
        g.history_enable(64)
    b = CudaBatch([g for _, g in pairs], groups=groups)
    assert b.groups == (groups or 1)
    b.step(11)
    b.step(5)
    assert b.last_ms() > 0
    for cpu, g in pairs:
        cpu.iter(16)
        _check(cpu, g)
    assert pairs[0][1].history().shape[0] == 16
    assert pairs[1][1].history().shape[0] == 16
    b.close()


def test_batch_rejects_mixed_block_lengths():
    from zpic_gb300._zc import CudaBatch, ZcError

    _, a = mirror("thermal", sort_every=2)
    _, b = mirror("thermal", sort_every=4)
    with pytest.raises(ZcError):
        CudaBatch([a, b])
    _, c = mirror("lwfa_window")
    with pytest.raises(ZcError):
        CudaBatch([a, c])


def test_scan_batched_equals_sequential():
    """A small scan of the same loaded runs, batched and one by one."""
    from zpic_gb300 import batch

    runs = batch.weibel_scan(n_runs=5, steps=24, nx_range=(32, 48), ppc_range=(2, 3), seed=7)
    a = batch.load_sims(runs, tile=(16, 16), sort_every=2, workers=3)
    b = batch.load_sims(runs, tile=(16, 16), sort_every=2, workers=1)
    ra = batch.run_batched(a, runs, group=3)
    rb = batch.run_sequential(b, runs)
    assert ra.groups == 2
    for ha, hb in zip(ra.histories, rb.histories):
        assert ha.shape == hb.shape == (24, 8)
        tot_a, tot_b = ha.sum(axis=1), hb.sum(axis=1)
        assert np.allclose(tot_a, tot_b, rtol=1e-5)
    for s in a + b:
        s.close()


@pytest.mark.parametrize("groups", [1, 2])
def test_batch_member_relayout_between_steps(groups):
    """A member re-laid out between batch steps is captured again and its
    branch of its group's graph updated."""
    from zpic_gb300._zc import CudaBatch

    pairs = [mirror(n, sort_every=2) for n in ("thermal", "weibel_smooth")]
    b = CudaBatch([g for _, g in pairs], groups=groups)
    b.step(8)
    for cpu, g in pairs:
        cpu.iter(8)
    cpu0, g0 = pairs[0]
    before = g0.info()["captures"]
    g0.set_particles(0, cpu0.particles(0))
    b.step(8)
    for cpu, g in pairs:
        cpu.iter(8)
        _check(cpu, g)
    assert g0.info()["captures"] > before
    assert g0.info()["relayouts"] >= 2
    b.close()


def _cluster(n, ix, iy, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(n, dtype=[("ix", "<i4"), ("iy", "<i4"), ("x", "<f4"), ("y", "<f4"),
                           ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])
    a["ix"], a["iy"] = ix, iy
    a["x"] = rng.uniform(0, 1, n).astype(np.float32)
    a["y"] = rng.uniform(0, 1, n).astype(np.float32)
    for f in ("ux", "uy", "uz"):
        a[f] = rng.normal(0, 0.05, n).astype(np.float32)
    return a


@pytest.mark.parametrize("graphs", [False, True])
def test_spill_path_matches_oracle(graphs):
    """Particles beyond a tile's capacity go to the spill list and are
    advanced there; a re-layout drains the list once it holds enough."""
    cpu, g = mirror("thermal", sort_every=2)
    g.set_graphs(graphs)
    base = cpu.particles(0)
    few = _cluster(2500, 5, 5, 1)          # more than the tile's spare room
    g.inject(0, few)
    cpu.set_particles(0, np.concatenate([base, few]))
    r0 = g.info()["relayouts"]
    for n in (3, 5):
        g.step(n)
        cpu.iter(n)
        _check(cpu, g)
    assert g.info()["relayouts"] == r0      # a short spill list stays
    more = _cluster(5000, 20, 9, 2)        # with the first, past the drain threshold
    g.inject(0, more)
    cpu.set_particles(0, np.concatenate([cpu.particles(0), more]))
    assert g.info()["relayouts"] > r0       # a long one is drained
    g.step(8)
    cpu.iter(8)
    _check(cpu, g)


def test_batch_groups_with_spilled_member():
    """Four runs dealt into two groups, one holding more particles in a tile
    than the tile has room for (its spill list is advanced beside the tiles):
    each run still gives its oracle run's results, and regrouping between
    calls changes nothing."""
    from zpic_gb300._zc import CudaBatch

    pairs = [mirror(n, sort_every=2) for n in ("thermal", "weibel_smooth", "thermal", "custom_ext")]
    cpu0, g0 = pairs[0]
    few = _cluster(2500, 5, 5, 3)
    g0.inject(0, few)
    cpu0.set_particles(0, np.concatenate([cpu0.particles(0), few]))
    b = CudaBatch([g for _, g in pairs], groups=2)
    b.step(8)
    for cpu, g in pairs:
        cpu.iter(8)
        _check(cpu, g)
    b.set_groups(0)
    assert b.groups == 1
    b.set_groups(9)
    assert b.groups == 4
    b.step(10)
    for cpu, g in pairs:
        cpu.iter(10)
        _check(cpu, g)
    b.close()


@pytest.mark.parametrize("groups", [1, 2])
def test_batch_member_spills_while_stepping(groups):
    """A dense cluster streams (ux = 2) from one tile into its neighbour,
    which has no room for it, while the batch runs: its particles go to the
    spill list, the batch drains every group's stream and re-lays the member
    out between blocks, and every run still gives its oracle run's results."""
    from zpic_gb300._zc import CudaBatch

    pairs = [mirror(n, sort_every=2) for n in ("thermal", "weibel_smooth", "thermal")]
    cpu0, g0 = pairs[0]
    jet = _cluster(6000, 14, 8, 4)
    jet["ux"] += np.float32(2.0)
    g0.inject(0, jet)
    cpu0.set_particles(0, np.concatenate([cpu0.particles(0), jet]))
    r0 = g0.info()["relayouts"]
    b = CudaBatch([g for _, g in pairs], groups=groups)
    b.step(16)
    assert g0.info()["relayouts"] > r0, "the cluster's spill list was drained inside the batch"
    for cpu, g in pairs:
        cpu.iter(16)
        _check(cpu, g)
    b.close()
