"""Parity of the CUDA path (through the C-ABI) with the CPU oracle.

Bars (written per test):
* particle push, current fold/smoothing, Yee advance: bit-exact for the
  same inputs (the kernels are compiled without FMA contraction and restate
  the reference operation by operation);
* deposited current: relative L2 error <= 1e-5 (the GPU adds the per-particle
  contributions in a different order; thermal currents largely cancel within
  a cell, so the rounding of the partial sums shows up relative to a small
  net current);
* full steps: per-step field relative L2 error <= 1e-5 over the first 10
  steps (the bar of the specification), for every field as a whole and for
  every component, except where the oracle itself, run with its particles
  in another buffer order, drifts by about as much: the weak plasma Ex
  beside the plane laser moves by 9.8e-6 from reordering alone, and both
  push builds (1.2e-5 exact, 1.3e-5 FMA) are held to twice that floor;
* energies: relative error <= 1e-6.
"""
import numpy as np
import pytest

from decks import DECKS, build_cpu
from gpu_util import canon, check_fields, field_err, field_err_joint, mirror, reordered_twin

pytestmark = pytest.mark.gpu


def _random_fields(cpu, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    nx, ny = cpu.nx
    E = (amp * rng.standard_normal((ny + 3, nx + 3, 3))).astype(np.float32)
    B = (amp * rng.standard_normal((ny + 3, nx + 3, 3))).astype(np.float32)
    return E, B


@pytest.mark.parametrize("tile", [(16, 16), (8, 8), (32, 16)])
def test_push_bit_exact_and_deposit(tile):
    cpu = build_cpu("weibel_smooth")
    E, B = _random_fields(cpu, 1)
    cpu.set_E(E)
    cpu.set_B(B)
    cpu, g = mirror("weibel_smooth", tile=tile, cpu=cpu)
    for step in range(3):
        cpu.current_zero()
        g.current_zero()
        for k in range(2):
            cpu.spec_advance(k)
            g.spec_advance(k)
            a, b = canon(cpu.particles(k)), canon(g.particles(k))
            assert a.size == b.size
            assert a.tobytes() == b.tobytes(), f"particles differ (step {step}, species {k})"
        assert field_err(g.J(), cpu.J()) <= 1e-5
        # all guard cells too
        Jc = cpu.J()
        assert np.allclose(g.J(), Jc, rtol=1e-4, atol=1e-5 * np.abs(Jc).max())
        _, kin = g.energy()
        for k in range(2):
            assert abs(kin[k] - cpu.energy(k)) <= 1e-6 * abs(cpu.energy(k))


@pytest.mark.parametrize("name", ["weibel_smooth", "thermal", "plane_slab", "lwfa_window", "window_smooth_xy"])
def test_current_update_bit_exact(name):
    cpu = build_cpu(name)
    cpu, g = mirror(name, cpu=cpu)
    rng = np.random.default_rng(7)
    nx, ny = cpu.nx
    J = rng.standard_normal((ny + 3, nx + 3, 3)).astype(np.float32)
    cpu.set_J(J)
    g.set_J(J)
    cpu.current_update()
    g.current_update()
    assert g.J().tobytes() == cpu.J().tobytes()


@pytest.mark.parametrize("name", ["weibel_smooth", "lwfa_window", "custom_ext"])
def test_emf_advance_bit_exact(name):
    cpu = build_cpu(name)
    E, B = _random_fields(cpu, 3, amp=1.0)
    cpu.set_E(E)
    cpu.set_B(B)
    cpu, g = mirror(name, cpu=cpu)
    rng = np.random.default_rng(5)
    nx, ny = cpu.nx
    J = (0.1 * rng.standard_normal((ny + 3, nx + 3, 3))).astype(np.float32)
    for it in range(25):  # includes window moves for the moving-window deck
        cpu.set_J(J)
        g.set_J(J)
        cpu.emf_advance()
        g.emf_advance()
        assert g.E().tobytes() == cpu.E().tobytes(), it
        assert g.B().tobytes() == cpu.B().tobytes(), it
        assert g.E_part().tobytes() == cpu.E_part().tobytes(), it
        assert g.B_part().tobytes() == cpu.B_part().tobytes(), it


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
@pytest.mark.parametrize("name", sorted(n for n in DECKS if not DECKS[n].get("moving_window")))
def test_steps_match_oracle(name, fast):
    cpu, g = mirror(name, fast_math=fast)
    twin = reordered_twin(name)
    for step in range(10):
        cpu.iter()
        twin.iter()
        g.step(1)
        check_fields(g, cpu, twin, f"at step {step}")
        emf_g, kin_g = g.energy()
        emf_c = cpu.emf_energy()
        assert np.all(np.abs(emf_g - emf_c) <= 1e-5 * np.abs(emf_c).max() + 1e-30)
        for k in range(cpu.n_species):
            assert abs(kin_g[k] - cpu.energy(k)) <= 1e-5 * abs(cpu.energy(k))
            assert g.count(k) == cpu.np_(k)


def test_incoming_list_overflow_matches_oracle():
    """A relativistic beam crossing 32 x 32 tiles: about 800 particles enter
    a tile per step, more than the push lists, so the rest are pushed while
    the outboxes are scanned."""
    # uniform initial fields keep every field component well above the
    # summation-order noise of the beam's current
    d = dict(nx=[64, 64], box=[6.4, 6.4], dt=0.07,
             species=[dict(name="e", m_q=-1.0, ppc=[6, 6], ufl=[10.0, 0.0, 0.0], uth=[0.01, 0.01, 0.01])],
             init_fld=dict(E_type="uniform", E_0=[0.0, 0.05, 0.05], B_type="uniform", B_0=[0.05, 0.05, 0.5]))
    cpu, g = mirror("beam", tile=(32, 32), deck=d)
    for step in range(6):
        cpu.iter()
        g.step(1)
        assert g.count(0) == cpu.np_(0), step
        for f in ("E", "B"):
            err = field_err(getattr(g, f)(), getattr(cpu, f)())
            assert err <= 1e-5, f"{f} relative error {err:.2e} at step {step}"
        err = field_err_joint(g.J(), cpu.J())
        assert err <= 1e-5, f"J relative error {err:.2e} at step {step}"
        _, kin = g.energy()
        assert abs(kin[0] - cpu.energy(0)) <= 1e-5 * abs(cpu.energy(0))


@pytest.mark.parametrize("name", ["lwfa_window", "window_smooth_xy"])
def test_moving_window_matches_oracle(name):
    cpu, g = mirror(name)
    for step in range(40):
        cpu.iter()
        g.step(1)
        assert g.count(0) == cpu.np_(0), step
        for f in ("E", "B"):
            err = field_err(getattr(g, f)(), getattr(cpu, f)())
            assert err <= 1e-5, f"{f} relative error {err:.2e} at step {step}"
    assert g.info()["n_move"] == cpu.n_move()


@pytest.mark.parametrize("name", ["lwfa_window", "window_smooth_xy"])
def test_moving_window_device_injection(name):
    """The window's new column drawn on the device (zc_set_device_injection,
    cold step profile) against the oracle's spec_move_window: the same
    particle counts every step, fields within 1e-5, the particles of the
    injected column identical."""
    cpu, g = mirror(name)
    sp = DECKS[name]["species"][0]
    assert not any(sp.get("uth", [0, 0, 0]))
    dens = sp["density"]
    g.set_device_injector(0, dens["type"], start=dens.get("start", 0.0), end=dens.get("end", 0.0),
                          ufl=sp.get("ufl", (0.0, 0.0, 0.0)))
    for step in range(40):
        cpu.iter()
        g.step(1)
        assert g.count(0) == cpu.np_(0), step
        for f in ("E", "B"):
            err = field_err(getattr(g, f)(), getattr(cpu, f)())
            assert err <= 1e-5, f"{f} relative error {err:.2e} at step {step}"
    assert g.info()["n_move"] == cpu.n_move()
    # the last column: particles that entered with the latest moves
    nx = cpu.nx[0]
    a, b = canon(cpu.particles(0)), canon(g.particles(0))
    ca, cb = a[a["ix"] == nx - 1], b[b["ix"] == nx - 1]
    assert ca.size == cb.size and ca.size > 0
    assert np.allclose(np.sort(ca["x"]), np.sort(cb["x"]), atol=1e-5)
    assert np.array_equal(np.bincount(ca["iy"], minlength=cpu.nx[1]), np.bincount(cb["iy"], minlength=cpu.nx[1]))


@pytest.mark.parametrize("name", ["lwfa_window", "window_smooth_xy"])
def test_moving_window_graph_replay(name):
    """Moving window with device injection under graph replay (blocks keyed
    by their window moves and injected lattice): particle counts and fields
    against the oracle after every call, calls of 4 steps so that blocks
    start both aligned and mid-way, and graphs actually captured."""
    cpu, g = mirror(name)
    sp = DECKS[name]["species"][0]
    dens = sp["density"]
    g.set_device_injector(0, dens["type"], start=dens.get("start", 0.0), end=dens.get("end", 0.0),
                          ufl=sp.get("ufl", (0.0, 0.0, 0.0)))
    g.set_graphs(True)
    for call in range(16):
        n = 4 if call % 3 else 20
        cpu.iter(n)
        g.step(n)
        assert g.count(0) == cpu.np_(0), call
        for f in ("E", "B"):
            err = field_err(getattr(g, f)(), getattr(cpu, f)())
            assert err <= 1e-5, f"{f} relative error {err:.2e} after call {call}"
    assert g.info()["n_move"] == cpu.n_move()
    assert g.info()["captures"] > 0


@pytest.mark.parametrize("name", ["lwfa_window", "plane_slab"])
def test_laser_launch(name):
    """The GPU laser kernel against the oracle's emf_add_laser."""
    from zpic_gb300._zc import CudaSim

    d = DECKS[name]
    cpu = build_cpu(name, deck={k: v for k, v in d.items() if k not in ("species",)} | {"species": []})
    g = CudaSim(d["nx"], d["box"], d["dt"])
    g.add_laser(**d["laser"])  # before the window is set, as the deck does
    if d.get("moving_window"):
        g.set_moving_window()
    for f in ("E", "B"):
        a, b = getattr(g, f)(), getattr(cpu, f)()
        assert np.allclose(a, b, rtol=1e-5, atol=1e-6 * np.abs(b).max()), f


def test_charge_density():
    cpu, g = mirror("custom_ext")
    g.step(3)
    cpu.iter(3)
    assert np.allclose(g.charge(0), cpu.charge(0), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name", ["custom_ext", "lwfa_window"])
def test_phasespace_density(name):
    cpu, g = mirror(name)
    g.step(4)
    cpu.iter(4)
    for qs, rg in ((("x1", "u1"), ((0.0, 6.0), (-0.5, 0.5))), (("x2", "u3"), ((0.0, 5.0), (-1.0, 1.0))),
                   (("u1", "u2"), ((-0.3, 0.3), (-0.3, 0.3)))):
        a, b = g.phasespace(0, qs, (40, 24), rg), cpu.phasespace(0, qs, (40, 24), rg)
        assert np.allclose(a, b, rtol=1e-5, atol=1e-6 * max(np.abs(b).max(), 1e-30)), qs


def _tile_runs(parts, tile, nx):
    """Tile index and local cell of every particle, in buffer order."""
    tx, ty = tile
    ntx = (nx + tx - 1) // tx
    t = parts["ix"] // tx + (parts["iy"] // ty) * ntx
    cell = parts["ix"] % tx + (parts["iy"] % ty) * tx
    return t, cell


LANE_RUN = 8  # kLaneRun of the device layout: particles a push lane takes in a row


def tile_slot(i, n):
    """Slot of the i-th particle in cell order of a tile of n particles:
    full chunks of 32 * LANE_RUN are stored transposed (the device layout)."""
    ch = 32 * LANE_RUN
    c0 = i - i % ch
    if c0 + ch > n:
        return i
    r = i - c0
    return c0 + (r % LANE_RUN) * 32 + r // LANE_RUN


@pytest.mark.parametrize("tile", [(16, 16), (8, 8), (32, 16)])
def test_tiles_are_cell_sorted_after_upload(tile):
    cpu, g = mirror("thermal", tile=tile)
    p = g.particles(0)  # slot order (no holes right after an upload)
    t, cell = _tile_runs(p, tile, cpu.nx[0])
    assert np.all(np.diff(t) >= 0), "particles grouped by tile"
    starts = np.flatnonzero(np.r_[True, np.diff(t) != 0, True])
    for a, b in zip(starts[:-1], starts[1:]):
        n = b - a
        order = np.array([tile_slot(i, n) for i in range(n)])
        assert np.array_equal(np.sort(order), np.arange(n))
        assert np.all(np.diff(cell[a:b][order]) >= 0), "tile in cell order through tile_slot"
    assert canon(p).tobytes() == canon(cpu.particles(0)).tobytes()


def test_sort_frequency_does_not_change_physics():
    runs = []
    for every in (1, -1):
        cpu, g = mirror("weibel_smooth", sort_every=every)
        g.step(8)
        runs.append((g.E(), g.B(), [canon(g.particles(k)) for k in range(2)]))
    for f in range(2):
        assert field_err(runs[0][f], runs[1][f]) <= 1e-5
    for k in range(2):
        a, b = runs[0][2][k], runs[1][2][k]
        assert a.size == b.size
        for c in ("x", "y"):  # position multisets (robust to round-off reordering)
            pa = np.sort(a["i" + c] + a[c].astype(np.float64))
            pb = np.sort(b["i" + c] + b[c].astype(np.float64))
            assert np.abs(pa - pb).max() < 1e-3


def test_fast_push_close_to_exact():
    """The FMA build against the exact build: one push from the same state."""
    cpu = build_cpu("thermal")
    E, B = _random_fields(cpu, 11)
    cpu.set_E(E)
    cpu.set_B(B)
    _, ge = mirror("thermal", cpu=cpu, fast_math=False)
    _, gf = mirror("thermal", cpu=cpu, fast_math=True)
    for g in (ge, gf):
        g.current_zero()
        g.spec_advance(0)
    # compare as multisets (the order of the warps' output runs is not fixed)
    a, b = ge.particles(0), gf.particles(0)
    assert a.size == b.size
    for c in ("x", "y"):
        pa = np.sort(a["i" + c] + a[c].astype(np.float64))
        pb = np.sort(b["i" + c] + b[c].astype(np.float64))
        assert np.abs(pa - pb).max() < 1e-5
    for f in ("ux", "uy", "uz"):
        assert np.allclose(np.sort(a[f]), np.sort(b[f]), rtol=1e-5, atol=1e-7)
    assert field_err(gf.J(), ge.J()) <= 1e-5


@pytest.mark.parametrize("nxy", [(24, 2), (4, 20)], ids=["24x2", "4x20"])
def test_thin_grid_steps_match_oracle(nxy):
    """Grids too thin for the fused fold (< 6 cells on an axis) and, at 2
    rows, for the guard cells written by the Yee kernel (< 3): the separate
    fold and guard-cell kernels take over, and the steps still follow the
    oracle (bit-exact phases: fields within 1e-5 after 10 steps)."""
    nx, ny = nxy
    d = dict(nx=[nx, ny], box=[0.1 * nx, 0.1 * ny], dt=0.06,
             species=[dict(name="e1", m_q=-1.0, ppc=[2, 2], ufl=[0.0, 0.0, 0.3], uth=[0.05, 0.05, 0.05]),
                      dict(name="e2", m_q=-1.0, ppc=[2, 2], ufl=[0.0, 0.0, -0.3], uth=[0.05, 0.05, 0.05])],
             smooth=dict(xtype="compensated", xlevel=1, ytype="binomial", ylevel=1))
    cpu, g = mirror("thin", tile=(8, 8), deck=d)
    for step in range(10):
        cpu.iter()
        g.step(1)
        for f in ("E", "B", "J"):
            err = field_err_joint(getattr(g, f)(), getattr(cpu, f)())
            assert err <= 1e-5, f"{f} relative error {err:.2e} at step {step}"
    for k in range(2):
        assert g.count(k) == cpu.np_(k)
