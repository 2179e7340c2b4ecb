"""The adjoint engine with a moving window, a laser and current filter
passes: its float32 forward against the oracle on the moving-window laser
deck (weights 1), and its float64 gradient of the on-axis Ex objective --
with respect to the laser amplitude and to density-ramp knots -- against
float64 central differences of the same engine."""
import numpy as np
import pytest

from decks import DECKS, build_cpu, _resolve

pytestmark = pytest.mark.gpu


def _pool(d, cpu_parts, nsteps):
    """initial particles plus the column each window move injects"""
    from zpic_gb300 import adjoint

    nx, ny = d["nx"]
    dx = float(np.float32(np.float32(d["box"][0]) / np.float32(nx)))
    moves = adjoint.window_moves(nsteps, d["dt"], dx)
    ppc = d["species"][0]["ppc"]
    hx, hy = np.float32(1.0) / np.float32(ppc[0]), np.float32(1.0) / np.float32(ppc[1])
    cols = [(nx - 1, j, hx * np.float32(a + 0.5), hy * np.float32(b + 0.5))
            for j in range(ny) for b in range(ppc[1]) for a in range(ppc[0])]
    n0 = cpu_parts.size
    n = n0 + len(moves) * len(cols)
    st = {k: np.zeros(n) for k in ("x", "y", "ux", "uy", "uz")}
    st["ix"] = np.zeros(n, dtype=np.int32)
    st["iy"] = np.zeros(n, dtype=np.int32)
    birth = np.zeros(n, dtype=np.int32)
    for f in ("ix", "iy", "x", "y", "ux", "uy", "uz"):
        st[f][:n0] = cpu_parts[f]
    k = n0
    for m, step in enumerate(moves):
        for (i, j, x, y) in cols:
            st["ix"][k], st["iy"][k], st["x"][k], st["y"][k] = i, j, x, y
            birth[k] = step + 1
            k += 1
    return st, birth, moves


def _grid(g, nx, ny):
    return np.transpose(g[1:ny + 1], (2, 0, 1)).astype(np.float64)


def test_forward_float32_matches_oracle_with_window():
    from zpic_gb300.adjoint import AdjointSim, smooth_passes

    name = "lwfa_window"
    d = DECKS[name]
    cpu = build_cpu(name)
    nx, ny = d["nx"]
    nsteps = 40
    st, birth, moves = _pool(d, cpu.particles(0), nsteps)
    assert len(moves) >= 20
    sim = AdjointSim((nx, ny), d["box"], d["dt"], st["ix"].size, cpu.q(0), checkpoint_every=10,
                     precision="float32", moving_window=True)
    sim.set_birth(birth)
    sm = d["smooth"]
    sim.set_smooth(smooth_passes(sm["xtype"], sm["xlevel"]))
    sim.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], np.ones(st["ix"].size),
                  _grid(cpu.E(), nx, ny), _grid(cpu.B(), nx, ny))
    sim.forward(nsteps)
    cpu.iter(nsteps)
    got = sim.state()
    assert cpu.n_move() == len(moves)
    alive = (got["alive"] == 1) & (birth <= nsteps)
    assert int(alive.sum()) == cpu.np_(0)
    for f, want in (("E", cpu.E()), ("B", cpu.B())):
        w_ = _grid(want, nx, ny)
        err = np.linalg.norm(got[f] - w_) / np.linalg.norm(w_)
        assert err < 1e-5, (f, err)


def test_gradient_float64_matches_finite_differences_with_window():
    from zpic_gb300 import adjoint

    name = "lwfa_window"
    d = DECKS[name]
    cpu = build_cpu(name)
    nx, ny = d["nx"]
    nsteps, K = 40, 10
    st, birth, moves = _pool(d, cpu.particles(0), nsteps)
    dx = float(np.float32(np.float32(d["box"][0]) / np.float32(nx)))
    X = (st["ix"] + st["x"]) * dx
    for k in range(len(moves)):  # lab position of the injected columns
        sl = slice(cpu.np_(0) + k * ny * 8, cpu.np_(0) + (k + 1) * ny * 8)
        X[sl] = (nx - 1 + (k + 1) + st["x"][sl]) * dx
    knots_x = np.linspace(2.0, (nx + len(moves)) * dx, 6)
    knots_n = np.array([0.3, 0.7, 1.0, 1.0, 0.9, 1.0])
    E0, B0 = _grid(cpu.E(), nx, ny), _grid(cpu.B(), nx, ny)
    sim = adjoint.AdjointSim((nx, ny), d["box"], d["dt"], st["ix"].size, cpu.q(0), checkpoint_every=K,
                             precision="float64", moving_window=True, objective="axis_ex", objective_row=ny // 2)
    sim.set_birth(birth)
    sm = d["smooth"]
    sim.set_smooth(adjoint.smooth_passes(sm["xtype"], sm["xlevel"]))

    def L(a0_scale, kn):
        w = adjoint.ramp_density(X, knots_x, kn)
        sim.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], w, a0_scale * E0,
                      a0_scale * B0)
        return sim.forward(nsteps)[0]

    L(1.0, knots_n)
    g = sim.backward()
    ga0 = float((g["E"] * E0).sum() + (g["B"] * B0).sum())   # d L / d(field scale) at 1
    gk = adjoint.ramp_gradient(g["w"], X, knots_x)
    eps = 1e-6
    fd0 = (L(1 + eps, knots_n) - L(1 - eps, knots_n)) / (2 * eps)
    assert abs(ga0 - fd0) <= 1e-5 * abs(fd0), (ga0, fd0)
    for k in (1, 2, 4):
        e = np.zeros_like(knots_n)
        e[k] = eps
        fdk = (L(1.0, knots_n + e) - L(1.0, knots_n - e)) / (2 * eps)
        assert abs(gk[k] - fdk) <= 1e-4 * max(abs(fdk), 1e-12), (k, gk[k], fdk)
