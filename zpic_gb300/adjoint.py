"""Differentiable em2d: gradients of the final field energy through the
hand-written adjoint of the step (libzpic_cuda's zc_adj_* engine).

``AdjointSim`` wraps one engine.  It runs the periodic em2d step with a
charge weight per particle, in float32 or float64, and returns the gradient
of the total field energy after the last step with respect to:

- every particle's weight, initial in-cell position and momentum;
- the initial E and B.

``FieldEnergy`` puts the engine behind ``torch.autograd.Function``, so that the
objective composes with torch code: density profiles, drifts and laser
amplitudes that parametrise the initial state. Torch is the interface here,
not the computation.

``profile_setup`` builds the differentiable-density configuration, and
``amplitude_gradient`` chains the weight gradient to its profile amplitudes.
The configuration is a uniform 4x4 lattice with weights
n(x) = 1 + 0.3 sum_k a_k sin(k_k x), with 8 seeded amplitudes in [-1, 1]/8, and a
thermal spread.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._zc import AdjDesc, _ck, _p, load

PREC = {"float32": 0, "float64": 1}


class AdjointSim:
    """One adjoint engine: nx x ny periodic cells, np particles."""

    def __init__(self, nx, box, dt, n_particles, q, m_q=-1.0, checkpoint_every=20, precision="float32", device=0,
                 moving_window=False, objective="field_energy", objective_row=0, objective_cells=(0, 0)):
        self.lib = load()
        d = AdjDesc()
        d.nx[0], d.nx[1] = int(nx[0]), int(nx[1])
        d.box[0], d.box[1] = float(box[0]), float(box[1])
        d.dt = float(dt)
        d.q = float(q)
        d.m_q = float(m_q)
        d.np = int(n_particles)
        d.checkpoint_every = int(checkpoint_every)
        d.precision = PREC[precision]
        d.device = int(device)
        d.moving_window = int(bool(moving_window))
        d.objective = {"field_energy": 0, "axis_ex": 1}[objective]
        d.objective_row = int(objective_row)
        d.objective_cells[0], d.objective_cells[1] = int(objective_cells[0]), int(objective_cells[1])
        h = C.c_void_p()
        _ck(self.lib.zc_adj_create(C.byref(d), C.byref(h)))
        self.h = h
        self.nx = (int(nx[0]), int(nx[1]))
        self.box = (float(box[0]), float(box[1]))
        self.dx = self.box[0] / self.nx[0]
        self.dy = self.box[1] / self.nx[1]
        self.n = int(n_particles)
        self.mw = bool(moving_window)
        self.cols = self.nx[0] + 3 if self.mw else self.nx[0]

    def close(self):
        if getattr(self, "h", None):
            self.lib.zc_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _grid(self, a):
        if a is None:
            return None
        g = np.ascontiguousarray(a, dtype=np.float64).reshape(3, self.nx[1], self.cols)
        return g

    def set_state(self, ix, iy, x, y, ux, uy, uz, w, E=None, B=None):
        """Initial state: cells and in-cell positions (as t_part), momenta,
        weights; E, B as [3, ny, nx] (None: zero)."""
        ints = [np.ascontiguousarray(v, dtype=np.int32) for v in (ix, iy)]
        reals = [np.ascontiguousarray(v, dtype=np.float64) for v in (x, y, ux, uy, uz, w)]
        for v in ints + reals:
            if v.size != self.n:
                raise ValueError(f"particle arrays must hold {self.n} entries")
        Eg, Bg = self._grid(E), self._grid(B)
        self._keep = (ints, reals, Eg, Bg)
        _ck(self.lib.zc_adj_set_state(self.h, *[_p(v) for v in ints], *[_p(v) for v in reals],
                                      None if Eg is None else _p(Eg), None if Bg is None else _p(Bg)))

    def forward(self, nsteps):
        """Runs nsteps; returns (objective, kinetic energy of the last step)."""
        obj, kin = C.c_double(), C.c_double()
        _ck(self.lib.zc_adj_forward(self.h, int(nsteps), C.byref(obj), C.byref(kin)))
        return obj.value, kin.value

    def backward(self):
        """Gradient of the last forward run's objective with respect to the
        initial state: dict of w, x, y, ux, uy, uz [n] and E, B [3, ny, nx]."""
        out = {k: np.zeros(self.n) for k in ("w", "x", "y", "ux", "uy", "uz")}
        for k in ("E", "B"):
            out[k] = np.zeros((3, self.nx[1], self.cols))
        _ck(self.lib.zc_adj_backward(self.h, *[_p(out[k]) for k in ("w", "x", "y", "ux", "uy", "uz", "E", "B")]))
        return out

    def state(self):
        """Current state (after forward: the end of the run)."""
        ix = np.zeros(self.n, dtype=np.int32)
        iy = np.zeros(self.n, dtype=np.int32)
        alive = np.zeros(self.n, dtype=np.int32)
        r = {k: np.zeros(self.n) for k in ("x", "y", "ux", "uy", "uz")}
        E = np.zeros((3, self.nx[1], self.cols))
        B = np.zeros_like(E)
        _ck(self.lib.zc_adj_get_state(self.h, _p(ix), _p(iy), _p(alive),
                                      *[_p(r[k]) for k in ("x", "y", "ux", "uy", "uz")], _p(E), _p(B)))
        return dict(ix=ix, iy=iy, alive=alive, E=E, B=B, **r)

    def set_birth(self, birth):
        """Step at which each particle starts (None: all at step 0)."""
        if birth is None:
            _ck(self.lib.zc_adj_set_birth(self.h, None))
            return
        b = np.ascontiguousarray(birth, dtype=np.int32)
        self._birth = b
        _ck(self.lib.zc_adj_set_birth(self.h, _p(b)))

    def set_smooth(self, passes):
        """Current filter passes along x: [(sa, sb), ...]."""
        sa = np.ascontiguousarray([p[0] for p in passes], dtype=np.float64)
        sb = np.ascontiguousarray([p[1] for p in passes], dtype=np.float64)
        self._passes = (sa, sb)
        _ck(self.lib.zc_adj_set_smooth(self.h, len(passes), _p(sa) if len(passes) else None,
                                       _p(sb) if len(passes) else None))

    def times(self):
        """(forward ms, backward ms) of the last calls, device time."""
        f, b = C.c_float(), C.c_float()
        _ck(self.lib.zc_adj_times(self.h, C.byref(f), C.byref(b)))
        return f.value, b.value


def _field_energy_fn():
    import torch

    class FieldEnergy(torch.autograd.Function):
        """L = field energy after `nsteps` of the engine, as a function of
        the weights, the momenta and the initial E, B (torch float64 tensors
        on the host).  Positions and cells are fixed inputs in `base`."""

        @staticmethod
        def forward(ctx, w, ux, uy, uz, E0, B0, sim, base, nsteps):
            sim.set_state(base["ix"], base["iy"], base["x"], base["y"], ux.detach().numpy(),
                          uy.detach().numpy(), uz.detach().numpy(), w.detach().numpy(), E0.detach().numpy(),
                          B0.detach().numpy())
            L, _ = sim.forward(nsteps)
            ctx.sim = sim
            return torch.tensor(L, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gL):
            g = ctx.sim.backward()
            t = {k: torch.as_tensor(v) * gL for k, v in g.items()}
            return t["w"], t["ux"], t["uy"], t["uz"], t["E"], t["B"], None, None, None

    return FieldEnergy


def field_energy(w, ux, uy, uz, E0, B0, sim, base, nsteps):
    """Differentiable objective (see FieldEnergy)."""
    return _field_energy_fn().apply(w, ux, uy, uz, E0, B0, sim, base, nsteps)


# ---------------------------------------------------------------------------
# the differentiable-density configuration
# ---------------------------------------------------------------------------
def profile_setup(nx=(256, 256), dx=0.1, ppc=(4, 4), uth=0.05, modes=8, amp=0.3, seed=7, drift=0.0):
    """Uniform ppc lattice (spec_set_x, em2d/particles.c:159-354, uniform),
    thermal momenta (seeded normal deviates) plus a drift along x, 8 seeded
    profile amplitudes in [-1, 1]/8, wave numbers 2 pi k / Lx.  Returns
    (state dict with weights, amplitudes, wave numbers, particle charge)."""
    rng = np.random.default_rng(seed)
    nxx, nyy = int(nx[0]), int(nx[1])
    px, py = int(ppc[0]), int(ppc[1])
    lx = (np.arange(px) + 0.5) / px
    ly = (np.arange(py) + 0.5) / py
    ix, iy, a_, b_ = np.meshgrid(np.arange(nxx), np.arange(nyy), np.arange(px), np.arange(py), indexing="ij")
    ix, iy = ix.ravel().astype(np.int32), iy.ravel().astype(np.int32)
    x = lx[a_.ravel()].astype(np.float32).astype(np.float64)
    y = ly[b_.ravel()].astype(np.float32).astype(np.float64)
    n = ix.size
    ux = (uth * rng.standard_normal(n)).astype(np.float32).astype(np.float64) + drift
    uy = (uth * rng.standard_normal(n)).astype(np.float32).astype(np.float64)
    uz = (uth * rng.standard_normal(n)).astype(np.float32).astype(np.float64)
    amps = rng.uniform(-1.0, 1.0, modes) / 8.0
    L = nxx * dx
    kk = 2 * math.pi * np.arange(1, modes + 1) / L
    st = dict(ix=ix, iy=iy, x=x, y=y, ux=ux, uy=uy, uz=uz)
    st["X"] = (ix + x) * dx
    st["w"] = weights(st["X"], amps, kk, amp)
    q = -1.0 / (px * py)
    return st, amps, kk, q


def weights(X, amps, kk, amp=0.3):
    """n(x) = 1 + amp sum_k a_k sin(k_k x)"""
    return 1.0 + amp * np.sin(np.outer(X, kk)) @ np.asarray(amps)


def amplitude_gradient(dw, X, kk, amp=0.3):
    """dL/da_k = sum_p dL/dw_p amp sin(k_k X_p)"""
    return amp * (np.asarray(dw) @ np.sin(np.outer(X, kk)))


# ---------------------------------------------------------------------------
# the moving-window laser-wakefield configuration
# ---------------------------------------------------------------------------
def smooth_passes(kind, level):
    """[(sa, sb), ...] of current_smooth along x (em2d/current.c:297-304,
    427-459): `level` binomial passes, then the compensator for
    "compensated"."""
    p = [(0.25, 0.5)] * int(level)
    if kind == "compensated":
        a = np.float32(-1.0)
        b = np.float32((4.0 + 2.0 * level) / level)
        tot = np.float32(2 * a + b)
        p.append((float(np.float32(a / tot)), float(np.float32(b / tot))))
    return p


def window_moves(nsteps, dt, dx):
    """Steps at which the window moves: (n + 1) dt > dx (n_move + 1) in
    float32, as spec_move_window / emf_move_window test it
    (em2d/particles.c:621, em2d/emf.c:650)."""
    dtf, dxf = np.float32(dt), np.float32(dx)
    moves, nm = [], 0
    for n in range(nsteps):
        if np.float32(np.float32(n + 1) * dtf) > np.float32(dxf * np.float32(nm + 1)):
            moves.append(n)
            nm += 1
    return moves


def ramp_density(X, knots_x, knots_n):
    """piecewise-linear density through the knots (0 before the first)"""
    return np.where(X < knots_x[0], 0.0, np.interp(X, knots_x, knots_n))


def ramp_gradient(dw, X, knots_x):
    """dL/dn_k = sum_p dL/dw_p hat_k(X_p) for the piecewise-linear ramp"""
    g = np.zeros(len(knots_x))
    for k in range(len(knots_x)):
        e = np.zeros(len(knots_x))
        e[k] = 1.0
        g[k] = np.asarray(dw) @ ramp_density(X, knots_x, e)
    return g


def wakefield_setup(nx=(2000, 256), box=(40.0, 51.2), dt=0.014, nsteps=3000, ppc=(4, 2), start=20.0, n_knots=16,
                    laser=None, smooth=("binomial", 4)):
    """The pool of every particle the run will hold: the initial step-density
    plasma (loaded as spec_new does) and, for each window move, the column
    the move uncovers (the ppc lattice of cell nx-1, cold), born the step
    after the move.  Returns a dict with the particle arrays, births, lab
    positions X (for the density ramp), the ramp knots, the initial fields
    of the laser (E, B as [3, ny, nx+3]) and the filter passes."""
    from . import em2d
    from ._zc import CudaSim

    dx = np.float32(np.float32(box[0]) / np.float32(nx[0]))
    em2d.set_rand_seed(12345, 67890, fresh=True)
    parts, q = em2d.load_particles(-1.0, ppc, nx, box, dt, density=em2d.Density(type="step", start=start))
    moves = window_moves(nsteps, dt, float(dx))
    hx, hy = np.float32(1.0) / np.float32(ppc[0]), np.float32(1.0) / np.float32(ppc[1])
    a_, j_, b_ = np.meshgrid(np.arange(ppc[0]), np.arange(nx[1]), np.arange(ppc[1]), indexing="ij")
    col_x = (hx * (a_.ravel() + np.float32(0.5))).astype(np.float32)
    col_y = (hy * (b_.ravel() + np.float32(0.5))).astype(np.float32)
    col_iy = j_.ravel().astype(np.int32)
    m = len(moves)
    nc = col_x.size
    n0 = parts.size
    n = n0 + m * nc
    st = {k: np.zeros(n) for k in ("x", "y", "ux", "uy", "uz")}
    st["ix"] = np.zeros(n, dtype=np.int32)
    st["iy"] = np.zeros(n, dtype=np.int32)
    birth = np.zeros(n, dtype=np.int32)
    X = np.zeros(n)
    for f in ("ix", "iy", "x", "y", "ux", "uy", "uz"):
        st[f][:n0] = parts[f]
    X[:n0] = (parts["ix"] + parts["x"].astype(np.float64)) * float(dx)
    for k, step in enumerate(moves):
        sl = slice(n0 + k * nc, n0 + (k + 1) * nc)
        st["ix"][sl] = nx[0] - 1
        st["iy"][sl] = col_iy
        st["x"][sl] = col_x
        st["y"][sl] = col_y
        birth[sl] = step + 1
        X[sl] = (nx[0] - 1 + (k + 1) + col_x.astype(np.float64)) * float(dx)
    x_end = (nx[0] + m) * float(dx)
    knots_x = np.linspace(start, x_end, n_knots)
    knots_n = np.clip(0.2 + 0.8 * np.arange(n_knots) / 5.0, 0.0, 1.0)
    lz = dict(type="gaussian", start=17.0, fwhm=2.0, a0=2.0, omega0=10.0, W0=4.0, focus=20.0,
              axis=box[1] / 2, polarization=0.0)
    if laser:
        lz.update(laser)
    sim = CudaSim(nx, box, dt)
    sim.add_laser(**lz)
    # reference layout (ny+3, nx+3, 3) -> [3, ny, nx+3] (interior rows)
    E = np.transpose(sim.E()[1:nx[1] + 1], (2, 0, 1)).astype(np.float64).copy()
    B = np.transpose(sim.B()[1:nx[1] + 1], (2, 0, 1)).astype(np.float64).copy()
    sim.close()
    return dict(state=st, birth=birth, X=X, q=q, knots_x=knots_x, knots_n=knots_n, E=E, B=B, a0=lz["a0"],
                passes=smooth_passes(*smooth) if smooth else [], moves=moves, n_initial=n0)
