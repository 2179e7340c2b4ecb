"""A float64 PyTorch re-expression of the periodic em2d step with per-particle
charge weights, differentiated by autograd: the checker of the hand-written
adjoint engine (zc_adj_*).

It follows the reference step (em2d/simulation.c:45-56) without smoothing or
moving window: staggered bilinear gather (interpolate_fld,
em2d/particles.c:1029-1071), relativistic Boris push and move
(particles.c:1145-1207), zigzag deposit (dep_current_zamb,
particles.c:773-924) scaled by the weight, Yee b/2, e, b/2 (emf.c:500-562),
on periodic planes [component][iy][ix] without guard cells.  Branches (cell
crossings, the half-cell switch of the staggered gather) are taken on the
values, so the gradient is that of the piece each trajectory lies in.
"""
import numpy as np
import torch

T = torch.float64


class Params:
    def __init__(self, nx, ny, dx, dy, dt, q, m_q):
        self.nx, self.ny = int(nx), int(ny)
        self.dx, self.dy, self.dt = float(dx), float(dy), float(dt)
        self.q, self.m_q = float(q), float(m_q)
        self.tem = 0.5 * self.dt / self.m_q
        self.dt_dx, self.dt_dy = self.dt / self.dx, self.dt / self.dy
        self.qnx, self.qny = self.q * self.dx / self.dt, self.q * self.dy / self.dt


def _wrap(i, n):
    return torch.remainder(i, n)


def _at(P, c, i, j):
    """flat index of component c at cell (i, j), periodic"""
    return c * P.nx * P.ny + _wrap(j, P.ny) * P.nx + _wrap(i, P.nx)


def _lerp2(F, P, c, a, b, wa, wb):
    f = F.reshape(-1)
    return ((f[_at(P, c, a, b)] * (1 - wa) + f[_at(P, c, a + 1, b)] * wa) * (1 - wb) +
            (f[_at(P, c, a, b + 1)] * (1 - wa) + f[_at(P, c, a + 1, b + 1)] * wa) * wb)


def gather(E, B, P, ix, iy, x, y):
    lx = (x.detach() < 0.5)
    ly = (y.detach() < 0.5)
    ih = ix - lx.long()
    jh = iy - ly.long()
    w1h = torch.where(lx, x + 0.5, x - 0.5)
    w2h = torch.where(ly, y + 0.5, y - 0.5)
    return (_lerp2(E, P, 0, ih, iy, w1h, y), _lerp2(E, P, 1, ix, jh, x, w2h), _lerp2(E, P, 2, ix, iy, x, y),
            _lerp2(B, P, 0, ix, jh, x, w2h), _lerp2(B, P, 1, ih, iy, w1h, y), _lerp2(B, P, 2, ih, jh, w1h, w2h))


def boris(ux, uy, uz, f, P):
    ex, ey, ez = f[0] * P.tem, f[1] * P.tem, f[2] * P.tem
    tx, ty, tz = ux + ex, uy + ey, uz + ez
    u2 = tx * tx + ty * ty + tz * tz
    g = torch.sqrt(1 + u2)
    tg = P.tem / g
    bx, by, bz = f[3] * tg, f[4] * tg, f[5] * tg
    s2 = 2 / (1 + bx * bx + by * by + bz * bz)
    vx = tx + ty * bz - tz * by
    vy = ty + tz * bx - tx * bz
    vz = tz + tx * by - ty * bx
    bx, by, bz = bx * s2, by * s2, bz * s2
    tx = tx + (vy * bz - vz * by)
    ty = ty + (vz * bx - vx * bz)
    tz = tz + (vx * by - vy * bx)
    ux, uy, uz = tx + ex, ty + ey, tz + ez
    rg = 1 / torch.sqrt(1 + ux * ux + uy * uy + uz * uz)
    return ux, uy, uz, P.dt_dx * rg * ux, P.dt_dy * rg * uy, P.q * uz * rg


def _segment(J, P, m, w, s):
    """the 8 contributions of segment s (dict) where mask m holds"""
    s0x0, s0x1, s1x0, s1x1 = 1 - s["x0"], s["x0"], 1 - s["x1"], s["x1"]
    s0y0, s0y1, s1y0, s1y1 = 1 - s["y0"], s["y0"], 1 - s["y1"], s["y1"]
    jx, jy, q = s["dx"] * P.qnx, s["dy"] * P.qny, s["q"]
    ix, iy = s["ix"], s["iy"]
    mw = m.to(T) * w
    Jf = J.reshape(-1)
    terms = [
        (0, ix, iy, jx * (0.5 * (s0y0 + s1y0))),
        (0, ix, iy + 1, jx * (0.5 * (s0y1 + s1y1))),
        (1, ix, iy, jy * (0.5 * (s0x0 + s1x0))),
        (1, ix + 1, iy, jy * (0.5 * (s0x1 + s1x1))),
        (2, ix, iy, q * (s0x0 * s0y0 + s1x0 * s1y0 + (s0x0 * s1y0 - s1x0 * s0y0) / 2)),
        (2, ix + 1, iy, q * (s0x1 * s0y0 + s1x1 * s1y0 + (s0x1 * s1y0 - s1x1 * s0y0) / 2)),
        (2, ix, iy + 1, q * (s0x0 * s0y1 + s1x0 * s1y1 + (s0x0 * s1y1 - s1x0 * s0y1) / 2)),
        (2, ix + 1, iy + 1, q * (s0x1 * s0y1 + s1x1 * s1y1 + (s0x1 * s1y1 - s1x1 * s0y1) / 2)),
    ]
    for c, i, j, v in terms:
        Jf = Jf.index_add(0, _at(P, c, i, j), torch.where(m, v, torch.zeros_like(v)) * mw)
    return Jf.reshape(J.shape)


def _sel(m, a, b):
    return {k: torch.where(m, a[k], b[k]) for k in a}


def _split_y(S, dj, m):
    """splits S at its y edge where m holds: (S before the edge, the rest)"""
    yb = (dj == 1).to(T)
    ddy = torch.where(m, S["dy"], torch.ones_like(S["dy"]))
    f = torch.where(m, (S["y1"] - yb) / ddy, torch.zeros_like(S["dy"]))
    xc = S["x0"] + S["dx"] * (1 - f)
    C = {"y0": 1 - yb, "y1": S["y1"] - dj.to(T), "dy": S["dy"] * f, "iy": S["iy"] + dj, "x0": xc, "x1": S["x1"],
         "dx": S["dx"] * f, "ix": S["ix"], "q": S["q"] * f}
    S2 = dict(S)
    S2.update({"y1": yb + 0 * S["y1"], "dy": S["dy"] * (1 - f), "dx": S["dx"] * (1 - f), "x1": xc,
               "q": S["q"] * (1 - f)})
    return _sel(m, S2, S), C


def deposit(J, P, ix, iy, x0, y0, dx, dy, qvz, w):
    x1, y1 = x0 + dx, y0 + dy
    di = (x1.detach() >= 1).long() - (x1.detach() < 0).long()
    dj = (y1.detach() >= 1).long() - (y1.detach() < 0).long()
    hasx, hasy = di != 0, dj != 0
    qh = qvz * 0.5
    A = {"x0": x0, "x1": x1, "y0": y0, "y1": y1, "dx": dx, "dy": dy, "q": qh, "ix": ix, "iy": iy}
    xb = (di == 1).to(T)
    ddx = torch.where(hasx, dx, torch.ones_like(dx))
    f = torch.where(hasx, (x1 - xb) / ddx, torch.zeros_like(dx))
    yc = y0 + dy * (1 - f)
    Bs = {"x0": 1 - xb + 0 * x0, "x1": x1 - di.to(T), "dx": dx * f, "ix": ix + di, "y0": yc, "y1": y1,
          "dy": dy * f, "iy": iy, "q": qh * f}
    A2 = dict(A)
    A2.update({"x1": xb + 0 * x1, "dx": dx * (1 - f), "dy": dy * (1 - f), "y1": yc, "q": qh * (1 - f)})
    A = _sel(hasx, A2, A)
    ay1 = A["y1"].detach()
    first = hasx & hasy & ((ay1 < 0) | (ay1 >= 1))   # the first piece crosses the y edge
    second = hasx & hasy & ~first                     # the x tail crosses it
    only_y = ~hasx & hasy
    A, Ca = _split_y(A, dj, first | only_y)
    Bs1 = dict(Bs)
    Bs1.update({"y0": Bs["y0"] - dj.to(T), "y1": Bs["y1"] - dj.to(T), "iy": Bs["iy"] + dj})
    Bs = _sel(first, Bs1, Bs)
    Bs, Cb = _split_y(Bs, dj, second)
    C = _sel(second, Cb, Ca)
    J = _segment(J, P, hasy, w, C)
    J = _segment(J, P, hasx, w, Bs)
    J = _segment(J, P, torch.ones_like(hasx), w, A)
    return J


def yee(E, B, J, P):
    def r(a, sh, dim):
        return torch.roll(a, shifts=sh, dims=dim)

    hx, hy = 0.5 * P.dt / P.dx, 0.5 * P.dt / P.dy
    cx, cy = P.dt / P.dx, P.dt / P.dy

    def yee_b(E, B, ax, ay):
        Ex, Ey, Ez = E[0], E[1], E[2]
        # f(i+1) = roll(f, -1, x); f(j+1) = roll(f, -1, y)
        Bx = B[0] + (-ay * (r(Ez, -1, 0) - Ez))
        By = B[1] + (ax * (r(Ez, -1, 1) - Ez))
        Bz = B[2] + (-ax * (r(Ey, -1, 1) - Ey) + ay * (r(Ex, -1, 0) - Ex))
        return torch.stack([Bx, By, Bz])

    B = yee_b(E, B, hx, hy)
    Bx, By, Bz = B[0], B[1], B[2]
    Ex = E[0] + cy * (Bz - r(Bz, 1, 0)) - P.dt * J[0]
    Ey = E[1] + (-cx * (Bz - r(Bz, 1, 1))) - P.dt * J[1]
    Ez = E[2] + cx * (By - r(By, 1, 1)) - cy * (Bx - r(Bx, 1, 0)) - P.dt * J[2]
    E = torch.stack([Ex, Ey, Ez])
    B = yee_b(E, B, hx, hy)
    return E, B


def step(state, E, B, w, P):
    ix, iy, x, y, ux, uy, uz = state
    f = gather(E, B, P, ix, iy, x, y)
    ux, uy, uz, mx, my, qvz = boris(ux, uy, uz, f, P)
    J = torch.zeros((3, P.ny, P.nx), dtype=T, device=E.device)
    J = deposit(J, P, ix, iy, x, y, mx, my, qvz, w)
    x1, y1 = x + mx, y + my
    di = (x1.detach() >= 1).long() - (x1.detach() < 0).long()
    dj = (y1.detach() >= 1).long() - (y1.detach() < 0).long()
    x1 = x1 - di.to(T)
    y1 = y1 - dj.to(T)
    ix = _wrap(ix + di, P.nx)
    iy = _wrap(iy + dj, P.ny)
    E, B = yee(E, B, J, P)
    return (ix, iy, x1, y1, ux, uy, uz), E, B, J


def run(state, E, B, w, P, nsteps):
    for _ in range(nsteps):
        state, E, B, _ = step(state, E, B, w, P)
    return state, E, B


def field_energy(E, B, P):
    return 0.5 * P.dx * P.dy * ((E * E).sum() + (B * B).sum())


def tensors(d):
    """numpy state dict -> torch tensors (ix, iy long; the rest float64)"""
    return (torch.as_tensor(np.asarray(d["ix"]), dtype=torch.long), torch.as_tensor(np.asarray(d["iy"]),
                                                                                    dtype=torch.long),
            torch.as_tensor(np.asarray(d["x"], dtype=np.float64)), torch.as_tensor(np.asarray(d["y"], dtype=np.float64)),
            torch.as_tensor(np.asarray(d["ux"], dtype=np.float64)), torch.as_tensor(np.asarray(d["uy"], dtype=np.float64)),
            torch.as_tensor(np.asarray(d["uz"], dtype=np.float64)))
