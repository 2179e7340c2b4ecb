"""The float64 PyTorch re-expression of the step (the adjoint's checker)
against the oracle, without a GPU: same deck, weights 1, no smoothing."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import adjoint_torch as AT  # noqa: E402
from decks import DECKS, build_cpu  # noqa: E402


def _interior(g, nx, ny):
    """oracle grid (ny+3, nx+3, 3) with guard cells -> [3, ny, nx]"""
    return np.transpose(g[1:ny + 1, 1:nx + 1, :], (2, 0, 1)).astype(np.float64)


@pytest.mark.parametrize("name", ["thermal", "weibel_smooth"])
def test_torch_step_matches_oracle(name):
    d = dict(DECKS[name])
    d.pop("smooth", None)
    cpu = build_cpu(name, deck=d)
    nx, ny = d["nx"]
    P = AT.Params(nx, ny, np.float32(d["box"][0]) / np.float32(nx), np.float32(d["box"][1]) / np.float32(ny),
                  np.float32(d["dt"]), 0.0, d["species"][0]["m_q"])
    E = torch.zeros((3, ny, nx), dtype=AT.T)
    B = torch.zeros((3, ny, nx), dtype=AT.T)
    states = []
    for k in range(cpu.n_species):
        p = cpu.particles(k)
        states.append((AT.tensors(p), torch.ones(p.size, dtype=AT.T), float(cpu.q(k))))
    for _ in range(5):
        J = torch.zeros((3, ny, nx), dtype=AT.T)
        new = []
        for st, w, q in states:
            P.q = q
            P.qnx, P.qny = q * P.dx / P.dt, q * P.dy / P.dt
            ix, iy, x, y, ux, uy, uz = st
            f = AT.gather(E, B, P, ix, iy, x, y)
            ux, uy, uz, mx, my, qvz = AT.boris(ux, uy, uz, f, P)
            J = AT.deposit(J, P, ix, iy, x, y, mx, my, qvz, w)
            x1, y1 = x + mx, y + my
            di = (x1 >= 1).long() - (x1 < 0).long()
            dj = (y1 >= 1).long() - (y1 < 0).long()
            new.append(((AT._wrap(ix + di, nx), AT._wrap(iy + dj, ny), x1 - di, y1 - dj, ux, uy, uz), w, q))
        states = new
        E, B = AT.yee(E, B, J, P)
    cpu.iter(5)
    for got, want in ((E, cpu.E()), (B, cpu.B())):
        w_ = _interior(want, nx, ny)
        err = np.linalg.norm(got.numpy() - w_) / np.linalg.norm(w_)
        assert err < 1e-5, err  # float32 oracle against float64: ~1e-6 here
