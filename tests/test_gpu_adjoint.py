"""The adjoint engine (zc_adj_*): its float64 forward against the float64
PyTorch re-expression, its hand-written gradient against PyTorch autograd of
that re-expression, its float32 forward against the oracle, and its float32
gradient against float64 central finite differences of the engine itself."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import adjoint_torch as AT  # noqa: E402
from decks import DECKS, build_cpu  # noqa: E402

pytestmark = pytest.mark.gpu


def _setup(nx=(24, 16), ppc=(2, 2), uth=0.1, drift=0.3, seed=3):
    from zpic_gb300 import adjoint

    st, amps, kk, q = adjoint.profile_setup(nx=nx, dx=0.1, ppc=ppc, uth=uth, seed=seed, drift=drift)
    rng = np.random.default_rng(seed + 1)
    ny_, nx_ = nx[1], nx[0]
    E0 = 0.05 * rng.standard_normal((3, ny_, nx_))
    B0 = 0.05 * rng.standard_normal((3, ny_, nx_))
    return st, amps, kk, q, E0, B0


def _engine(st, q, nx, dt, prec, K):
    from zpic_gb300.adjoint import AdjointSim

    sim = AdjointSim(nx, (nx[0] * 0.1, nx[1] * 0.1), dt, st["ix"].size, q, checkpoint_every=K, precision=prec)
    return sim


def _torch_run(st, E0, B0, q, nx, dt, nsteps, grad=False):
    P = AT.Params(nx[0], nx[1], 0.1, 0.1, dt, q, -1.0)
    leaves = {k: torch.tensor(st[k], dtype=AT.T, requires_grad=grad) for k in ("x", "y", "ux", "uy", "uz", "w")}
    E = torch.tensor(E0, dtype=AT.T, requires_grad=grad)
    B = torch.tensor(B0, dtype=AT.T, requires_grad=grad)
    s = (torch.as_tensor(st["ix"], dtype=torch.long), torch.as_tensor(st["iy"], dtype=torch.long), leaves["x"],
         leaves["y"], leaves["ux"], leaves["uy"], leaves["uz"])
    s2, E2, B2 = AT.run(s, E, B, leaves["w"], P, nsteps)
    L = AT.field_energy(E2, B2, P)
    return L, s2, E2, B2, leaves, E, B


def test_forward_float64_matches_torch():
    nx, dt, n = (24, 16), 0.06, 10
    st, amps, kk, q, E0, B0 = _setup(nx)
    sim = _engine(st, q, nx, dt, "float64", 4)
    sim.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], st["w"], E0, B0)
    L, _ = sim.forward(n)
    Lt, s2, E2, B2, *_ = _torch_run(st, E0, B0, q, nx, dt, n)
    got = sim.state()
    assert abs(L - float(Lt)) <= 1e-11 * abs(float(Lt))
    assert np.allclose(got["E"], E2.detach().numpy(), rtol=0, atol=1e-11)
    assert np.allclose(got["B"], B2.detach().numpy(), rtol=0, atol=1e-11)
    assert np.array_equal(got["ix"], s2[0].numpy()) and np.array_equal(got["iy"], s2[1].numpy())
    for k, t in zip(("x", "y", "ux", "uy", "uz"), s2[2:]):
        assert np.allclose(got[k], t.detach().numpy(), rtol=0, atol=1e-11), k


@pytest.mark.parametrize("K", [1, 4, 20])
def test_gradient_float64_matches_autograd(K):
    nx, dt, n = (24, 16), 0.06, 10
    st, amps, kk, q, E0, B0 = _setup(nx)
    sim = _engine(st, q, nx, dt, "float64", K)
    sim.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], st["w"], E0, B0)
    sim.forward(n)
    g = sim.backward()
    L, s2, E2, B2, leaves, E, B = _torch_run(st, E0, B0, q, nx, dt, n, grad=True)
    L.backward()
    want = {k: leaves[k].grad.numpy() for k in leaves}
    want["E"], want["B"] = E.grad.numpy(), B.grad.numpy()
    for k in ("w", "x", "y", "ux", "uy", "uz", "E", "B"):
        err = np.linalg.norm(g[k] - want[k]) / np.linalg.norm(want[k])
        assert err < 1e-9, (k, err)


def test_forward_float32_matches_oracle():
    """Weights 1 on the thermal deck without smoothing: the engine's float32
    step against the oracle within the forward bar."""
    from zpic_gb300.adjoint import AdjointSim

    d = dict(DECKS["thermal"])
    d.pop("smooth")
    cpu = build_cpu("thermal", deck=d)
    p = cpu.particles(0)
    nx = d["nx"]
    sim = AdjointSim(nx, d["box"], d["dt"], p.size, cpu.q(0), checkpoint_every=5, precision="float32")
    sim.set_state(p["ix"], p["iy"], p["x"], p["y"], p["ux"], p["uy"], p["uz"], np.ones(p.size))
    sim.forward(10)
    cpu.iter(10)
    got = sim.state()
    for f, want in (("E", cpu.E()), ("B", cpu.B())):
        w_ = np.transpose(want[1:nx[1] + 1, 1:nx[0] + 1, :], (2, 0, 1))
        err = np.linalg.norm(got[f] - w_) / np.linalg.norm(w_)
        assert err < 1e-5, (f, err)


def test_gradient_float32_matches_float64_finite_differences():
    """Profile amplitudes and drift: the float32 adjoint against central
    differences (eps 1e-4) of the float64 forward, relative 1e-3."""
    from zpic_gb300 import adjoint

    nx, dt, n, K = (64, 64), 0.06, 60, 20
    st, amps, kk, q = adjoint.profile_setup(nx=nx, dx=0.1, ppc=(2, 2), uth=0.05, seed=11, drift=0.05)
    sim32 = _engine(st, q, nx, dt, "float32", K)
    sim32.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], st["w"])
    sim32.forward(n)
    g = sim32.backward()
    ga = adjoint.amplitude_gradient(g["w"], st["X"], kk)
    gd = g["ux"].sum()
    sim64 = _engine(st, q, nx, dt, "float64", K)

    def L(a, drift):
        w = adjoint.weights(st["X"], a, kk)
        sim64.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"] + drift, st["uy"], st["uz"], w)
        return sim64.forward(n)[0]

    eps = 1e-4
    fd = np.array([(L(amps + eps * e, 0.0) - L(amps - eps * e, 0.0)) / (2 * eps) for e in np.eye(len(amps))])
    assert np.linalg.norm(ga - fd) <= 1e-3 * np.linalg.norm(fd), (ga, fd)
    fdd = (L(amps, eps) - L(amps, -eps)) / (2 * eps)
    assert abs(gd - fdd) <= 1e-3 * abs(fdd), (gd, fdd)


def test_autograd_function():
    from zpic_gb300 import adjoint

    nx, dt, n = (24, 16), 0.06, 8
    st, amps, kk, q, E0, B0 = _setup(nx)
    sim = _engine(st, q, nx, dt, "float64", 4)
    a = torch.tensor(amps, dtype=torch.float64, requires_grad=True)
    X = torch.as_tensor(st["X"])
    kt = torch.as_tensor(kk)
    w = 1.0 + 0.3 * torch.sin(torch.outer(X, kt)) @ a
    ux = torch.tensor(st["ux"], requires_grad=True)
    uy, uz = torch.tensor(st["uy"]), torch.tensor(st["uz"])
    E, B = torch.tensor(E0, requires_grad=True), torch.tensor(B0)
    L = adjoint.field_energy(w, ux, uy, uz, E, B, sim, st, n)
    L.backward()
    # the same through autograd of the re-expression
    Lt, s2, E2, B2, leaves, Et, Bt = _torch_run(dict(st, w=w.detach().numpy()), E0, B0, q, nx, dt, n, grad=True)
    Lt.backward()
    ga_t = 0.3 * (leaves["w"].grad @ torch.sin(torch.outer(X, kt)))
    assert torch.allclose(a.grad, ga_t, rtol=1e-9, atol=0)
    assert torch.allclose(ux.grad, leaves["ux"].grad, rtol=1e-9, atol=1e-14)
    assert torch.allclose(E.grad, Et.grad, rtol=1e-9, atol=1e-14)
