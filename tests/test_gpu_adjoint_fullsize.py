"""The adjoint engine at the full size of the differentiable-step
configuration (256^2 cells, 4x4 ppc: 1,048,576 particles, dt 0.06, 200
steps, checkpoints every 20, weights 1 + 0.3 sum of 8 sinusoids, uth 0.05)
against autograd of the float64 PyTorch re-expression (tests/adjoint_torch.py)
run on the same GPU, checkpointed every 20 steps.

Both differentiate the same discrete step, branch by branch, so they agree
to round-off (the engine's and PyTorch's float64 deposit sums land in
different orders): the gradient with respect to a drift added to every
particle's u_x, and the projections of the weight gradient onto the 8 profile
amplitudes, within 1e-6 relative.  Central differences of this objective
cannot pin the drift gradient as tightly: the objective is piecewise smooth
with tens of thousands of kinks (cell edges and the staggered gather's
half-cell crossed by some trajectory) inside a step of 1e-6 or 1e-7: they
meet the adjoint within 1e-3 at a step of 1e-6 for the amplitudes and 1e-8
for the drift, which the second test checks.  The third checks the float32
engine's cost (forward and backward within 4x the forward) and its gradient
against the float64 engine's: within 1e-2 (measured 2.3-2.8e-3 for the
amplitudes, 4.3-4.7e-3 for the drift), the limit that float32 per-particle
gradients reach once projected with the 10^3-fold cancellation of these
sums.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import adjoint_torch as AT  # noqa: E402

pytestmark = pytest.mark.gpu

NX, DT, STEPS, K = (256, 256), 0.06, 200, 20


def test_c4_gradient_matches_autograd_at_full_size():
    from torch.utils.checkpoint import checkpoint

    from zpic_gb300 import adjoint

    st, amps, kk, q = adjoint.profile_setup(nx=NX, dx=0.1, ppc=(4, 4), uth=0.05, seed=7, drift=0.0)
    n = st["ix"].size
    box = (NX[0] * 0.1, NX[1] * 0.1)
    sim = adjoint.AdjointSim(NX, box, DT, n, q, checkpoint_every=K, precision="float64")
    try:
        sim.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"], st["uy"], st["uz"], st["w"])
        L_eng, _ = sim.forward(STEPS)
        g = sim.backward()
    finally:
        sim.close()
    drift_eng = float(np.sum(g["ux"]))
    amp_eng = adjoint.amplitude_gradient(g["w"], st["X"], kk)

    dev = torch.device("cuda:0")
    P = AT.Params(NX[0], NX[1], 0.1, 0.1, DT, q, -1.0)
    w = torch.tensor(st["w"], dtype=AT.T, device=dev, requires_grad=True)
    drift = torch.zeros((), dtype=AT.T, device=dev, requires_grad=True)
    ix = torch.as_tensor(st["ix"], dtype=torch.long, device=dev)
    iy = torch.as_tensor(st["iy"], dtype=torch.long, device=dev)
    x = torch.tensor(st["x"], dtype=AT.T, device=dev)
    y = torch.tensor(st["y"], dtype=AT.T, device=dev)
    ux = torch.tensor(st["ux"], dtype=AT.T, device=dev) + drift
    uy = torch.tensor(st["uy"], dtype=AT.T, device=dev)
    uz = torch.tensor(st["uz"], dtype=AT.T, device=dev)
    E = torch.zeros((3, NX[1], NX[0]), dtype=AT.T, device=dev)
    B = torch.zeros((3, NX[1], NX[0]), dtype=AT.T, device=dev)

    def segment(ix, iy, x, y, ux, uy, uz, E, B, w):
        s = (ix, iy, x, y, ux, uy, uz)
        for _ in range(K):
            s, E, B, _ = AT.step(s, E, B, w, P)
        return (*s, E, B)

    for _ in range(STEPS // K):
        ix, iy, x, y, ux, uy, uz, E, B = checkpoint(segment, ix, iy, x, y, ux, uy, uz, E, B, w, use_reentrant=False)
    L = AT.field_energy(E, B, P)
    L.backward()
    assert abs(float(L.detach()) / L_eng - 1) <= 1e-9
    drift_ag = float(drift.grad)
    amp_ag = adjoint.amplitude_gradient(w.grad.cpu().numpy(), st["X"], kk)
    assert abs(drift_eng / drift_ag - 1) <= 1e-6, (drift_eng, drift_ag)
    assert np.linalg.norm(amp_eng - amp_ag) <= 1e-6 * np.linalg.norm(amp_ag), (amp_eng, amp_ag)


def _engine_gradient(st, kk, prec):
    from zpic_gb300 import adjoint

    n = st["ix"].size
    sim = adjoint.AdjointSim(NX, (NX[0] * 0.1, NX[1] * 0.1), DT, n, st["q"], checkpoint_every=K, precision=prec)
    return sim


def _setup():
    from zpic_gb300 import adjoint

    st, amps, kk, q = adjoint.profile_setup(nx=NX, dx=0.1, ppc=(4, 4), uth=0.05, seed=7, drift=0.0)
    st["q"] = q
    return st, amps, kk


def _load(sim, st, w, drift=0.0):
    sim.set_state(st["ix"], st["iy"], st["x"], st["y"], st["ux"] + drift, st["uy"], st["uz"], w)


def test_c4_float64_gradient_matches_finite_differences():
    from zpic_gb300 import adjoint

    st, amps, kk = _setup()
    sim = _engine_gradient(st, kk, "float64")
    try:
        _load(sim, st, st["w"])
        sim.forward(STEPS)
        g = sim.backward()
        ga = adjoint.amplitude_gradient(g["w"], st["X"], kk)
        gd = float(np.sum(g["ux"]))

        def L(a, drift=0.0):
            _load(sim, st, adjoint.weights(st["X"], a, kk), drift)
            return sim.forward(STEPS)[0]

        e = 1e-6
        fa = np.array([(L(amps + e * u) - L(amps - e * u)) / (2 * e) for u in np.eye(len(amps))])
        ed = 1e-8
        fd = (L(amps, ed) - L(amps, -ed)) / (2 * ed)
    finally:
        sim.close()
    assert np.linalg.norm(ga - fa) <= 1e-3 * np.linalg.norm(fa), (ga, fa)
    assert abs(gd - fd) <= 1e-3 * abs(fd), (gd, fd)


def test_c4_float32_cost_and_accuracy():
    from zpic_gb300 import adjoint

    st, amps, kk = _setup()
    out = {}
    for prec in ("float32", "float64"):
        sim = _engine_gradient(st, kk, prec)
        try:
            for _ in range(2 if prec == "float32" else 1):  # float32: a warm-up run, then the timed one
                _load(sim, st, st["w"])
                sim.forward(STEPS)
                g = sim.backward()
            out[prec] = (adjoint.amplitude_gradient(g["w"], st["X"], kk), float(np.sum(g["ux"])), sim.times())
        finally:
            sim.close()
    (ga32, gd32, (fwd, bwd)), (ga64, gd64, _) = out["float32"], out["float64"]
    assert (fwd + bwd) / fwd <= 4.0, (fwd, bwd)
    assert np.linalg.norm(ga32 - ga64) <= 1e-2 * np.linalg.norm(ga64)
    assert abs(gd32 - gd64) <= 1e-2 * abs(gd64)
