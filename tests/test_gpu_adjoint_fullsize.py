"""The float64 adjoint at the full size of the differentiable-step
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
half-cell crossed by some trajectory) inside any useful step.
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
    assert abs(float(L) / L_eng - 1) <= 1e-9
    drift_ag = float(drift.grad)
    amp_ag = adjoint.amplitude_gradient(w.grad.cpu().numpy(), st["X"], kk)
    assert abs(drift_eng / drift_ag - 1) <= 1e-6, (drift_eng, drift_ag)
    assert np.linalg.norm(amp_eng - amp_ag) <= 1e-6 * np.linalg.norm(amp_ag), (amp_eng, amp_ag)
