"""Discrete charge continuity of the zigzag deposit (dep_current_zamb,
em2d/particles.c:773-924): for every cell, the change of the node charge
over one particle advance plus dt times the backward-difference divergence
of the deposited current (periodically folded) vanishes to rounding."""
import numpy as np


def residual(rho0, rho1, J, nx, ny, dx, dy, dt):
    """rho0, rho1: (ny+1, nx+1) node charge before / after; J: the raw
    deposit in reference layout (ny+3, nx+3, 3) with guard cells.  Returns
    (max |residual|, max |charge change|)."""
    Jf = np.asarray(J, dtype=np.float64).copy()
    # periodic fold of the guard cells (current_update_gc, em2d/current.c:118-159)
    Jf[:, nx, :] += Jf[:, 0, :]
    Jf[:, 1, :] += Jf[:, nx + 1, :]
    Jf[:, 2, :] += Jf[:, nx + 2, :]
    Jf[ny, :, :] += Jf[0, :, :]
    Jf[1, :, :] += Jf[ny + 1, :, :]
    Jf[2, :, :] += Jf[ny + 2, :, :]
    Ji = Jf[1:ny + 1, 1:nx + 1, :]
    drho = (np.asarray(rho1, np.float64) - np.asarray(rho0, np.float64))[:ny, :nx]
    div = (Ji[:, :, 0] - np.roll(Ji[:, :, 0], 1, axis=1)) * (float(dt) / float(dx)) + \
          (Ji[:, :, 1] - np.roll(Ji[:, :, 1], 1, axis=0)) * (float(dt) / float(dy))
    return float(np.abs(drho + div).max()), float(np.abs(drho).max())
