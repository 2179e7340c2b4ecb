"""Size-independent properties at the benchmark's full size (2048 x 2048
cells, 4 x 4 ppc: 67,108,864 particles), where the oracle would take
minutes per step: discrete charge continuity of one advance, with the exact
and the fast push, and bit-reproducibility of the deterministic mode."""
import numpy as np
import pytest

import continuity

pytestmark = pytest.mark.gpu

NX, BOX, DT = (2048, 2048), (204.8, 204.8), 0.05


def _sim(**kw):
    from zpic_gb300._zc import CudaSim

    g = CudaSim(NX, BOX, DT, tile=(32, 16), **kw)
    g.add_species_device(-1.0, (4, 4), uth=(0.05, 0.05, 0.05), seed=21)
    return g


@pytest.mark.parametrize("fast", [False, True], ids=["exact", "fast"])
def test_charge_continuity_full_size(fast):
    g = _sim(fast_math=fast)
    g.set_smooth("compensated", 1, "compensated", 1)
    g.step(3)                      # some fields, some motion
    rho0 = g.charge(0)
    g.current_zero()
    g.spec_advance(0)
    J = g.J()
    rho1 = g.charge(0)
    dx = np.float32(BOX[0]) / np.float32(NX[0])
    res, dmax = continuity.residual(rho0, rho1, J, NX[0], NX[1], dx, dx, np.float32(DT))
    assert dmax > 1e-3, dmax
    assert res < 4e-6, (res, dmax)
    assert g.count(0) == NX[0] * NX[1] * 16
    g.close()


def test_deterministic_full_size_is_bit_reproducible():
    out = []
    for _ in range(2):
        g = _sim(deterministic=True, fast_math=True)
        g.set_smooth("compensated", 1, "compensated", 1)
        g.step(4)
        emf, kin = g.energy()
        out.append((g.E(), g.B(), g.J(), emf, kin))
        g.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
