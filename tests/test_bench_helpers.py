"""Host-side helpers of bench.py (no GPU): the em1d deck's step count follows
the reference's main loop, and the decks handed to the CPU checker carry the
reference deck's parameters."""
import math
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_em1d_steps_follow_the_reference_loop():
    import bench

    # for (n=0, t=0; t<=tmax; n++, t=n*dt) in float: 1201 iterations for
    # dt 0.019, tmax 22.8 (em1d/input/lwfa.c)
    assert bench.em1d_steps(0.019, 22.8) == 1201
    assert bench.em1d_steps(0.1, 1.0) == 11


def test_em1d_deck_matches_the_reference_deck():
    import bench

    d = bench.em1d_deck()
    assert (d["nx"], d["box"], d["dt"]) == (1000, 20.0, 0.019)
    sp = d["species"][0]
    assert sp["ppc"] == 128 and sp["m_q"] == -1.0 and sp["density"] == {"type": "step", "start": 20.0}
    L = d["laser"]
    assert (L["start"], L["fwhm"], L["a0"], L["omega0"]) == (17.0, 2.0, 2.0, 10.0)
    assert math.isclose(L["polarization"], math.pi / 2)
    assert d["moving_window"] and d["smooth"] == {"type": "compensated", "level": 4}
