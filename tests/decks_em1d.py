"""1-D test decks (plain dicts) for the em1d step: each is built on the
reference em1d (oracle/pyoracle_em1d.RefSim1D) to make the fixtures in
tests/golden/em1d/, and mirrored onto the GPU by the tests."""
import math

DECKS_1D = {
    # two streams (the reference's em1d/input/twostream.c set-up, 64 ppc) of
    # unequal drift, so that the net current stands well above round-off,
    # with compensated smoothing
    "twostream": dict(
        nx=120, box=4 * math.pi, dt=0.1,
        species=[dict(name="right", m_q=-1.0, ppc=64, ufl=[0.2, 0, 0], uth=[0.001, 0.001, 0.001]),
                 dict(name="left", m_q=-1.0, ppc=64, ufl=[-0.1, 0.05, 0.03], uth=[0.001, 0.001, 0.001])],
        smooth=dict(type="compensated", level=1),
        steps=60),
    # a laser entering a warm slab between open boundaries (Mur fields,
    # absorbed particles)
    "open_slab": dict(
        nx=400, box=8.0, dt=0.019,
        species=[dict(name="e", m_q=-1.0, ppc=16, uth=[0.02, 0.02, 0.02],
                      density=dict(type="slab", start=3.0, end=6.0))],
        laser=dict(start=2.5, fwhm=1.0, a0=1.5, omega0=10.0, polarization=math.pi / 4),
        open_fields=True, open_particles=True,
        smooth=dict(type="binomial", level=2),
        steps=200),
    # laser wakefield with a moving window over a cold step plasma
    "lwfa": dict(
        nx=1000, box=20.0, dt=0.019,
        species=[dict(name="e", m_q=-1.0, ppc=8, density=dict(type="step", start=20.0))],
        laser=dict(start=17.0, fwhm=2.0, a0=2.0, omega0=10.0, polarization=math.pi / 2),
        moving_window=True,
        smooth=dict(type="compensated", level=2),
        steps=400),
}


# grids wider than the fields kernel keeps in shared memory (its global-memory
# variant): no committed fixtures, the tests run the C restatement of the
# em1d step (pinned to the reference by the decks above) beside the GPU
WIDE_1D = {
    "wide_periodic": dict(
        nx=6000, box=300.0, dt=0.045,
        species=[dict(name="right", m_q=-1.0, ppc=4, ufl=[0.2, 0, 0], uth=[0.001, 0.001, 0.001]),
                 dict(name="left", m_q=-1.0, ppc=4, ufl=[-0.1, 0.05, 0.03], uth=[0.001, 0.001, 0.001])],
        smooth=dict(type="compensated", level=1),
        steps=60),
    "wide_open": dict(
        nx=6000, box=120.0, dt=0.019,
        species=[dict(name="e", m_q=-1.0, ppc=4, uth=[0.02, 0.02, 0.02],
                      density=dict(type="slab", start=40.0, end=80.0))],
        laser=dict(start=38.0, fwhm=4.0, a0=1.0, omega0=10.0, polarization=math.pi / 4),
        open_fields=True, open_particles=True,
        smooth=dict(type="binomial", level=2),
        steps=200),
    "wide_window": dict(
        nx=6000, box=120.0, dt=0.019,
        species=[dict(name="e", m_q=-1.0, ppc=4, density=dict(type="step", start=110.0))],
        laser=dict(start=108.0, fwhm=3.0, a0=2.0, omega0=10.0, polarization=math.pi / 2),
        moving_window=True,
        smooth=dict(type="compensated", level=2),
        steps=200),
}
