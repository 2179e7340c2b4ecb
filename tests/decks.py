"""Small em2d input decks shared by the golden-vector generator and the tests.

Each deck is a plain dict (grid, species, smoothing, laser, window, external
fields) so that the same physics set-up can be built on the CPU checker and
on the CUDA path.  Custom profiles are named functions here, not lambdas, so
that a deck can be rebuilt from its name alone.
"""
import math

import numpy as np


def dens_sine_x(x):
    return 1.5 + 0.5 * math.sin(x)


def dens_lin_y(y):
    return 1.0 + 0.2 * y


def dens_ramp_x(x):
    return 0.0 if x < 1.0 else min(1.5, 0.3 + (x - 1.0))


def ext_E_lin(ix, dx, iy, dy):
    return (0.01 * ix * dx, 0.0, 0.02)


def init_B_lin(ix, dx, iy, dy):
    return (0.0, 0.0, 0.01 * iy * dy)


FUNCS = {f.__name__: f for f in (dens_sine_x, dens_lin_y, dens_ramp_x, ext_E_lin, init_B_lin)}

DECKS = {
    # two counter-streaming electron species (Weibel set-up), periodic, smoothing on
    "weibel_smooth": dict(
        nx=[32, 24], box=[3.2, 2.4], dt=0.07,
        species=[dict(name="e1", m_q=-1.0, ppc=[2, 2], ufl=[0, 0, 0.6], uth=[0.1, 0.1, 0.1]),
                 dict(name="e2", m_q=-1.0, ppc=[2, 2], ufl=[0, 0, -0.6], uth=[0.1, 0.1, 0.1])],
        smooth=dict(xtype="compensated", xlevel=2, ytype="binomial", ylevel=1),
        steps=20),
    # uniform thermal plasma, compensated level-1 smoothing on both axes
    "thermal": dict(
        nx=[32, 16], box=[3.2, 1.6], dt=0.05,
        species=[dict(name="e", m_q=-1.0, ppc=[4, 4], uth=[0.05, 0.05, 0.05])],
        smooth=dict(xtype="compensated", xlevel=1, ytype="compensated", ylevel=1),
        steps=20),
    # moving window with a Gaussian laser entering a step plasma
    "lwfa_window": dict(
        nx=[128, 24], box=[2.56, 4.8], dt=0.014,
        species=[dict(name="e", m_q=-1.0, ppc=[4, 2], density=dict(type="step", start=2.0))],
        laser=dict(type="gaussian", start=1.7, fwhm=0.5, a0=2.0, omega0=10.0, W0=1.5,
                   focus=2.0, axis=2.4, polarization=math.pi / 2),
        moving_window=True,
        smooth=dict(xtype="compensated", xlevel=4),
        steps=60),
    # plane laser on a slab, mixed smoothing kinds
    "plane_slab": dict(
        nx=[64, 16], box=[6.4, 1.6], dt=0.05,
        species=[dict(name="e", m_q=-1.0, ppc=[2, 2], uth=[0.02, 0.02, 0.02],
                      density=dict(type="slab", start=2.0, end=4.0))],
        laser=dict(type="plane", start=1.5, rise=0.4, flat=0.3, fall=0.4, a0=1.0, omega0=5.0,
                   polarization=0.3),
        smooth=dict(xtype="binomial", xlevel=2, ytype="compensated", ylevel=3),
        steps=30),
    # custom density profile with external fields
    "custom_ext": dict(
        nx=[32, 24], box=[3.2, 2.4], dt=0.05,
        species=[dict(name="e", m_q=-1.0, ppc=[3, 2], uth=[0.05, 0.05, 0.05],
                      density=dict(type="custom", custom_x="dens_sine_x", custom_y="dens_lin_y"))],
        ext_fld=dict(B_type="uniform", B_0=[0.0, 0.0, 0.5], E_type="custom", E_custom="ext_E_lin"),
        steps=20),
    # moving window over a custom ramp, two species, initial fields and a plane pulse
    "custom_window": dict(
        nx=[100, 16], box=[2.0, 3.2], dt=0.014,
        species=[dict(name="e", m_q=-1.0, ppc=[2, 2], uth=[0.01, 0.01, 0.01],
                      density=dict(type="custom", custom_x="dens_ramp_x")),
                 dict(name="i", m_q=100.0, ppc=[2, 2], density=dict(type="uniform", n=2.0))],
        init_fld=dict(E_type="uniform", E_0=[0.0, 0.01, 0.0], B_type="custom", B_custom="init_B_lin"),
        laser=dict(type="plane", start=0.9, fwhm=0.3, a0=0.5, omega0=8.0),
        moving_window=True,
        steps=60),
    # moving window with current smoothing along both axes (the window keeps
    # the x guard columns out of the x passes)
    "window_smooth_xy": dict(
        nx=[96, 24], box=[1.92, 4.8], dt=0.014,
        species=[dict(name="e", m_q=-1.0, ppc=[2, 2], density=dict(type="step", start=1.0))],
        laser=dict(type="gaussian", start=1.3, fwhm=0.4, a0=1.5, omega0=10.0, W0=1.2,
                   focus=1.5, axis=2.4, polarization=0.0),
        moving_window=True,
        smooth=dict(xtype="binomial", xlevel=2, ytype="compensated", ylevel=2),
        steps=50),
}


def _resolve(d):
    out = dict(d)
    for k, v in d.items():
        if isinstance(v, str) and v in FUNCS:
            out[k] = FUNCS[v]
    return out


def build_cpu(name, backend="oracle", fast=False, deck=None):
    """Build a deck on the CPU checker (``oracle.pyoracle.CpuSim``)."""
    from oracle.pyoracle import CpuSim, set_rand_seed

    d = deck or DECKS[name]
    set_rand_seed(12345, 67890, backend=backend, fast=fast, fresh=(backend == "oracle"))
    s = CpuSim(d["nx"], d["box"], d["dt"], backend=backend, fast=fast)
    for sp in d["species"]:
        dens = _resolve(sp["density"]) if "density" in sp else None
        s.add_species(sp["name"], sp["m_q"], sp["ppc"], ufl=sp.get("ufl"), uth=sp.get("uth"),
                      density=dens)
    if "init_fld" in d:
        s.init_fld(**_resolve(d["init_fld"]))
    if "ext_fld" in d:
        s.set_ext_fld(**_resolve(d["ext_fld"]))
    if "laser" in d:
        s.add_laser(**d["laser"])
    if d.get("moving_window"):
        s.set_moving_window()
    if "smooth" in d:
        s.set_smooth(**d["smooth"])
    return s


def rel_l2(a, b):
    """||a-b|| / max(||b||, tiny) over float64 copies."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / max(nb, 1e-30))


# The benchmark configurations the tests hold to the reference at full size
# (or, for the 2048^2 thermal plasma, on a 256^2 box of the same density,
# cell size, time step, ppc and smoothing).
CONFIG_DECKS = {
    # Weibel instability: 128^2 cells, box 12.8^2, dt 0.07, two electron
    # species drifting +-0.6 c along z with uth 0.1, 4x4 ppc each
    # (524,288 particles), periodic, no smoothing, 500 steps
    # (em2d/input/weibel.c with electron-electron streams and 4x4 ppc)
    "c1_weibel": dict(
        nx=[128, 128], box=[12.8, 12.8], dt=0.07,
        species=[dict(name="e1", m_q=-1.0, ppc=[4, 4], ufl=[0, 0, 0.6], uth=[0.1, 0.1, 0.1]),
                 dict(name="e2", m_q=-1.0, ppc=[4, 4], ufl=[0, 0, -0.6], uth=[0.1, 0.1, 0.1])],
        steps=500),
    # uniform thermal plasma of the 2048^2 throughput workload on a 256^2
    # box: dx = dy = 0.1, dt 0.05, uth 0.05, 4x4 ppc (1,048,576 particles),
    # compensated level-1 smoothing on x and y
    "c2_thermal_256": dict(
        nx=[256, 256], box=[25.6, 25.6], dt=0.05,
        species=[dict(name="e", m_q=-1.0, ppc=[4, 4], uth=[0.05, 0.05, 0.05])],
        smooth=dict(xtype="compensated", xlevel=1, ytype="compensated", ylevel=1),
        steps=10),
    # moving-window laser wakefield: 2000 x 256 cells, box 40 x 51.2,
    # dt 0.014, 3000 steps; Gaussian laser a0 2, omega0 10, W0 4, FWHM 2,
    # start 17, focus 20, axis 25.6, polarisation along y; cold electrons of
    # density 1 from x = 20, 4x2 ppc; binomial x smoothing, level 4
    # (em2d/input/lwfa.c at the larger box)
    "c5_lwfa": dict(
        nx=[2000, 256], box=[40.0, 51.2], dt=0.014,
        species=[dict(name="e", m_q=-1.0, ppc=[4, 2], density=dict(type="step", start=20.0))],
        laser=dict(type="gaussian", start=17.0, fwhm=2.0, a0=2.0, omega0=10.0, W0=4.0,
                   focus=20.0, axis=25.6, polarization=0.0),
        moving_window=True,
        smooth=dict(xtype="binomial", xlevel=4),
        steps=3000),
}
