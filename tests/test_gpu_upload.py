"""Particle upload (zc_species_set_particles): records in page-locked host
memory are read in place by the staging kernel, any other buffer (pageable,
or not 4-byte aligned) is copied to the device first.  Every route must give
the same particles, the same sorted tile layout and the same run."""
import numpy as np
import pytest

from decks import DECKS, build_cpu
from gpu_util import canon
from test_gpu_parity import _tile_runs, tile_slot

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _pinned_copy(parts, offset=0):
    """The records in page-locked host memory, `offset` bytes into the buffer."""
    raw = torch.empty(parts.nbytes + 64, dtype=torch.uint8, pin_memory=True).numpy()
    view = raw[offset:offset + parts.nbytes].view(parts.dtype)
    view[:] = parts
    return raw, view


def _check_layout(p, tile, nx):
    t, cell = _tile_runs(p, tile, nx)
    assert np.all(np.diff(t) >= 0), "particles grouped by tile"
    starts = np.flatnonzero(np.r_[True, np.diff(t) != 0, True])
    for a, b in zip(starts[:-1], starts[1:]):
        order = np.array([tile_slot(i, b - a) for i in range(b - a)])
        assert np.all(np.diff(cell[a:b][order]) >= 0), "tile in cell order through tile_slot"


def _run(name, cpu, parts_by_species, tile):
    from zpic_gb300._zc import CudaSim

    g = CudaSim(cpu.nx, cpu.box, cpu.dt, tile=tile, deterministic=True)
    for k, parts in enumerate(parts_by_species):
        sp = DECKS[name]["species"][k]
        g.add_species(sp["m_q"], cpu.q(k), sp["ppc"], parts)
    g.set_fields(E=cpu.E(), B=cpu.B())
    return g


@pytest.mark.parametrize("offset", [0, 4, 2], ids=["pinned", "pinned+4", "pinned+2 (copied)"])
def test_pinned_upload_matches_pageable(offset):
    tile = (16, 16)
    cpu = build_cpu("weibel_smooth")
    pageable = [cpu.particles(k) for k in range(cpu.n_species)]
    keep, pinned = [], []
    for p in pageable:
        raw, view = _pinned_copy(p, offset)
        keep.append(raw)
        pinned.append(view)
    ga = _run("weibel_smooth", cpu, pageable, tile)
    gb = _run("weibel_smooth", cpu, pinned, tile)
    for k in range(cpu.n_species):
        pa, pb = ga.particles(k), gb.particles(k)
        _check_layout(pb, tile, cpu.nx[0])
        assert canon(pa).tobytes() == canon(pb).tobytes() == canon(pageable[k]).tobytes()
    ga.step(6)
    gb.step(6)
    for f in ("E", "B", "J"):
        assert np.array_equal(getattr(ga, f)(), getattr(gb, f)()), f
    ga.close()
    gb.close()


def test_reupload_and_empty_upload():
    """set_particles replaces the species (also with nothing), from either memory."""
    tile = (32, 16)
    cpu = build_cpu("thermal")
    p = cpu.particles(0)
    g = _run("thermal", cpu, [p], tile)
    raw, view = _pinned_copy(p[::-1].copy())
    g.set_particles(0, view)
    assert g.count(0) == p.size
    q = g.particles(0)
    _check_layout(q, tile, cpu.nx[0])
    assert canon(q).tobytes() == canon(p).tobytes()
    g.set_particles(0, p[:0])
    assert g.count(0) == 0
    g.set_particles(0, p[: p.size // 3])
    assert g.count(0) == p.size // 3
    assert canon(g.particles(0)).tobytes() == canon(p[: p.size // 3]).tobytes()
    g.close()
