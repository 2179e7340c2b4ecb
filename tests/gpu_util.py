"""Helpers for the GPU parity tests: mirror an oracle simulation onto the
CUDA path (same particles, same fields, same settings) and compare."""
import numpy as np

from decks import DECKS, FUNCS, _resolve, build_cpu


def ext_grid(fn, nx, ny, dx, dy):
    """Evaluates a custom field callback on every buffer cell, reference layout."""
    g = np.zeros((ny + 3, nx + 3, 3), dtype=np.float32)
    for j in range(-1, ny + 2):
        for i in range(-1, nx + 2):
            # the callback sees the cell sizes as the C float values, in double
            g[j + 1, i + 1] = fn(i, float(np.float32(dx)), j, float(np.float32(dy)))
    return g


def column_injector(deck, cpu):
    """Injection provider for cold decks: the particles the reference injects
    in column nx-1 when the window moves (uniform / step lattice, zero
    momentum plus fluid drift).  Only valid when uth == 0."""
    nx, ny = deck["nx"]
    dx = np.float32(np.float32(deck["box"][0]) / np.float32(nx))
    specs = deck["species"]

    def inject(k, n_move):
        sp = specs[k]
        assert not any(sp.get("uth", [0, 0, 0])), "column injector needs a cold species"
        px, py = sp["ppc"]
        dens = sp.get("density", {"type": "uniform"})
        xs = (np.float32(1.0) / np.float32(px)) * (np.arange(px, dtype=np.float64) + 0.5)
        ys = (np.float32(1.0) / np.float32(py)) * (np.arange(py, dtype=np.float64) + 0.5)
        xs = xs.astype(np.float32)
        ys = ys.astype(np.float32)
        out = []
        i = nx - 1
        for j in range(ny):
            for b in range(py):
                for a in range(px):
                    if dens.get("type", "uniform") == "step":
                        edge = np.float32(np.float32(dens["start"]) / np.float32(dx)) - np.float32(n_move)
                        if not (np.float32(i + xs[a]) > edge):
                            continue
                    out.append((i, j, xs[a], ys[b]) + tuple(sp.get("ufl", [0, 0, 0])))
        arr = np.zeros(len(out), dtype=[("ix", "<i4"), ("iy", "<i4"), ("x", "<f4"), ("y", "<f4"),
                                         ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4")])
        for n, r in enumerate(out):
            arr[n] = r
        return arr

    return inject


def mirror(name, tile=(16, 16), deck=None, cpu=None, injector=None, **kw):
    """Builds the deck on the oracle and mirrors its state onto the GPU
    (extra keywords go to CudaSim: fast_math, sort_every, ...)."""
    from zpic_gb300._zc import CudaSim

    d = deck or DECKS[name]
    cpu = cpu or build_cpu(name, deck=d)
    g = CudaSim(d["nx"], d["box"], d["dt"], tile=tile, **kw)
    for k, sp in enumerate(d["species"]):
        g.add_species(sp["m_q"], cpu.q(k), sp["ppc"], cpu.particles(k))
    g.set_fields(E=cpu.E(), B=cpu.B())
    if "ext_fld" in d:
        e = _resolve(d["ext_fld"])
        nx, ny = d["nx"]
        dx = np.float32(d["box"][0]) / np.float32(nx)
        dy = np.float32(d["box"][1]) / np.float32(ny)
        kw = {}
        for f in ("E", "B"):
            t = e.get(f + "_type", "none")
            kw[f + "_type"] = t
            if t == "uniform":
                kw[f + "_0"] = e[f + "_0"]
            elif t == "custom":
                kw[f + "_grid"] = ext_grid(e[f + "_custom"], nx, ny, dx, dy)
        g.set_ext_fld(**kw)
    if d.get("moving_window"):
        g.set_moving_window()
        g.set_injector(injector or column_injector(d, cpu))
    if "smooth" in d:
        g.set_smooth(**d["smooth"])
    return cpu, g


def canon(parts):
    """Particles in a canonical order (all fields as the sort key)."""
    keys = [parts[f].view(np.uint32) if parts.dtype[f] == np.float32 else parts[f]
            for f in ("uz", "uy", "ux", "y", "x", "iy", "ix")]
    return parts[np.lexsort(keys)]


def field_err(a, b):
    """Largest component-wise relative L2 error over the interior."""
    a = np.asarray(a, dtype=np.float64)[1:-2, 1:-2]
    b = np.asarray(b, dtype=np.float64)[1:-2, 1:-2]
    errs = []
    for c in range(3):
        nb = np.linalg.norm(b[..., c])
        na = np.linalg.norm(a[..., c] - b[..., c])
        errs.append(0.0 if nb == 0 and na == 0 else na / max(nb, 1e-30))
    return max(errs)


def field_err_joint(a, b):
    """Relative L2 error of the whole vector field (all three components
    together) over the interior."""
    a = np.asarray(a, dtype=np.float64)[1:-2, 1:-2]
    b = np.asarray(b, dtype=np.float64)[1:-2, 1:-2]
    nb = np.linalg.norm(b)
    na = np.linalg.norm(a - b)
    return 0.0 if nb == 0 and na == 0 else na / max(nb, 1e-30)


def field_err_components(a, b):
    """Relative L2 error of each component over the interior."""
    a = np.asarray(a, dtype=np.float64)[1:-2, 1:-2]
    b = np.asarray(b, dtype=np.float64)[1:-2, 1:-2]
    out = []
    for c in range(3):
        nb = np.linalg.norm(b[..., c])
        na = np.linalg.norm(a[..., c] - b[..., c])
        out.append(0.0 if nb == 0 and na == 0 else na / max(nb, 1e-30))
    return np.array(out)


def reordered_twin(name, deck=None, seed=0):
    """The oracle on the same deck with every species' particles in a
    shuffled buffer order: the same physics, only the float32 order of the
    current sums differs.  How far it drifts from the oracle in unshuffled
    order is the floor of any implementation that sums in another order."""
    twin = build_cpu(name, deck=deck)
    rng = np.random.default_rng(seed)
    for k in range(twin.n_species):
        p = twin.particles(k)
        twin.set_particles(k, p[rng.permutation(p.size)])
    return twin


def check_fields(g, cpu, twin, where, bar=1e-5):
    """The spec's bar, per field and per component: each of E, B, J within
    ``bar`` relative L2 of the oracle as a whole vector field, and each
    component within ``bar`` or, where summation order alone moves it
    further (currents that cancel between species or within a cell), within
    twice the oracle's own drift under reordering (``twin``).  Returns the
    largest per-component error for reporting."""
    worst = 0.0
    for f in ("E", "B", "J"):
        a, b, t = getattr(g, f)(), getattr(cpu, f)(), getattr(twin, f)()
        joint = field_err_joint(a, b)
        assert joint <= bar, f"{f} relative error {joint:.2e} (whole field) {where}"
        err, floor = field_err_components(a, b), field_err_components(t, b)
        for c in range(3):
            assert err[c] <= max(bar, 2 * floor[c]), \
                f"{f}{'xyz'[c]} relative error {err[c]:.2e} (order floor {floor[c]:.2e}) {where}"
        worst = max(worst, float(err.max()))
    return worst
