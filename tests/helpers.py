"""Shared test inputs: deterministic seeded scenes for every compiled-reference variant."""
import re
from pathlib import Path

import numpy as np

import oracle
import ref_variants
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes


def params_of(variant, **over):
    d = ref_variants.params_dict(variant)
    d.update(over)
    nx, ny = d.pop("nx"), d.pop("ny")
    return P.make_params(nx, ny, **d)


def variant_inputs(variant, seed=1, noisy_tmp=True, smooth=False, **over):
    """(params, fields dict, xy, nbc) for a variant: its mask, spatially varying
    tables, a pulse plus noise in phi/psi, and (optionally) noise in tmp so that
    cells the stepper must not write are visible.  `over` replaces parameter values
    (e.g. oscillate_left=1 for a build of one oscillating_bc schedule)."""
    m = ref_variants.VARIANTS[variant]["macros"]
    p = params_of(variant, **over)
    rng = np.random.default_rng(seed)
    dom = m["B_DOMAIN"]
    if dom == 20:
        circ = scenes.seeded_discs(rng, 6, 0.1, 0.3)
        xy = scenes.mask(p, dom, circles=circ)
    else:
        xy = scenes.mask(p, dom, lam=m["LAMBDA"], npoly=m["NPOLY"], apoly=m["APOLY"])
    nbc = None
    if m["BC_NEUMANN"]:
        import oracle
        xy, nbc = oracle.init_neumann(p, dom, m["LAMBDA"], xy, npoly=m["NPOLY"], apoly=m["APOLY"])
    n = p.nx * p.ny
    tcc, tc, tg = scenes.tables(p, xy)
    tcc = tcc * (1.0 + 0.2 * rng.random(n))
    tc = tc * (1.0 + 0.2 * rng.random(n))
    tg = tg + 1e-3 * rng.random(n)
    if p.nx > 4 and p.ny > 4:
        inside = np.argwhere(xy.reshape(p.nx, p.ny) > 0)
        ci, cj = inside[len(inside) // 2] if len(inside) else (p.nx // 2, p.ny // 2)
    else:
        ci, cj = p.nx // 2, p.ny // 2
    x, y = scenes.grid_xy(p)
    phi = scenes.pulse(p, np.ones(n, np.int16), x[ci], y[cj], variance=0.15 ** 2)
    if not smooth:
        phi = phi + 0.05 * rng.standard_normal(n)
    psi = phi * 0.98 + (0.0 if smooth else 0.01 * rng.standard_normal(n))
    tmp = 0.3 * rng.standard_normal(n) if noisy_tmp else np.zeros(n)
    fields = dict(phi=phi, psi=psi, tmp=tmp, tcc=tcc, tc=tc, tgamma=tg)
    return p, fields, xy, nbc


# add_circular_wave cases: (variant, factor, x, y); full builds of the reference carry it
PULSE_CASES = [("full_stadium", -0.7, 0.31, -0.12), ("full_neu_ellipse", 1.3, -0.52, 0.21), ("c1", 0.9, 0.4, -0.3)]


def pulse_inputs(variant, seed=7):
    """(params, macros, phi, psi, xy) for an add_circular_wave case: the variant's mask
    (the oracle's restatement of the reference's, pinned elsewhere), seeded phi/psi."""
    m = ref_variants.VARIANTS[variant]["macros"]
    p = params_of(variant)
    xy = oracle.mask(p, m["B_DOMAIN"], m["LAMBDA"], m.get("NPOLY", 6), m.get("APOLY", 0.0))
    rng = np.random.default_rng(seed)
    phi = rng.standard_normal(p.nx * p.ny) * 0.01
    psi = rng.standard_normal(p.nx * p.ny) * 0.01
    return p, m, phi, psi, xy


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def written_cells(p, xy):
    """Cells the reference's stepper writes on every update (boundary lines with
    xy != 0 or TWOSPEEDS, interior with xy > 0 or TWOSPEEDS)."""
    xy2 = np.asarray(xy).reshape(p.nx, p.ny)
    w = (xy2 > 0) | bool(p.twospeeds)
    edge = np.zeros_like(w)
    edge[0, :] = edge[-1, :] = edge[:, 0] = edge[:, -1] = True
    w = np.where(edge, (xy2 != 0) | bool(p.twospeeds), w)
    return w.reshape(-1)


def equalize_unwritten(p, f, xy, nbc=None):
    """Make phi = psi = tmp on cells no update writes, so that the in-place two-buffer
    form of a native scene and the reference's three-buffer rotation hold the same
    values there (both then keep them)."""
    w = written_cells(p, xy).copy()
    if nbc is not None and len(nbc):
        act = nbc[nbc["active"] != 0]
        w.reshape(p.nx, p.ny)[act["i"], act["j"]] = True
    if p.oscillate_left:
        beam = p.oscillation_schedule in (42, 43, 44, 51)

        def y_to_j(y):
            return int((y - p.ymin) / (p.ymax - p.ymin) * p.ny)
        jmin, jmax = (y_to_j(p.oscil_ymid - p.oscil_ymax), y_to_j(p.oscil_ymid + p.oscil_ymax)) if beam else (0, p.ny - 1)
        col = w.reshape(p.nx, p.ny)[0]
        for j in range(p.ny - 1):
            if jmin < j < jmax:
                col[j] = True
        if not beam:
            col[0] = True
            if p.nx <= p.ny:
                col[p.nx - 1] = True
    f = dict(f)
    for k in ("psi", "tmp"):
        f[k] = np.where(w, f[k], f["phi"])
    return f


_TURBO_SRC = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "src" / "turbo_colormap.c"


def turbo_palette():
    """The reference's turbo palette (turbo_colormap.c: turbo_srgb_bytes [256][3] and
    turbo_srgb_floats [256][3]), read at run time from the snapshot of the reference's
    sources that oracle/build_ref.py keeps beside the compiled reference (git-ignored,
    never committed).  None when the snapshot is absent."""
    if not _TURBO_SRC.exists():
        return None
    text = _TURBO_SRC.read_text(encoding="latin-1")

    def table(name):
        m = re.search(name + r"\s*\[256\]\s*\[3\]\s*=\s*\{(.*?)\};", text, re.S)
        nums = re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", m.group(1))
        return np.array([float(x) for x in nums]).reshape(256, 3)
    return table("turbo_srgb_bytes").astype(np.uint8), table("turbo_srgb_floats").astype(np.float32)


def frame_lut(seed=0):
    """The palette of the frame tests: the reference's turbo bytes where its snapshot is
    present, else a seeded 256-entry byte table (the frame arithmetic does not depend on
    the entries)."""
    t = turbo_palette()
    if t is not None:
        return t[0]
    return np.random.default_rng(seed).integers(0, 256, size=(256, 3), dtype=np.uint8)
