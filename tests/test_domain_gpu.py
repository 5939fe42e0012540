"""Masks and tables built on the device (wg_scene_build_domain) against the oracle's
restatement of xy_in_billiard_single_domain (pinned to the reference's own SETUP) and
init_ior_2d.  Masks: equal cell for cell; for the polygon, whose cos/sin are CUDA's,
a cell may differ only where it lies within 1e-12 of an edge.  Tables: an FP64 table
scene built on the device steps bit for bit like the same scene uploaded from the host
(uniform and per-cell tgamma, absorbing tc)."""
import math

import numpy as np
import pytest

import oracle
from helpers import params_of
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu

DISCS = scenes.seeded_discs(np.random.default_rng(4), 24, 0.05, 0.25)
DOMAINS = [
    ("rectangle", scenes.D_RECTANGLE, dict(lam=1.7)),
    ("ellipse", scenes.D_ELLIPSE, dict(lam=1.8)),
    ("stadium", scenes.D_STADIUM, dict(lam=1.2)),
    ("polygon", scenes.D_POLYGON, dict(lam=0.9, npoly=7, apoly=0.3)),
    ("discs", scenes.D_CIRCLES, dict(lam=1.8, circles=DISCS)),
    ("discs_in_rect", scenes.D_CIRCLES_IN_RECT, dict(lam=1.9, circles=DISCS)),
]


def polygon_margin(p, lam, npoly, apoly):
    """min over edges of c - (x cos + y sin) at every cell centre (the polygon test)."""
    x = p.xmin + np.arange(p.nx) * (p.xmax - p.xmin) / p.nx
    y = p.ymin + np.arange(p.ny) * (p.ymax - p.ymin) / p.ny
    X, Y = np.meshgrid(x, y, indexing="ij")
    omega = 6.283185307 / npoly
    c = lam * math.cos(omega * 0.5)
    m = np.full(X.shape, np.inf)
    for k in range(npoly):
        a = apoly * 1.570796327 + (k + 0.5) * omega
        m = np.minimum(m, c - (X * math.cos(a) + Y * math.sin(a)))
    return m.reshape(-1)


@pytest.mark.parametrize("name,domain,kw", DOMAINS)
@pytest.mark.parametrize("nx,ny", [(128, 96), (301, 517)])
def test_device_mask_matches_oracle(name, domain, kw, nx, ny):
    p = params_of("s_abs", nx=nx, ny=ny)
    ref = oracle.mask(p, domain, kw["lam"], kw.get("npoly", 6), kw.get("apoly", 0.0), circles=kw.get("circles"))
    with W.Scene(p, P.FP32, P.COEF_MASK) as s:
        s.build_domain(domain, **kw)
        got = s.download_mask()
    diff = got != (ref != 0)
    if domain == scenes.D_POLYGON:
        near = np.abs(polygon_margin(p, kw["lam"], kw["npoly"], kw["apoly"])) < 1e-12
        assert not np.any(diff & ~near)
    else:
        assert not np.any(diff)
    assert 0 < got.sum() < got.size


@pytest.mark.parametrize("variant,over", [
    ("s_abs", dict(twospeeds=1, gamma=1e-4, gammab=1e-4)),       # uniform tgamma, absorbing (tc)
    ("s_dir", dict(twospeeds=1, gamma=0.0, gammab=2e-4)),        # tgamma per cell
    ("s_dir", dict(twospeeds=0)),
])
def test_device_tables_step_like_host_upload(variant, over):
    p = params_of(variant, nx=96, ny=80)
    for k, v in over.items():
        setattr(p, k, v)
    xy = oracle.mask(p, scenes.D_CIRCLES, 1.8, circles=DISCS)
    tcc, tc, tg = oracle.init_ior(p, xy)
    rng = np.random.default_rng(2)
    phi = scenes.pulse(p, np.ones(p.nx * p.ny, np.int16), 0.2, -0.1, variance=0.05 ** 2) + \
        0.001 * rng.standard_normal(p.nx * p.ny)
    psi = phi * 0.98
    with W.Scene(p, P.FP64, P.COEF_TABLE) as a, W.Scene(p, P.FP64, P.COEF_TABLE) as b:
        a.upload(phi, psi, xy, tcc, tc, tg)
        b.build_domain(scenes.D_CIRCLES, lam=1.8, circles=DISCS)
        b.upload_state(phi, psi)
        a.step(20)
        b.step(20)
        pa, qa = a.download()
        pb, qb = b.download()
    assert np.array_equal(pa, pb) and np.array_equal(qa, qb)


def test_build_domain_refusals():
    p = params_of("s_neu")
    with W.Scene(p, P.FP64, P.COEF_MASK) as s:
        with pytest.raises(W.WaveGpuError):
            s.build_domain(scenes.D_ELLIPSE)
    p = params_of("s_abs")
    with W.Scene(p, P.FP64, P.COEF_MASK) as s:
        with pytest.raises(W.WaveGpuError):
            s.upload_state(np.zeros(p.nx * p.ny), np.zeros(p.nx * p.ny))   # no mask yet
        with pytest.raises(W.WaveGpuError):
            s.build_domain(5)


NEU = [("full_neu_ellipse", 301, 221), ("full_neu_polygon", 301, 221), ("full_neu_ellipse", 67, 45)]


@pytest.mark.parametrize("variant,nx,ny", NEU)
def test_device_neumann_setup_matches_oracle(variant, nx, ny):
    """init_neumann_bc on the device: the ghost marks (-1), and every record (cell,
    normal weights, neighbours, active flag) in the reference's order, against the
    oracle's restatement (pinned bit for bit to the reference's SETUP).  Ellipse: equal
    in every bit.  Polygon: its normal uses CUDA's atan/cos/sin, so weights agree to
    1e-12 and a cell within rounding of a side may take the neighbouring side's normal."""
    import ref_variants
    m = ref_variants.VARIANTS[variant]["macros"]
    p = params_of(variant, nx=nx, ny=ny)
    dom, lam, npoly, apoly = m["B_DOMAIN"], m["LAMBDA"], m["NPOLY"], m["APOLY"]
    mask = oracle.mask(p, dom, lam, npoly, apoly)
    ref_xy, ref = oracle.init_neumann(p, dom, lam, mask, npoly=npoly, apoly=apoly)
    with W.Scene(p, P.FP64, P.COEF_TABLE) as s:
        s.build_domain(dom, lam=lam, npoly=npoly, apoly=apoly)
        got_xy = s.download_mask()
        got = s.neumann_records()
    assert len(ref) > 0 and np.count_nonzero(ref_xy == -1) == len(ref)
    assert np.array_equal(got_xy, ref_xy)
    assert len(got) == len(ref)
    assert np.array_equal(got["i"], ref["i"]) and np.array_equal(got["j"], ref["j"])
    ints = ["signx1", "signy1", "signx2", "signy2", "nbi1", "nbj1", "nbi2", "nbj2", "top", "active"]
    if dom == scenes.D_ELLIPSE:
        for k in ints + ["nx", "ny"]:
            assert np.array_equal(got[k], ref[k]), k
    else:
        same = np.ones(len(ref), bool)
        for k in ints:
            same &= got[k] == ref[k]
        assert np.mean(same) >= 0.98
        assert np.max(np.abs(got["nx"][same] - ref["nx"][same])) <= 1e-12
        assert np.max(np.abs(got["ny"][same] - ref["ny"][same])) <= 1e-12


@pytest.mark.parametrize("prec", [P.FP64, P.FP32])
def test_device_neumann_scene_steps_like_host_setup(prec):
    """A Neumann ellipse scene built on the device steps bit for bit like the same scene
    uploaded from the host with the oracle's ghost marks, tables and records (tables from
    the mask before the ghost marks, as the reference calls init_ior_2d before
    init_neumann_bc)."""
    variant = "full_neu_ellipse"
    p = params_of(variant, nx=161, ny=121)
    mask = oracle.mask(p, scenes.D_ELLIPSE, 1.8)
    tcc, tc, tg = scenes.tables(p, mask)
    xy, nbc = oracle.init_neumann(p, scenes.D_ELLIPSE, 1.8, mask)
    rng = np.random.default_rng(3)
    x, y = scenes.grid_xy(p)
    phi = scenes.pulse(p, np.ones(p.nx * p.ny, np.int16), x[70], y[60], variance=0.05 ** 2)
    phi = np.where(xy != 0, phi + 0.01 * rng.standard_normal(p.nx * p.ny), 0.0)
    psi = phi * 0.99
    out = []
    for device in (False, True):
        with W.Scene(p, prec, P.COEF_TABLE) as s:
            if device:
                s.build_domain(scenes.D_ELLIPSE, lam=1.8)
                s.upload_state(phi, psi)
            else:
                s.upload(phi, psi, xy, tcc, tc, tg)
                s.set_neumann(nbc)
            s.step(40)
            out.append(s.download())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
