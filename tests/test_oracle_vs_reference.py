"""Pins the CPU oracle against the reference itself, compiled headlessly from its own
sources (oracle/build_ref.py).  Bit-for-bit equality (every bit of every FP64 value,
signs of zero included) is required for every update, boundary rule, source schedule,
Neumann gather, energy sum and setup table.
Skipped when the compiled reference is absent (tests/test_golden.py then pins the
oracle against committed fixtures made by the same compiled reference)."""
import numpy as np
import pytest

import oracle
import ref_variants
import refio
from helpers import PULSE_CASES, params_of, pulse_inputs, variant_inputs

pytestmark = pytest.mark.skipif(not refio.available("s_dir"), reason="compiled reference absent")

STEP_VARIANTS = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "wb_fn" and not v.get("dropin")]


def same_bits(a, b):
    """FP64 arrays equal in every bit (signs of zero and NaN payloads included)."""
    a, b = np.ascontiguousarray(a, np.float64), np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))
ENERGY_VARIANTS = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "we_fn"]
OSC_VARIANTS = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "osc"]


@pytest.mark.parametrize("variant", STEP_VARIANTS)
@pytest.mark.parametrize("nsteps", [1, 5, 30])
def test_evolve_wave_bitexact(variant, nsteps):
    p, f, xy, nbc = variant_inputs(variant, seed=nsteps)
    ref = refio.run(variant, p.nx, p.ny, refio.STEP, nsteps, fields=f, xy=xy, nbc=nbc)
    new, prev, third, t = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"],
                                     nsteps, nbc=nbc)
    assert t == nsteps
    assert same_bits(new, ref["phi"])
    assert same_bits(prev, ref["psi"])
    assert same_bits(third, ref["tmp"])
    assert oracle.energy_total(p, new, prev, xy, compensated=False) == ref["energy"]


@pytest.mark.parametrize("variant", ["s_abs", "s_dir"])
def test_point_source_bitexact(variant):
    p, f, xy, nbc = variant_inputs(variant, seed=3)
    inside = np.argwhere(xy.reshape(p.nx, p.ny) > 0)[7]
    p.src_on, p.src_i, p.src_j, p.src_amp, p.src_period = 1, int(inside[0]), int(inside[1]), 0.05, 23.7
    ref = refio.run(variant, p.nx, p.ny, refio.STEP, 40, fields=f, xy=xy,
                    src=(p.src_i, p.src_j, p.src_amp, p.src_period))
    new, prev, third, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], 40)
    assert same_bits(new, ref["phi"]) and same_bits(prev, ref["psi"])


@pytest.mark.parametrize("variant", OSC_VARIANTS)
def test_oscillating_bc_bitexact(variant):
    p = params_of(variant)
    times = [1, 2, 3, 17, 100, 251, 999, 5000]
    ref = refio.run(variant, p.nx, p.ny, refio.OSC, times=times)
    mine = np.array([[oracle.oscillating_bc(p, t, j) for j in range(p.ny)] for t in times])
    assert same_bits(mine, ref)


@pytest.mark.parametrize("variant", ENERGY_VARIANTS)
@pytest.mark.parametrize("nsteps", [1, 9, 31])
def test_wave_energy_variant_bitexact(variant, nsteps):
    p, f, xy, _ = variant_inputs(variant, seed=10 + nsteps)
    circles = [(-0.5, 0.1, 0.2), (0.7, -0.3, 0.15)]
    ref = refio.run(variant, p.nx, p.ny, refio.STEP, nsteps, fields=f, xy=xy, circles=circles)
    bufs = [f["phi"].copy(), f["psi"].copy(), f["tmp"].copy()]
    cur, prv, fre = 0, 1, 2
    for s in range(1, nsteps + 1):
        oracle.evolve_wave_half_energy(p, s, bufs[cur], bufs[prv], bufs[fre], xy)
        cur, prv, fre = fre, cur, prv
    assert same_bits(bufs[cur], ref["phi"])
    assert same_bits(bufs[prv], ref["psi"])
    assert same_bits(bufs[fre], ref["tmp"])
    # compute_energy_x and compute_energy_tblr of the reference on the same state
    assert same_bits(oracle.energy_x(p, bufs[cur], bufs[prv], xy), ref["energy_x"])
    ileft, iright = box_limits(p, circles)
    assert same_bits(oracle.energy_tblr(p, bufs[cur], bufs[prv], xy, ileft, iright), ref["tblr"])


def box_limits(p, circles):
    """ileft/iright of compute_energy_tblr (sub_wave_comp.c:1764-1785)."""
    xleft, xright = p.xmax, p.xmin
    for xc, yc, r in circles:
        if xc - r < xleft:
            xleft = xc - r
        if xc + r > xright:
            xright = xc + r
    return (int((xleft - p.xmin) / (p.xmax - p.xmin) * p.nx),
            int((xright - p.xmin) / (p.xmax - p.xmin) * p.nx))


@pytest.mark.parametrize("variant,domain,kw", [
    ("full_neu_ellipse", 1, dict(lam=1.8)),
    ("full_neu_polygon", 8, dict(lam=0.9, npoly=7, apoly=0.3)),
])
def test_neumann_setup_bitexact(variant, domain, kw):
    p = params_of(variant)
    ref = refio.run(variant, p.nx, p.ny, refio.SETUP)
    xy0 = oracle.mask(p, domain, kw["lam"], kw.get("npoly", 6), kw.get("apoly", 0.0))
    xy, recs = oracle.init_neumann(p, domain, kw["lam"], xy0, npoly=kw.get("npoly", 6),
                                   apoly=kw.get("apoly", 0.0))
    assert np.array_equal(xy, ref["xy"])
    assert len(recs) == len(ref["nbc"]) > 0
    for name in ["nx", "ny", "nbi1", "nbj1", "nbi2", "nbj2", "i", "j", "active", "signx1", "signy2"]:
        assert np.array_equal(recs[name], ref["nbc"][name]), name
    # tables of init_ior_2d, which the reference builds before the ghosts are marked
    tcc, tc, tg = oracle.init_ior(p, xy0)
    assert same_bits(tcc, ref["tcc"]) and same_bits(tg, ref["tgamma"])
    assert same_bits(tc, ref["tc"])


def test_mask_and_tables_c2_discs():
    """Config-2 mask (64 seeded discs, D_CIRCLES) and two-speed tables of the
    reference, against the oracle and the product's host setup."""
    from youtube_simulations_gb300 import scenes
    p = params_of("c2")
    rng = np.random.default_rng(0)
    discs = scenes.seeded_discs(rng, 64)
    ref = refio.run("c2", p.nx, p.ny, refio.SETUP, circles=discs)
    xy = oracle.mask(p, 20, 1.8, circles=discs)
    assert np.array_equal(xy, ref["xy"])
    assert np.array_equal(scenes.mask(p, 20, circles=discs), ref["xy"])
    tcc, tc, tg = scenes.tables(p, ref["xy"])
    assert same_bits(tcc, ref["tcc"]) and same_bits(tc, ref["tc"]) and same_bits(tg, ref["tgamma"])


@pytest.mark.parametrize("variant,domain,lam", [("c1", 1, 1.8), ("full_stadium", 2, 1.2)])
def test_mask_setup_bitexact(variant, domain, lam):
    from youtube_simulations_gb300 import scenes
    p = params_of(variant)
    ref = refio.run(variant, p.nx, p.ny, refio.SETUP)
    assert np.array_equal(oracle.mask(p, domain, lam), ref["xy"])
    assert np.array_equal(scenes.mask(p, domain, lam=lam), ref["xy"])
    tcc, tc, tg = scenes.tables(p, ref["xy"])
    assert same_bits(tcc, ref["tcc"]) and same_bits(tg, ref["tgamma"])


@pytest.mark.parametrize("variant,factor,x,y", PULSE_CASES)
def test_add_circular_wave_bitexact(variant, factor, x, y):
    """add_circular_wave (wave_common.c:337-351) of the reference's full build against
    the oracle, bit for bit (psi untouched)."""
    if not refio.available(variant):
        pytest.skip("full build absent")
    p, m, phi, psi, xy = pulse_inputs(variant)
    ref = refio.run(variant, p.nx, p.ny, refio.PULSE, fields={"phi": phi, "psi": psi}, xy=xy, pulse=(factor, x, y))
    mine = oracle.add_circular_wave(p, m["INITIAL_AMP"], factor, x, y, m["INITIAL_VARIANCE"], m["INITIAL_WAVELENGTH"],
                                    phi, xy)
    assert same_bits(mine, ref["phi"])
    assert same_bits(psi, ref["psi"])
    assert not np.array_equal(mine, phi)
