"""Temporally blocked FP32 passes (k_step_tb) against the oracle and against the
single-step FP32 kernel, on grids of several tiles in both directions, for every
boundary rule the blocked form covers (mirror "Dirichlet" edges, absorbing edges,
OSCILLATE_LEFT, OSCILLATE_TOPBOT, FLOOR, TWOSPEEDS, the point source) and each depth
and tile shape the autotuner may pick.  Against the FP64 oracle: 1e-5 relative to the
field maximum.  Against the single-step FP32 kernels: equal bit for bit, since every
FP32 stepper applies the same per-cell rules (bulk update, edge32 on the boundary
lines, the source added in FP64)."""
import numpy as np
import pytest

import oracle
from helpers import equalize_unwritten, params_of, rel_err
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu


# Widths put column ny-1 at each of the four positions of a four-column group
# (517: first, 518: second, 611: third, 520: last).
WIDTH = {"dir_kappa_floor": 517, "abs_twospeeds_src": 517, "abs_stadium": 520, "topbot": 518}


def case(name, nx=301, ny=None, seed=0):
    rng = np.random.default_rng(seed)
    ny = ny or WIDTH.get(name, 517)
    over = dict(nx=nx, ny=ny)
    if name == "dir_kappa_floor":
        p = params_of("s_dir", **over)
        xy = scenes.mask(p, scenes.D_ELLIPSE, lam=1.8)
    elif name == "abs_twospeeds_src":
        p = params_of("s_abs", **over)
        discs = scenes.seeded_discs(rng, 12, 0.05, 0.2)
        xy = scenes.mask(p, scenes.D_CIRCLES, circles=discs)
        inside = np.argwhere(xy.reshape(nx, ny) > 0)
        if len(inside):  # tiny grids may hold no disc cell: no source then
            si, sj = inside[len(inside) // 3]
            p.src_on, p.src_i, p.src_j, p.src_amp, p.src_period = 1, int(si), int(sj), 0.05, 31.0
    elif name == "abs_stadium":
        p = params_of("s_abs_mask", **over)
        xy = scenes.mask(p, scenes.D_STADIUM, lam=3.0)
    elif name == "topbot":
        p = params_of("s_topbot", **over)
        xy = scenes.mask(p, scenes.D_ELLIPSE, lam=1.8)
    elif name == "osc_left_tall":
        p = params_of("s_square", nx=97, ny=611)
        p.oscil_left_yshift = 4.0
        xy = scenes.mask(p, scenes.D_RECTANGLE, lam=3.0)
    else:
        raise KeyError(name)
    tcc, tc, tg = scenes.tables(p, xy)
    x, y = scenes.grid_xy(p)
    phi = scenes.pulse(p, np.ones(p.nx * p.ny, np.int16), 0.3, 0.1, variance=0.1 ** 2)
    phi = np.where(scenes.tables(p, xy)[0] != 0, phi, 0.0)
    f = dict(phi=phi, psi=phi * 0.99, tmp=np.zeros_like(phi), tcc=tcc, tc=tc, tgamma=tg)
    f = equalize_unwritten(p, f, xy)
    return p, f, xy


CASES = ["dir_kappa_floor", "abs_twospeeds_src", "abs_stadium", "topbot", "osc_left_tall"]
SHAPES = [(2, 32, 256), (4, 32, 128), (5, 48, 256), (8, 64, 128), (3, 16, 256),
          (2, 64, 1), (3, 37, 1), (4, 24, 1), (4, 128, 1), (2, 8, 1), (5, 16, 1), (6, 40, 1)]


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("coef", [P.COEF_MASK, P.COEF_TABLE])
def test_blocked_matches_oracle_and_single_step(name, coef):
    p, f, xy = case(name)
    n = 37
    new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], n)
    with W.Scene(p, P.FP32, coef) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.set_blocking(1)
        s.step(n)
        ref1, ref1p = s.download()
    for k, L, Wd in SHAPES:
        with W.Scene(p, P.FP32, coef) as s:
            s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
            s.set_blocking(k, L, Wd)
            s.step(n)
            assert s.time == n
            phi, psi = s.download()
        assert rel_err(phi, new) <= 1e-5, (k, L, Wd)
        assert rel_err(psi, prev) <= 1e-5, (k, L, Wd)
        assert np.array_equal(phi, ref1), (k, L, Wd)
        assert np.array_equal(psi, ref1p), (k, L, Wd)


def test_autotuned_blocking_and_launch_count():
    p, f, xy = case("abs_twospeeds_src", nx=640, ny=700)
    with W.Scene(p, P.FP32, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.step(1)  # autotunes on a copy of the state
        k, L, Wd = s.blocking()
        assert k >= 1
        before = s.launches()
        s.step(40)
        launched = s.launches() - before
        if k > 1:
            assert launched <= 40 // k + 8
        phi, _ = s.download()
        assert s.time == 41
    new, _, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], 41)
    assert rel_err(phi, new) <= 1e-5


@pytest.mark.parametrize("nx,ny", [(3, 8), (5, 9), (9, 8), (17, 12), (20, 131), (64, 124)])
@pytest.mark.parametrize("name", ["dir_kappa_floor", "abs_twospeeds_src"])
def test_skewed_blocking_on_small_and_odd_grids(nx, ny, name):
    """Grids where every task of the skewed pass takes the general rule (fewer than
    2(K+1)+1 rows), where one column tile holds both boundary columns, and odd widths."""
    p, f, xy = case(name, nx=nx, ny=ny, seed=1)
    n = 13
    new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], n)
    with W.Scene(p, P.FP32, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.set_blocking(1)
        s.step(n)
        ref1, ref1p = s.download()
    for k, L in [(2, 8), (3, 16), (6, 16)]:
        with W.Scene(p, P.FP32, P.COEF_TABLE) as s:
            s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
            s.set_blocking(k, L, 1)
            s.step(n)
            phi, psi = s.download()
        assert rel_err(phi, new) <= 1e-5, (k, L)
        assert rel_err(psi, prev) <= 1e-5, (k, L)
        assert np.array_equal(phi, ref1) and np.array_equal(psi, ref1p), (k, L)


def test_skewed_blocking_refuses_narrow_grids():
    p, f, xy = case("dir_kappa_floor", nx=20, ny=7, seed=1)
    with W.Scene(p, P.FP32, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.set_blocking(3, 16, 1)
        with pytest.raises(W.WaveGpuError):
            s.step(6)
