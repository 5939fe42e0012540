"""Skewed passes in FP32 batches (k_batch_skew): frames of 2..6-update passes over many
scenes, written between two buffer pairs, at a depth (and row chunk) fixed or tuned per size class.

The skewed cells are the single-update cells, so every scene must come out bit for bit
as with the skewed passes off and as a native scene on the single-step kernels: over
frames of 10, 1 (single updates), 3, 7 and 2 updates, with admissions and removals
between frames, on grids from 3 to 300 rows and 5 to 300 columns (one tile, a partial
last lane group, no room for a skew: ny < 8), mirror and absorbing boundaries, an
oscillating left edge, a point source, two speeds and the FLOOR clamp.  Periodic scenes
take the skewed passes in the ghost layout (wrapped halos as ghost rows and columns),
including grids narrower than one tile and odd widths; a periodic scene with a point
source keeps single updates."""
import numpy as np
import pytest

from helpers import equalize_unwritten
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu

SHAPES = [  # nx, ny, boundary, extras
    (64, 64, P.BC_DIRICHLET, {}),
    (40, 128, P.BC_ABSORBING, {}),
    (130, 257, P.BC_PERIODIC, dict(floor=True)),   # ghost layout; leaves after the second frame
    (120, 250, P.BC_ABSORBING, dict(twospeeds=True)),
    (3, 40, P.BC_DIRICHLET, {}),
    (10, 13, P.BC_ABSORBING, {}),
    (17, 8, P.BC_DIRICHLET, dict(osc=True)),
    (300, 131, P.BC_DIRICHLET, dict(osc=True, src=True)),
    (90, 300, P.BC_ABSORBING, dict(floor=True)),
    (50, 5, P.BC_DIRICHLET, {}),          # ny < 8: single updates only
    (80, 96, P.BC_PERIODIC, {}),          # periodic: ghost layout
    (37, 129, P.BC_DIRICHLET, dict(src=True)),
    (9, 131, P.BC_PERIODIC, {}),          # fewer rows than the ghost rows
    (60, 70, P.BC_PERIODIC, dict(src=True)),  # a source: single updates only
    (200, 217, P.BC_DIRICHLET, dict(twospeeds=True, src=True)),
    (33, 45, P.BC_PERIODIC, dict(twospeeds=True)),  # narrower than a tile; arrives after the first frame
]
FRAMES = [10, 1, 3, 7, 2]


def scene(k, nx, ny, bc, ex):
    rng = np.random.default_rng(100 + k)
    p = scenes.make_params(nx, ny, b_cond=bc, courant=float(rng.uniform(0.05, 0.15)))
    xy = scenes.mask(p, scenes.D_ELLIPSE, lam=1.7)
    if xy.sum() < 4:
        xy = np.ones_like(xy)
    if ex.get("twospeeds"):
        p.twospeeds, p.courantb, p.gammab = 1, p.courant / 1.5, 1e-4
    if ex.get("osc"):
        p.oscillate_left, p.omega = 1, 0.07
    if ex.get("floor"):
        p.floor_clamp, p.vmax = 1, 0.3
    if ex.get("src"):
        inside = np.argwhere(xy.reshape(nx, ny) > 0)
        si, sj = inside[len(inside) // 2]
        p.src_on, p.src_i, p.src_j, p.src_amp, p.src_period = 1, int(si), int(sj), 0.05, 23.0
    phi = scenes.pulse(p, xy, 0.1, -0.05, variance=0.05 ** 2) + 0.01 * rng.standard_normal(nx * ny)
    f = equalize_unwritten(p, dict(phi=phi, psi=phi * 0.98, tmp=np.zeros_like(phi)), xy)
    return p, f, xy


def solo(p, f, xy, n):
    with W.Scene(p, P.FP32, P.COEF_MASK) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy)
        s.step(n)
        return s.download()


def run_batch(mode, ms, frames):
    """All scenes but the last two from the start; scene 2 leaves after the second frame,
    the last two arrive after the first."""
    out = {}
    with W.Batch(P.FP32) as b:
        b.set_skew(mode)
        slots = {k: b.add(p, f["phi"], f["psi"], xy) for k, (p, f, xy) in enumerate(ms[:-2])}
        done = {k: 0 for k in slots}
        for q, n in enumerate(frames):
            b.step(n)
            for k in done:
                done[k] += n
            if q == 0:
                for k in (len(ms) - 2, len(ms) - 1):
                    p, f, xy = ms[k]
                    slots[k] = b.add(p, f["phi"], f["psi"], xy)
                    done[k] = 0
            if q == 1:
                out[2] = (b.download(slots[2]), done.pop(2))
                b.remove(slots.pop(2))
        for k, sl in slots.items():
            out[k] = (b.download(sl), done[k])
        depths, rows, _ = b.skew_tuning()
    return out, (depths, rows)


@pytest.fixture(scope="module")
def members():
    return [scene(k, *s) for k, s in enumerate(SHAPES)]


@pytest.fixture(scope="module")
def unskewed(members):
    out, _ = run_batch(0, members, FRAMES)
    return out


def test_single_updates_match_native_scenes(members, unskewed):
    for k, ((phi, psi), n) in unskewed.items():
        p, f, xy = members[k]
        a, b = solo(p, f, xy, n)
        assert np.array_equal(phi, a) and np.array_equal(psi, b), k


@pytest.mark.parametrize("mode", [2, 3, 4, 5, 6, -1])
def test_skewed_passes_bit_identical(mode, members, unskewed):
    out, (depths, rows) = run_batch(mode, members, FRAMES)
    assert out.keys() == unskewed.keys()
    for k in out:
        (phi, psi), n = out[k]
        (phi0, psi0), n0 = unskewed[k]
        assert n == n0
        assert np.array_equal(phi, phi0), (mode, k, SHAPES[k])
        assert np.array_equal(psi, psi0), (mode, k, SHAPES[k])
    if mode > 0:
        assert set(depths) == {mode}
    else:  # every size class with a skewed scene got a depth of 2..6
        for nx, ny, bc, ex in SHAPES:
            c = min(15, max(0, int(np.floor(np.log2(nx * ny))) - 10))
            if ny >= 8 and not (bc == P.BC_PERIODIC and ex.get("src")):
                assert 2 <= depths[c] <= 6, (c, depths)
                assert rows[c] in (0, 32, 64, 128, 256), (c, rows)


def test_energy_after_skewed_frames_matches(members):
    p, f, xy = members[3]
    e = []
    for mode in (0, 4):
        with W.Batch(P.FP32) as b:
            b.set_skew(mode)
            s = b.add(p, f["phi"], f["psi"], xy)
            b.step(9)
            e.append(b.energy(s))
    assert e[0] == e[1]


def test_set_skew_rejects_bad_modes():
    with W.Batch(P.FP32) as b:
        for bad in (1, 7, -2):
            with pytest.raises(W.WaveGpuError):
                b.set_skew(bad)
