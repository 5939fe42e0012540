"""Pins the frame oracle (oracle.frame_rgb8) against the reference's own colour path.

The reference colours each sampled cell with wave_value (wave_common.c:1053-1162):
color_scheme_palette / color_scheme_asym_palette (colors_waves.c:161-258),
color_amplitude (colors_waves.c:3-16) and amp_to_rgb_palette with COL_TURBO
(colormaps.c:2449-2482), i.e. an entry of turbo_srgb_floats (turbo_colormap.c); GL then
turns the float colour into a byte.  oracle/ref_driver.c's FRAME mode runs those
functions (compiled from the reference's sources) for every plot mode and returns the
float colours; here a byte is round-half-up(255 x colour).

The frame oracle (and the GPU frame kernels, which the frame tests hold to it) index the
byte table turbo_srgb_bytes instead.  turbo_srgb_bytes is round(255 x turbo_srgb_floats)
entry by entry (checked below), so every mode whose colour is a palette entry gives the
same bytes exactly.  The total-flux mode scales the entry by tanh(flux) and the fading
options by the fade factor: there the oracle rounds the scaled byte and the reference
the scaled float, and a byte may differ by one."""
import numpy as np
import pytest

import oracle
import refio
from helpers import params_of, turbo_palette

pytestmark = pytest.mark.skipif(not (refio.available("frame") and turbo_palette() is not None),
                                reason="compiled reference or its sources absent")

FRAME_ARGS = {  # oracle.frame_rgb8 keywords for each variant's macros (ref_variants.py)
    "frame": dict(vshift=-0.2, vscale=1.0, slope=1.0, color_range=0.8, attenuation=0.0, log_shift=0.75,
                  log_scale=0.75, flux_scale=250.0, avrg_e_factor=0.95),
    "frame_att": dict(vshift=0.1, vscale=2.0, slope=1.5, color_range=1.0, attenuation=0.01, log_shift=1.0,
                      log_scale=0.5, flux_scale=100.0, avrg_e_factor=0.9),
    "frame_ts": dict(vshift=-0.2, vscale=1.0, slope=1.0, color_range=0.8, attenuation=0.0, log_shift=0.75,
                     log_scale=0.75, flux_scale=250.0, avrg_e_factor=0.95),
}
SIZE, FRAMES, T0 = 2, 3, 5


def to_bytes(rgb):
    return np.clip(np.floor(255.0 * rgb + 0.5), 0, 255).astype(np.uint8)


def test_turbo_bytes_are_the_rounded_floats():
    b, f = turbo_palette()
    assert np.array_equal(b, to_bytes(f.astype(np.float64)))


def fields(variant, seed):
    p = params_of(variant)
    su = refio.run(variant, p.nx, p.ny, refio.SETUP)
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, p.nx)[:, None]
    y = np.linspace(-1, 1, p.ny)[None, :]
    phi = (0.6 * np.sin(3.1 * x + 1.7 * y) + 0.3 * np.cos(5.3 * x * y) + 0.05 * rng.standard_normal((p.nx, p.ny)))
    psi = phi * 0.97 + 0.02 * rng.standard_normal((p.nx, p.ny))
    return p, phi.reshape(-1), psi.reshape(-1), su["xy"], su["tcc"]


@pytest.mark.parametrize("variant", list(FRAME_ARGS))
@pytest.mark.parametrize("plot", range(10))
def test_frame_oracle_matches_reference(variant, plot):
    p, phi, psi, xy, tcc = fields(variant, seed=plot)
    rgb, _, _ = refio.frame(variant, p.nx, p.ny, phi, psi, xy, tcc, plot, size=SIZE, frames=FRAMES, t0=T0)
    ref = to_bytes(rgb)
    m = xy.reshape(p.nx, p.ny)[::SIZE, ::SIZE][: p.nx // SIZE, : p.ny // SIZE].T
    drawn = (m != 0) | bool(p.twospeeds)
    ref[~drawn] = 0  # draw_wave_highres_palette draws only these cells
    lut = turbo_palette()[0]
    state = {}
    for k in range(FRAMES):
        mine = oracle.frame_rgb8(p, phi, xy, lut, size=SIZE, plot=plot, psi=psi, state=state, time=T0 + k,
                                 **FRAME_ARGS[variant])
    diff = np.abs(mine.astype(int) - ref.astype(int))
    if plot == 7:  # the entry scaled by tanh(flux): one byte of rounding either way
        assert diff.max() <= 1
        assert np.mean(diff == 0) >= 0.5
    else:
        assert np.array_equal(mine, ref), (int(diff.max()), int(np.count_nonzero(diff)))


@pytest.mark.parametrize("plot", [0, 1])
def test_frame_oracle_fade_matches_reference(plot):
    """FADE_IN_OBSTACLE (init_fade_table: (tcc/courant^2)^0.1) in a two-speed scene."""
    variant = "frame_ts"
    p, phi, psi, xy, tcc = fields(variant, seed=11)
    rgb, _, fade = refio.frame(variant, p.nx, p.ny, phi, psi, xy, tcc, plot, size=SIZE, frames=1, t0=T0)
    ref = to_bytes(rgb * fade[..., None])
    mine = oracle.frame_rgb8(p, phi, xy, turbo_palette()[0], size=SIZE, plot=plot, psi=psi, time=T0,
                             fade_in_obstacle=True, tcc=tcc, **FRAME_ARGS[variant])
    diff = np.abs(mine.astype(int) - ref.astype(int))
    assert diff.max() <= 1
    assert np.mean(diff == 0) >= 0.5
