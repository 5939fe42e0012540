"""RGB8 frames of a scene (wg_scene_frame_rgb8) against the oracle's restatement of
draw_wave_highres_palette / wave_value for every plot mode (amplitude, energy, mixed,
mean, log, flux, total flux, average), with the running sums carried over frames.
The palette is the reference's turbo byte table (turbo_srgb_bytes, read at run time
from the reference's sources beside the compiled reference; a seeded byte table where
those are absent), the table test_frame_pin.py pins the oracle with.  tanh, log and atan on the GPU and in numpy may differ in the
last bit, which can move a value across a palette boundary: a few pixels (0.1-0.2%)
may differ."""
import numpy as np
import pytest

import oracle
from helpers import frame_lut, variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu


def lut(seed=0):
    return frame_lut(seed)


@pytest.mark.parametrize("prec,coef", [(P.FP64, P.COEF_TABLE), (P.FP32, P.COEF_MASK), (P.FP32, P.COEF_TABLE)])
@pytest.mark.parametrize("opts", [dict(), dict(size=1, fade=True, fade_value=0.7), dict(size=3, fade_in_obstacle=True)])
def test_frame_matches_oracle(prec, coef, opts):
    p, f, xy, _ = variant_inputs("s_abs", seed=5, smooth=True)
    if coef == P.COEF_MASK:
        tcc, tc, tg = scenes.tables(p, xy)
        f = dict(f, tcc=tcc, tc=tc, tgamma=tg)
    L = lut(1)
    with W.Scene(p, prec, coef) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.step(5)
        img = s.frame_rgb8(L, vshift=-0.1, slope=2.0, **opts)
        phi, _ = s.download()
    ref = oracle.frame_rgb8(p, phi, xy, L, vshift=-0.1, slope=2.0, tcc=f["tcc"] if coef == P.COEF_TABLE else None,
                            **opts)
    assert img.shape == ref.shape
    diff = np.any(img != ref, axis=-1)
    assert diff.mean() <= 1e-3


# chosen so that every mode gives a varied image on this scene (20 to 130 distinct colours)
PLOT_KW = dict(slope=1.5, scale=40.0, log_shift=0.75, log_scale=0.25, flux_scale=3.0e4, avrg_e_factor=0.9)


@pytest.mark.parametrize("plot", list(range(10)))
@pytest.mark.parametrize("prec", [P.FP64, P.FP32])
def test_frame_plot_modes_match_oracle(plot, prec):
    """Every P_* mode of wave_value (wave_common.c:1053-1162) over four frames, so that
    the running sums of the mean, average and total-flux modes accumulate."""
    p, f, xy, _ = variant_inputs("s_abs", seed=5, smooth=True)
    L = lut(2)
    state = {}
    with W.Scene(p, prec, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        for t in range(4):
            s.step(3)
            img = s.frame_rgb8(L, size=1, plot=plot, time=t, **PLOT_KW)
            phi, psi = s.download()
            ref = oracle.frame_rgb8(p, phi, xy, L, size=1, plot=plot, psi=psi, state=state, time=t, **PLOT_KW)
            diff = np.any(img != ref, axis=-1)
            assert diff.sum() <= max(2, 2e-3 * diff.size), (plot, t, int(diff.sum()))


def test_frame_reset_restarts_running_sums():
    p, f, xy, _ = variant_inputs("s_abs", seed=5, smooth=True)
    L = lut(3)
    with W.Scene(p, P.FP64, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        first = s.frame_rgb8(L, plot=P.P_MEAN_ENERGY, time=0, **PLOT_KW)
        s.frame_rgb8(L, plot=P.P_MEAN_ENERGY, time=0, **PLOT_KW)  # the sum is now twice the energy
        s.frame_reset()
        again = s.frame_rgb8(L, plot=P.P_MEAN_ENERGY, time=0, **PLOT_KW)
    assert np.array_equal(first, again)


def test_server_refuses_non_amplitude_frames():
    lut_ = lut(4)
    with pytest.raises(W.WaveGpuError):
        W.Server(lut_, precision=P.FP32, plot=P.P_ENERGY).close()
