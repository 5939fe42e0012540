"""RGB8 frames of a scene (wg_scene_frame_rgb8) against the oracle's restatement of
draw_wave_highres_palette's P_AMPLITUDE colour map.  The palette is a seeded
synthetic 256x3 byte table (the caller supplies the reference's own palette).
tanh on the GPU and in numpy may differ in the last bit, which can move a value across
a palette boundary: at most 0.1% of pixels may differ, by one palette step."""
import numpy as np
import pytest

import oracle
from helpers import variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu


def lut(seed=0):
    return np.random.default_rng(seed).integers(0, 256, size=(256, 3), dtype=np.uint8)


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
