"""add_circular_wave (wave_common.c:337-351) on the GPU against the oracle.

Scenes: FP64 within 1e-12 relative to the field maximum (exp and cos are CUDA's, not
the host libm's), FP32 within a few FP32 roundings; psi is never touched.  The c1 case
(1280x720) checks the support box: the cells outside it must equal the oracle's, which
adds an exact zero there.  The drop-in form in strict and resident mode, and resident
re-injection between steps as in the reference's animation loop (wave_billiard.c:916-934).
"""
import numpy as np
import pytest

import oracle
from helpers import PULSE_CASES, pulse_inputs, rel_err
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu


def reference(p, m, factor, x, y, phi, xy):
    return oracle.add_circular_wave(p, m["INITIAL_AMP"], factor, x, y, m["INITIAL_VARIANCE"], m["INITIAL_WAVELENGTH"],
                                    phi, xy)


def kw(m):
    return dict(init_amp=m["INITIAL_AMP"], variance=m["INITIAL_VARIANCE"], wavelength=m["INITIAL_WAVELENGTH"])


@pytest.mark.parametrize("variant,factor,x,y", PULSE_CASES)
@pytest.mark.parametrize("prec", [P.FP64, P.FP32])
def test_scene_add_circular_wave(variant, factor, x, y, prec):
    p, m, phi, psi, xy = pulse_inputs(variant)
    ref = reference(p, m, factor, x, y, phi, xy)
    with W.Scene(p, prec, P.COEF_MASK) as s:
        s.upload(phi, psi, xy)
        s.add_circular_wave(factor, x, y, **kw(m))
        got_phi, got_psi = s.download()
    if prec == P.FP64:
        assert rel_err(got_phi, ref) <= 1e-12
        assert np.array_equal(got_psi, psi)
        outside = ref == phi  # the cells the pulse leaves alone (an exact zero added)
        assert outside.any()
        assert np.array_equal(got_phi[outside], phi[outside])
    else:
        # FP32 scenes hold phi and the velocity phi - psi, which takes the same increment:
        # psi = phi - v comes back within FP32 roundings of the values involved
        assert np.max(np.abs(got_phi - ref)) <= 4 * np.finfo(np.float32).eps * np.max(np.abs(ref))
        scale = max(np.max(np.abs(ref)), np.max(np.abs(psi)))
        assert np.max(np.abs(got_psi - psi)) <= 8 * np.finfo(np.float32).eps * scale


def test_scene_add_circular_wave_rejects_bad_variance():
    p, m, phi, psi, xy = pulse_inputs("full_stadium")
    with W.Scene(p, P.FP64, P.COEF_MASK) as s:
        s.upload(phi, psi, xy)
        with pytest.raises(W.WaveGpuError):
            s.add_circular_wave(1.0, 0.0, 0.0, variance=0.0)


@pytest.mark.parametrize("resident", [False, True])
def test_dropin_add_circular_wave(resident):
    p, m, phi, psi, xy = pulse_inputs("full_neu_ellipse")
    factor, x, y = -1.1, 0.2, 0.05
    ref = reference(p, m, factor, x, y, phi, xy)
    W.configure(p)
    W.set_mode(resident)
    rf = W.RowFields(p, phi, psi, np.zeros_like(phi), xy)
    W.add_circular_wave(rf, factor, x, y, **kw(m))
    if resident:
        W.sync()
    assert rel_err(rf.phi.reshape(-1), ref) <= 1e-12
    assert np.array_equal(rf.psi.reshape(-1), psi)
    W.set_mode(False)


def test_dropin_resident_reinjection_between_steps():
    """evolve_wave, add_circular_wave, evolve_wave with the fields resident in HBM, as
    animation() does with an oscillating source (wave_billiard.c:897-934)."""
    p, m, phi, psi, xy = pulse_inputs("full_stadium")
    tcc, tc, tg = scenes.tables(p, xy)
    tmp = np.zeros_like(phi)
    a, b, c, _ = oracle.run(p, phi, psi, tmp, xy, tcc, tc, tg, 6)
    a = reference(p, m, 0.8, -0.3, 0.1, a, xy)
    new, prev, third, _ = oracle.run(p, a, b, c, xy, tcc, tc, tg, 6)
    W.configure(p)
    W.set_mode(True)
    rf = W.RowFields(p, phi, psi, tmp, xy, tcc, tc, tg)
    for _ in range(2):
        W.evolve_wave(rf)
    W.add_circular_wave(rf, 0.8, -0.3, 0.1, **kw(m))
    for _ in range(2):
        W.evolve_wave(rf)
    W.sync()
    assert rel_err(rf.phi.reshape(-1), new) <= 1e-12
    assert rel_err(rf.psi.reshape(-1), prev) <= 1e-12
    W.set_mode(False)
