"""Argument checks of the C ABI, on CPU: every entry point below refuses a bad argument
with WG_ERR_INVALID and a message (wg_last_error) before it touches CUDA, so these
calls need no GPU.  The checks follow the reference's own limits where it has them
(NX, NY >= 3; B_COND 0..3; Neumann cells inside 1..NX-2 x 1..NY-2, global_pdes.c:518-528)
and the library's (a point source inside the grid with a non-zero period, a box of
non-zero size, the fixed scratch of the allocation-free energy entry point)."""
import ctypes

import numpy as np
import pytest

from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import wavegpu as W

INVALID = -1


@pytest.fixture(scope="module")
def lib():
    return W.lib()


def refused(lib, status, words):
    assert status == INVALID
    msg = lib.wg_last_error().decode()
    assert words in msg, msg


def create(lib, p, precision=P.FP32, coef=P.COEF_MASK):
    h = ctypes.c_void_p()
    st = lib.wg_scene_create(None if p is None else ctypes.byref(p), precision, coef, None, ctypes.byref(h))
    assert not h.value  # nothing created
    return st


@pytest.mark.parametrize("change, words", [
    (dict(nx=2), "NX and NY must be >= 3"),
    (dict(ny=1), "NX and NY must be >= 3"),
    (dict(b_cond=4), "B_COND 4 not supported"),
    (dict(src_on=1, src_i=64, src_j=3, src_period=30.0), "outside the grid"),
    (dict(src_on=1, src_i=3, src_j=3, src_period=0.0), "period must be non-zero"),
    (dict(xmin=1.0, xmax=1.0), "empty box"),
])
def test_scene_create_refuses_bad_params(lib, change, words):
    p = P.make_params(64, 48)
    for k, v in change.items():
        setattr(p, k, v)
    refused(lib, create(lib, p), words)


def test_scene_create_refuses_bad_modes(lib):
    p = P.make_params(64, 48)
    refused(lib, create(lib, None), "NULL")
    refused(lib, create(lib, p, precision=7), "precision")
    refused(lib, create(lib, p, coef=9), "coefficient mode")


def test_dropin_configure_refuses_bad_params(lib):
    refused(lib, lib.wg_dropin_configure(None), "NULL")
    p = P.make_params(2, 48)
    refused(lib, lib.wg_dropin_configure(ctypes.byref(p)), "NX and NY must be >= 3")


def test_batch_create_refuses_bad_precision(lib):
    h = ctypes.c_void_p()
    refused(lib, lib.wg_batch_create(5, None, ctypes.byref(h)), "precision")
    refused(lib, lib.wg_batch_create(P.FP32, None, None), "NULL")


def test_server_create_refuses_bad_config(lib):
    h = ctypes.c_void_p()
    refused(lib, lib.wg_server_create(None, None, ctypes.byref(h)), "NULL")
    cfg = P.WgServerConfig()
    cfg.precision, cfg.steps_per_frame, cfg.max_scenes, cfg.hbm_budget = P.FP32, 0, 4, 1 << 30
    cfg.frame = P.WgFrameParams(2, 0, -0.2, 1.0, 1.0, 0.8, 1.0, 1.0, 0, int(P.P_AMPLITUDE))
    refused(lib, lib.wg_server_create(ctypes.byref(cfg), None, ctypes.byref(h)), "bad server configuration")
    cfg.steps_per_frame = 10
    cfg.frame.plot = int(P.P_AMPLITUDE) + 1
    refused(lib, lib.wg_server_create(ctypes.byref(cfg), None, ctypes.byref(h)), "P_AMPLITUDE")
    assert not h.value


def test_noalloc_energy_refuses_before_any_cuda_call(lib):
    buf = np.zeros(16, np.float64)
    out = np.zeros(16, np.float64)
    ptr = buf.ctypes.data  # never dereferenced: every call below is refused first
    p = P.make_params(20000, 64)  # more columns than the fixed scratch holds
    refused(lib, lib.wg_compute_energy_device_noalloc(ctypes.byref(p), ptr, ptr, ptr, 64, 0, 0, out.ctypes.data, None),
            "exceeds the fixed scratch")
    p = P.make_params(64, 48)
    refused(lib, lib.wg_compute_energy_device_noalloc(ctypes.byref(p), ptr, ptr, ptr, 40, 0, 0, out.ctypes.data, None),
            "pitch")
    refused(lib, lib.wg_compute_energy_device_noalloc(ctypes.byref(p), ptr, ptr, ptr, 64, 10, 5, out.ctypes.data, None),
            "box limits")
    refused(lib, lib.wg_compute_energy_device_noalloc(ctypes.byref(p), None, ptr, ptr, 64, 0, 0, out.ctypes.data, None),
            "NULL")
