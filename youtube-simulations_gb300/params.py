"""ctypes/numpy mirrors of the C types in include/wavegpu.h.

``WgParams`` is the runtime form of the reference's compile-time macros
(wave_billiard.c:46-285); ``NEUMANN_DTYPE`` is the record layout of
``t_neumann_bc`` (global_pdes.c:518-528).
"""
import ctypes

import numpy as np

BC_DIRICHLET, BC_PERIODIC, BC_ABSORBING, BC_VPER_HABS = 0, 1, 2, 3
FP64, FP32 = 0, 1
COEF_MASK, COEF_TABLE = 0, 1


class WgParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("b_cond", ctypes.c_int32), ("twospeeds", ctypes.c_int32),
        ("bc_neumann", ctypes.c_int32), ("oscillate_left", ctypes.c_int32),
        ("oscillate_topbot", ctypes.c_int32), ("oscillation_schedule", ctypes.c_int32),
        ("floor_clamp", ctypes.c_int32), ("src_on", ctypes.c_int32),
        ("src_i", ctypes.c_int32), ("src_j", ctypes.c_int32),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
        ("courant", ctypes.c_double), ("courantb", ctypes.c_double),
        ("gamma", ctypes.c_double), ("gammab", ctypes.c_double),
        ("kappa", ctypes.c_double), ("kappa_sides", ctypes.c_double),
        ("kappa_topbot", ctypes.c_double),
        ("gamma_sides", ctypes.c_double), ("gamma_topbot", ctypes.c_double),
        ("omega", ctypes.c_double), ("omega_b", ctypes.c_double),
        ("amplitude", ctypes.c_double), ("damping", ctypes.c_double),
        ("achirp", ctypes.c_double),
        ("oscil_ymax", ctypes.c_double), ("oscil_ymid", ctypes.c_double),
        ("oscil_left_yshift", ctypes.c_double),
        ("initial_variance", ctypes.c_double), ("initial_shift", ctypes.c_double),
        ("wave_packet_shift", ctypes.c_double),
        ("vmax", ctypes.c_double), ("e_scale", ctypes.c_double),
        ("src_amp", ctypes.c_double), ("src_period", ctypes.c_double),
    ]

    def copy(self):
        out = WgParams()
        ctypes.pointer(out)[0] = self
        return out

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# Macro defaults of wave_billiard.c:46-285 for the fields wg_params shares, box of
# the benchmark configurations; the same values as wg_params_default() in C.
DEFAULTS = dict(
    b_cond=BC_DIRICHLET, twospeeds=0, bc_neumann=0, oscillate_left=0, oscillate_topbot=0,
    oscillation_schedule=0, floor_clamp=0, src_on=0, src_i=0, src_j=0,
    xmin=-2.0, xmax=2.0, ymin=-1.125, ymax=1.125,
    courant=0.1, courantb=0.05, gamma=0.0, gammab=0.0,
    kappa=0.0, kappa_sides=5.0e-4, kappa_topbot=0.0, gamma_sides=1.0e-4, gamma_topbot=1.0e-7,
    omega=0.005, omega_b=0.01, amplitude=1.0, damping=0.0, achirp=0.25,
    oscil_ymax=1.2, oscil_ymid=0.0, oscil_left_yshift=0.0,
    initial_variance=0.0003, initial_shift=20.0, wave_packet_shift=200.0,
    vmax=2.5, e_scale=300.0, src_amp=0.0, src_period=1.0,
)


def make_params(nx, ny, **kw):
    p = WgParams()
    vals = dict(DEFAULTS, nx=nx, ny=ny)
    for k, v in kw.items():
        if k not in vals:
            raise KeyError(f"unknown wg_params field {k!r}")
        vals[k] = v
    for k, v in vals.items():
        setattr(p, k, v)
    return p


NEUMANN_DTYPE = np.dtype([
    ("nx", "f8"), ("ny", "f8"),
    ("signx1", "i2"), ("signy1", "i2"), ("signx2", "i2"), ("signy2", "i2"),
    ("nbi1", "i4"), ("nbj1", "i4"), ("nbk1", "i4"),
    ("nbi2", "i4"), ("nbj2", "i4"), ("nbk2", "i4"),
    ("i", "i4"), ("j", "i4"), ("k", "i4"),
    ("top", "i2"), ("active", "i2"),
], align=True)
assert NEUMANN_DTYPE.itemsize == 64


# plot modes of draw_wave_highres_palette (global_pdes.c:318-327; wg_frame_params.plot)
(P_AMPLITUDE, P_ENERGY, P_MIXED, P_MEAN_ENERGY, P_LOG_ENERGY, P_LOG_MEAN_ENERGY, P_ENERGY_FLUX,
 P_TOTAL_ENERGY_FLUX, P_AVERAGE_ENERGY, P_LOG_AVERAGE_ENERGY) = range(10)


class WgFrameParams(ctypes.Structure):
    _fields_ = [
        ("size", ctypes.c_int32), ("fade", ctypes.c_int32),
        ("vshift", ctypes.c_double), ("vscale", ctypes.c_double),
        ("slope", ctypes.c_double), ("color_range", ctypes.c_double),
        ("scale", ctypes.c_double), ("fade_value", ctypes.c_double),
        ("fade_in_obstacle", ctypes.c_int32), ("plot", ctypes.c_int32),
        ("log_shift", ctypes.c_double), ("log_scale", ctypes.c_double),
        ("flux_scale", ctypes.c_double), ("avrg_e_factor", ctypes.c_double),
        ("attenuation", ctypes.c_double), ("time", ctypes.c_int32), ("reserved", ctypes.c_int32),
    ]


class WgServerConfig(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int32), ("steps_per_frame", ctypes.c_int32),
        ("max_scenes", ctypes.c_int32), ("pipeline", ctypes.c_int32),
        ("hbm_budget", ctypes.c_uint64), ("frame", WgFrameParams),
        ("lut", ctypes.c_uint8 * 768),
    ]


REQ_QUEUED, REQ_RESIDENT, REQ_DONE, REQ_CANCELLED = 0, 1, 2, 3


class WgServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64), ("admitted", ctypes.c_int64), ("completed", ctypes.c_int64),
        ("queued", ctypes.c_int64), ("resident", ctypes.c_int64), ("frames", ctypes.c_int64),
        ("ticks", ctypes.c_int64), ("cell_updates", ctypes.c_double), ("busy_seconds", ctypes.c_double),
        ("frame_latency_p50_ms", ctypes.c_double), ("frame_latency_p99_ms", ctypes.c_double),
        ("frame_latency_max_ms", ctypes.c_double), ("first_frame_p50_ms", ctypes.c_double),
        ("first_frame_p99_ms", ctypes.c_double), ("bytes_resident", ctypes.c_uint64),
        ("bytes_peak", ctypes.c_uint64), ("tick_device_p50_ms", ctypes.c_double),
        ("tick_device_p99_ms", ctypes.c_double), ("cancelled", ctypes.c_int64),
    ]
