"""ctypes binding of libwavegpu.so (C ABI in include/wavegpu.h).

Mirrors the reference's function surface for Python callers and tests:
``evolve_wave_half`` / ``evolve_wave`` (wave_billiard.c:302-631) take fields as
``[NX][NY]`` numpy arrays whose rows stand in for the reference's ``double *phi[NX]``
row pointers; ``Scene`` wraps the native handle API.  There is no CPU fallback: if the
library is missing or a GPU is not present, every call raises.
"""
import ctypes
from pathlib import Path

import numpy as np

from . import params as P

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libwavegpu.so"
_lib = None


class WaveGpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"wavegpu status {status}: {msg}")
        self.status = status


def lib():
    """Load the in-tree library (building it first if it is absent)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import build
            build.build()
        if not LIB_PATH.exists():
            raise WaveGpuError(-2, f"{LIB_PATH} missing: run the build")
        _lib = ctypes.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


_V, _I32, _I64, _D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
_PP = ctypes.POINTER(ctypes.c_void_p)

SIGNATURES = {
    "wg_abi_version": (_I32, []),
    "wg_last_error": (ctypes.c_char_p, []),
    "wg_status_string": (ctypes.c_char_p, [_I32]),
    "wg_params_default": (None, [_V, _I32, _I32]),
    "wg_dropin_configure": (_I32, [_V]),
    "wg_dropin_set_mode": (_I32, [_I32]),
    "wg_dropin_set_rows": (_I32, [_I32]),
    "wg_dropin_sync": (_I32, []),
    "wg_dropin_invalidate": (_I32, []),
    "wg_dropin_get_time": (_I32, [ctypes.POINTER(_I64)]),
    "wg_dropin_set_time": (_I32, [_I64]),
    "wg_evolve_wave_half": (_I32, [_PP, _PP, _PP, _PP, _PP, _PP, _PP, _V, _I32]),
    "wg_evolve_wave": (_I32, [_PP, _PP, _PP, _PP, _PP, _PP, _PP, _V, _I32]),
    "wg_evolve_wave_half_energy": (_I32, [_PP, _PP, _PP, _PP]),
    "wg_evolve_wave_energy": (_I32, [_PP, _PP, _PP, _PP]),
    "wg_compute_energy": (_I32, [_PP, _PP, _PP, _I32, _I32, ctypes.POINTER(_D)]),
    "wg_compute_energy_x_all": (_I32, [_PP, _PP, _PP, _V]),
    "wg_compute_energy_tblr": (_I32, [_PP, _PP, _PP, _I32, _I32, _V]),
    "wg_compute_energy_device_noalloc": (_I32, [_V, _V, _V, _V, _I32, _I32, _I32, _V, _V]),
    "wg_dropin_add_circular_wave": (_I32, [_D, _D, _D, _D, _D, _D, _PP, _PP, _PP]),
    "wg_dropin_cell": (_I32, [_PP, _I32, _I32, ctypes.POINTER(_D)]),
    "wg_scene_create": (_I32, [_V, _I32, _I32, _V, ctypes.POINTER(_V)]),
    "wg_scene_destroy": (_I32, [_V]),
    "wg_scene_bytes": (_I32, [_V, _I32, _I32, ctypes.POINTER(ctypes.c_size_t)]),
    "wg_scene_upload": (_I32, [_V, _V, _V, _V, _V, _V, _V]),
    "wg_scene_upload_state": (_I32, [_V, _V, _V, _I32]),
    "wg_scene_set_neumann": (_I32, [_V, _V, _I32]),
    "wg_scene_step": (_I32, [_V, _I32]),
    "wg_scene_download": (_I32, [_V, _V, _V, _I32]),
    "wg_scene_energy": (_I32, [_V, _V, _V, _I32, _I32, _V]),
    "wg_scene_get_time": (_I32, [_V, ctypes.POINTER(_I64)]),
    "wg_scene_set_time": (_I32, [_V, _I64]),
    "wg_scene_sync": (_I32, [_V]),
    "wg_scene_set_blocking": (_I32, [_V, _I32, _I32, _I32]),
    "wg_scene_get_blocking": (_I32, [_V, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "wg_scene_launch_count": (_I32, [_V, ctypes.POINTER(_I64)]),
    "wg_scene_check_finite": (_I32, [_V, ctypes.POINTER(_I64)]),
    "wg_scene_frame_rgb8": (_I32, [_V, _V, _V, _V, _V]),
    "wg_scene_frame_reset": (_I32, [_V]),
    "wg_scene_build_domain": (_I32, [_V, _I32, _D, _I32, _D, _V, _I32]),
    "wg_scene_download_mask": (_I32, [_V, _V]),
    "wg_scene_neumann_records": (_I32, [_V, _V, _I32, ctypes.POINTER(_I32)]),
    "wg_write_tiff": (_I32, [ctypes.c_char_p, ctypes.c_char_p, _V, _I32, _I32]),
    "wg_write_ppm": (_I32, [ctypes.c_char_p, _V, _I32, _I32]),
    "wg_scene_set_probes": (_I32, [_V, _I32, _V, _V, _I32]),
    "wg_scene_read_probes": (_I32, [_V, _V, _I32, ctypes.POINTER(_I32)]),
    "wg_scene_add_circular_wave": (_I32, [_V, _D, _D, _D, _D, _D, _D]),
    "wg_batch_create": (_I32, [_I32, _V, ctypes.POINTER(_V)]),
    "wg_batch_destroy": (_I32, [_V]),
    "wg_batch_add": (_I32, [_V, _V, _V, _V, _V, ctypes.POINTER(_I32)]),
    "wg_batch_remove": (_I32, [_V, _I32]),
    "wg_batch_step": (_I32, [_V, _I32]),
    "wg_batch_download": (_I32, [_V, _I32, _V, _V]),
    "wg_batch_energy": (_I32, [_V, _I32, ctypes.POINTER(_D)]),
    "wg_batch_count": (_I32, [_V, ctypes.POINTER(_I32), ctypes.POINTER(_I64)]),
    "wg_batch_launch_count": (_I32, [_V, ctypes.POINTER(_I64)]),
    "wg_batch_set_skew": (_I32, [_V, _I32]),
    "wg_batch_skew_depths": (_I32, [_V, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(ctypes.c_double)]),
    "wg_server_create": (_I32, [_V, _V, ctypes.POINTER(_V)]),
    "wg_server_destroy": (_I32, [_V]),
    "wg_server_submit": (_I32, [_V, _V, _V, _V, _V, _I32, _I32, ctypes.POINTER(_I64)]),
    "wg_server_tick": (_I32, [_V, ctypes.POINTER(_I32)]),
    "wg_server_drain": (_I32, [_V, ctypes.POINTER(_I32)]),
    "wg_server_cancel": (_I32, [_V, _I64]),
    "wg_server_frame": (_I32, [_V, _I64, _V, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "wg_server_result": (_I32, [_V, _I64, _V, _V]),
    "wg_server_request_state": (_I32, [_V, _I64, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "wg_server_get_stats": (_I32, [_V, _V]),
    "wg_server_request_bytes": (_I32, [_V, _V, ctypes.POINTER(ctypes.c_uint64)]),
}


def _declare(L):
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args


def check(status):
    if status != 0:
        raise WaveGpuError(status, lib().wg_last_error().decode(errors="replace"))


def _rows(a, ctype):
    """Row-pointer array (the reference's `double *phi[NX]`) into a 2-D numpy array."""
    assert a.ndim == 2 and a.flags.c_contiguous
    base = a.ctypes.data
    stride = a.strides[0]
    arr = (ctypes.c_void_p * a.shape[0])(*[base + i * stride for i in range(a.shape[0])])
    return ctypes.cast(arr, _PP), arr


class RowFields:
    """Keeps numpy arrays and their row-pointer tables alive across drop-in calls,
    so that resident mode sees stable row-array identities, as the reference's
    animation() does with its phi/psi/tmp arrays."""

    def __init__(self, params, phi, psi, tmp, xy, tcc=None, tc=None, tgamma=None):
        nx, ny = params.nx, params.ny
        shape = (nx, ny)
        self.params = params
        self.phi = np.ascontiguousarray(np.asarray(phi, np.float64).reshape(shape)).copy()
        self.psi = np.ascontiguousarray(np.asarray(psi, np.float64).reshape(shape)).copy()
        self.tmp = np.ascontiguousarray(np.asarray(tmp, np.float64).reshape(shape)).copy()
        self.xy = np.ascontiguousarray(np.asarray(xy, np.int16).reshape(shape)).copy()
        z = np.zeros(shape)
        self.tcc = z.copy() if tcc is None else np.asarray(tcc, np.float64).reshape(shape).copy()
        self.tc = z.copy() if tc is None else np.asarray(tc, np.float64).reshape(shape).copy()
        self.tgamma = z.copy() if tgamma is None else np.asarray(tgamma, np.float64).reshape(shape).copy()
        self._r = {k: _rows(getattr(self, k), None) for k in ("phi", "psi", "tmp", "xy", "tcc", "tc", "tgamma")}

    def rows(self, name):
        return self._r[name][0]


def configure(params):
    check(lib().wg_dropin_configure(ctypes.byref(params)))


def set_mode(resident):
    check(lib().wg_dropin_set_mode(1 if resident else 0))


def sync():
    check(lib().wg_dropin_sync())


def invalidate():
    check(lib().wg_dropin_invalidate())


def _nbc(nbc):
    if nbc is None or len(nbc) == 0:
        return None, 0
    nbc = np.ascontiguousarray(nbc, dtype=P.NEUMANN_DTYPE)
    return nbc.ctypes.data, len(nbc), nbc


def evolve_wave_half(f, src="phi", prev="psi", dst="tmp", nbc=None):
    """evolve_wave_half(phi_in=f.src, psi_in=f.prev, phi_out=f.dst) on a RowFields."""
    ptr = _nbc(nbc)
    check(lib().wg_evolve_wave_half(f.rows(src), f.rows(prev), f.rows(dst), f.rows("xy"), f.rows("tcc"),
                                    f.rows("tc"), f.rows("tgamma"), ptr[0], ptr[1]))


def evolve_wave(f, nbc=None):
    ptr = _nbc(nbc)
    check(lib().wg_evolve_wave(f.rows("phi"), f.rows("psi"), f.rows("tmp"), f.rows("xy"), f.rows("tcc"),
                               f.rows("tc"), f.rows("tgamma"), ptr[0], ptr[1]))


def evolve_wave_energy(f):
    check(lib().wg_evolve_wave_energy(f.rows("phi"), f.rows("psi"), f.rows("tmp"), f.rows("xy")))


def evolve_wave_half_energy(f, src="phi", prev="psi", dst="tmp"):
    check(lib().wg_evolve_wave_half_energy(f.rows(src), f.rows(prev), f.rows(dst), f.rows("xy")))


def compute_energy(f, i, j, a="phi", b="psi"):
    out = ctypes.c_double()
    check(lib().wg_compute_energy(f.rows(a), f.rows(b), f.rows("xy"), i, j, ctypes.byref(out)))
    return out.value


def compute_energy_x(f, a="phi", b="psi"):
    out = np.zeros(f.params.nx)
    check(lib().wg_compute_energy_x_all(f.rows(a), f.rows(b), f.rows("xy"), out.ctypes.data))
    return out


def compute_energy_tblr(f, ileft, iright, a="phi", b="psi"):
    out = np.zeros(6)
    check(lib().wg_compute_energy_tblr(f.rows(a), f.rows(b), f.rows("xy"), ileft, iright, out.ctypes.data))
    return out


def add_circular_wave(f, factor, x, y, init_amp=1.0, variance=0.0003, wavelength=0.01, a="phi", b="psi"):
    """wg_dropin_add_circular_wave: the reference's add_circular_wave (wave_common.c:337-351)
    on the row arrays of a RowFields (or on their resident device copy)."""
    check(lib().wg_dropin_add_circular_wave(init_amp, factor, x, y, variance, wavelength, f.rows(a), f.rows(b),
                                            f.rows("xy")))


def dropin_cell(f, i, j, a="phi"):
    """wg_dropin_cell: phi[i][j] of a RowFields, from the resident device copy if there is one."""
    v = _D()
    check(lib().wg_dropin_cell(f.rows(a), int(i), int(j), ctypes.byref(v)))
    return v.value


def write_tiff(path, rgb, description=""):
    """wg_write_tiff: an RGB8 frame [rows][cols][3] (row 0 at the bottom) as writetiff's TIFF."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    check(lib().wg_write_tiff(str(path).encode(), description.encode(), rgb.ctypes.data, rgb.shape[1], rgb.shape[0]))


def write_ppm(path, rgb):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    check(lib().wg_write_ppm(str(path).encode(), rgb.ctypes.data, rgb.shape[1], rgb.shape[0]))


def write_time_series(path, values):
    """Lines of SAVE_TIME_SERIES (wave_billiard.c:900-908): (long int)(v*1e16) as %019ld."""
    with open(path, "w") as f:
        for v in np.asarray(values, np.float64).reshape(-1):
            f.write("%019d\n" % int(v * 1.0e16))


def dropin_time():
    t = ctypes.c_int64()
    check(lib().wg_dropin_get_time(ctypes.byref(t)))
    return t.value


def set_dropin_time(t):
    check(lib().wg_dropin_set_time(int(t)))


class Scene:
    """Native resident scene (wg_scene_*)."""

    def __init__(self, params, precision=P.FP64, coef=P.COEF_MASK, stream=None):
        self.params = params.copy()
        self.precision, self.coef = precision, coef
        h = ctypes.c_void_p()
        check(lib().wg_scene_create(ctypes.byref(self.params), precision, coef,
                                    None if stream is None else ctypes.c_void_p(stream), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().wg_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def dtype(self):
        return np.float32 if self.precision == P.FP32 else np.float64

    def upload(self, phi, psi, xy, tcc=None, tc=None, tgamma=None):
        keep = [np.ascontiguousarray(a, np.float64).reshape(-1) if a is not None else None
                for a in (phi, psi, tcc, tc, tgamma)]
        xy = np.ascontiguousarray(xy, np.int16).reshape(-1)
        ptr = [None if a is None else a.ctypes.data for a in keep]
        check(lib().wg_scene_upload(self.h, ptr[0], ptr[1], xy.ctypes.data, ptr[2], ptr[3], ptr[4]))

    def upload_state(self, phi, psi):
        a = np.ascontiguousarray(phi)
        b = np.ascontiguousarray(psi)
        prec = P.FP32 if a.dtype == np.float32 else P.FP64
        check(lib().wg_scene_upload_state(self.h, a.ctypes.data, b.ctypes.data, prec))
        check(lib().wg_scene_sync(self.h))

    def set_neumann(self, nbc):
        nbc = np.ascontiguousarray(nbc, dtype=P.NEUMANN_DTYPE)
        check(lib().wg_scene_set_neumann(self.h, nbc.ctypes.data if len(nbc) else None, len(nbc)))

    def step(self, n):
        check(lib().wg_scene_step(self.h, int(n)))

    def sync(self):
        check(lib().wg_scene_sync(self.h))

    def download(self, native=False):
        """(phi, psi) in FP64, or in the scene's precision with native=True; an FP32 scene
        returns psi = phi - v formed in FP64."""
        n = self.params.nx * self.params.ny
        dt = self.dtype if native else np.float64
        phi, psi = np.empty(n, dt), np.empty(n, dt)
        prec = self.precision if native else P.FP64
        check(lib().wg_scene_download(self.h, phi.ctypes.data, psi.ctypes.data, prec))
        return phi, psi

    def energy(self, ileft=0, iright=0):
        total = ctypes.c_double()
        cols = np.zeros(self.params.nx)
        boxes = np.zeros(6)
        check(lib().wg_scene_energy(self.h, ctypes.byref(total), cols.ctypes.data, ileft, iright, boxes.ctypes.data))
        return total.value, cols, boxes

    def add_circular_wave(self, factor, x, y, init_amp=1.0, variance=0.0003, wavelength=0.01):
        """add_circular_wave (wave_common.c:337-351) on the scene's phi."""
        check(lib().wg_scene_add_circular_wave(self.h, init_amp, factor, x, y, variance, wavelength))

    def total_energy(self):
        total = ctypes.c_double()
        check(lib().wg_scene_energy(self.h, ctypes.byref(total), None, 0, 0, None))
        return total.value

    @property
    def time(self):
        t = ctypes.c_int64()
        check(lib().wg_scene_get_time(self.h, ctypes.byref(t)))
        return t.value

    @time.setter
    def time(self, t):
        check(lib().wg_scene_set_time(self.h, int(t)))

    def set_blocking(self, k, tile_i=0, tile_j=0):
        check(lib().wg_scene_set_blocking(self.h, int(k), int(tile_i), int(tile_j)))

    def blocking(self):
        k, ti, tj = _I32(), _I32(), _I32()
        check(lib().wg_scene_get_blocking(self.h, ctypes.byref(k), ctypes.byref(ti), ctypes.byref(tj)))
        return k.value, ti.value, tj.value

    def launches(self):
        n = _I64()
        check(lib().wg_scene_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def build_domain(self, domain, lam=1.8, npoly=6, apoly=0.0, circles=None):
        """wg_scene_build_domain: the mask (and tables) on the device; then upload_state."""
        c = np.zeros((0, 3)) if circles is None else np.ascontiguousarray(np.asarray(circles, np.float64)[:, :3])
        check(lib().wg_scene_build_domain(self.h, int(domain), float(lam), int(npoly), float(apoly),
                                          c.ctypes.data if len(c) else None, len(c)))

    def neumann_records(self):
        """The Neumann records built on the device by build_domain (NEUMANN_DTYPE array)."""
        n = _I32()
        check(lib().wg_scene_neumann_records(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=P.NEUMANN_DTYPE)
        if n.value:
            check(lib().wg_scene_neumann_records(self.h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def download_mask(self):
        xy = np.zeros(self.params.nx * self.params.ny, np.int16)
        check(lib().wg_scene_download_mask(self.h, xy.ctypes.data))
        return xy

    def set_probes(self, cells, capacity):
        """wg_scene_set_probes: record phi at cells [(i, j), ...] after every update."""
        cells = np.asarray(cells, np.int32).reshape(-1, 2)
        ii, jj = np.ascontiguousarray(cells[:, 0]), np.ascontiguousarray(cells[:, 1])
        check(lib().wg_scene_set_probes(self.h, len(cells), ii.ctypes.data, jj.ctypes.data, int(capacity)))
        self._nprobes, self._probe_cap = len(cells), int(capacity)

    def read_probes(self, max_updates=None):
        """The recorded samples [update][probe], oldest first (at most max_updates)."""
        n = getattr(self, "_nprobes", 0)
        if n == 0:
            return np.zeros((0, 0))
        c = _I32()
        out = np.zeros((self._probe_cap if max_updates is None else min(max_updates, self._probe_cap), n))
        check(lib().wg_scene_read_probes(self.h, out.ctypes.data, out.shape[0], ctypes.byref(c)))
        return out[:c.value].copy()

    def frame_reset(self):
        check(lib().wg_scene_frame_reset(self.h))

    def nonfinite(self):
        n = _I64()
        check(lib().wg_scene_check_finite(self.h, ctypes.byref(n)))
        return n.value

    def frame_rgb8(self, lut, size=2, vshift=-0.2, vscale=1.0, slope=1.0, color_range=0.8, scale=1.0,
                   fade=False, fade_value=1.0, fade_in_obstacle=False, plot=P.P_AMPLITUDE, log_shift=0.75,
                   log_scale=0.75, flux_scale=250.0, avrg_e_factor=0.95, attenuation=0.0, time=0):
        """wg_scene_frame_rgb8; the keyword defaults are wave_billiard.c's macros."""
        fp = P.WgFrameParams(size, int(fade), vshift, vscale, slope, color_range, scale, fade_value,
                             int(fade_in_obstacle), int(plot), log_shift, log_scale, flux_scale, avrg_e_factor,
                             attenuation, int(time), 0)
        lut = np.ascontiguousarray(lut, np.uint8).reshape(256, 3)
        out = np.zeros((self.params.ny // size, self.params.nx // size, 3), np.uint8)
        check(lib().wg_scene_frame_rgb8(self.h, ctypes.byref(fp), lut.ctypes.data, out.ctypes.data, None))
        return out


def scene_bytes(params, precision=P.FP32, coef=P.COEF_MASK):
    n = ctypes.c_size_t()
    check(lib().wg_scene_bytes(ctypes.byref(params), precision, coef, ctypes.byref(n)))
    return n.value


class Batch:
    """Uneven scenes advanced together, each frame replayed as a CUDA graph (wg_batch_*):
    single updates by one persistent kernel per update, or skewed passes of 2..6 updates
    for FP32 scenes with mirror, absorbing or periodic boundaries (same fields bit for
    bit).  FP32 scenes hold phi and the velocity phi - psi.  Masks are 0/1 (WG_COEF_MASK
    coefficients)."""

    def __init__(self, precision=P.FP32, stream=None):
        h = ctypes.c_void_p()
        check(lib().wg_batch_create(precision, None if stream is None else ctypes.c_void_p(stream), ctypes.byref(h)))
        self.h, self.precision, self.params = h, precision, {}

    def close(self):
        if self.h:
            lib().wg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add(self, params, phi, psi, xy):
        a = np.ascontiguousarray(phi, np.float64).reshape(-1)
        b = np.ascontiguousarray(psi, np.float64).reshape(-1)
        m = np.ascontiguousarray(xy, np.int16).reshape(-1)
        slot = _I32()
        check(lib().wg_batch_add(self.h, ctypes.byref(params), a.ctypes.data, b.ctypes.data, m.ctypes.data,
                                 ctypes.byref(slot)))
        self.params[slot.value] = params.copy()
        return slot.value

    def remove(self, slot):
        check(lib().wg_batch_remove(self.h, int(slot)))
        self.params.pop(slot, None)

    def step(self, n):
        check(lib().wg_batch_step(self.h, int(n)))

    def set_skew(self, mode):
        """Skewed passes: -1 tuned per size class (default), 0 off, 2..6 a fixed depth."""
        check(lib().wg_batch_set_skew(self.h, int(mode)))

    def skew_depths(self):
        """(depth per size class [16], autotuner ms per update [16, 8] by class and depth);
        size class = floor(log2(cells)) - 10, clamped to 0..15."""
        d, _, ms = self.skew_tuning()
        return d, ms

    def skew_tuning(self):
        """(depth [16], row chunk [16] (0: list-wide size), ms per update [16, 8]) per size class."""
        d = (_I32 * 16)()
        r = (_I32 * 16)()
        ms = (ctypes.c_double * 128)()
        check(lib().wg_batch_skew_depths(self.h, d, r, ms))
        return list(d), list(r), np.array(ms[:]).reshape(16, 8)

    def download(self, slot):
        if slot not in self.params:  # let the library report the unknown slot
            check(lib().wg_batch_download(self.h, int(slot), None, None))
        p = self.params[slot]
        phi, psi = np.empty(p.nx * p.ny), np.empty(p.nx * p.ny)
        check(lib().wg_batch_download(self.h, int(slot), phi.ctypes.data, psi.ctypes.data))
        return phi, psi

    def energy(self, slot):
        e = ctypes.c_double()
        check(lib().wg_batch_energy(self.h, int(slot), ctypes.byref(e)))
        return e.value

    def count(self):
        n, c = _I32(), _I64()
        check(lib().wg_batch_count(self.h, ctypes.byref(n), ctypes.byref(c)))
        return n.value, c.value

    def launches(self):
        n = _I64()
        check(lib().wg_batch_launch_count(self.h, ctypes.byref(n)))
        return n.value


class Server:
    """Serving loop (wg_server_*): requests admitted under an HBM budget into a running
    batch, one frame per tick for every resident scene, RGB8 frames to host memory.
    pipeline=True: a tick enqueues its device work and then waits for the previous
    tick's frames (drain() waits for the last one)."""

    def __init__(self, lut, precision=P.FP32, steps_per_frame=10, max_scenes=512, hbm_budget=150 << 30,
                 size=2, vshift=-0.2, vscale=1.0, slope=1.0, color_range=0.8, scale=1.0, stream=None,
                 plot=P.P_AMPLITUDE, pipeline=False):
        cfg = P.WgServerConfig()
        cfg.precision, cfg.steps_per_frame, cfg.max_scenes, cfg.hbm_budget = precision, steps_per_frame, max_scenes, hbm_budget
        cfg.pipeline = 1 if pipeline else 0
        cfg.frame = P.WgFrameParams(size, 0, vshift, vscale, slope, color_range, scale, 1.0, 0, int(plot))
        lut = np.ascontiguousarray(lut, np.uint8).reshape(-1)
        ctypes.memmove(cfg.lut, lut.ctypes.data, 768)
        h = ctypes.c_void_p()
        check(lib().wg_server_create(ctypes.byref(cfg), None if stream is None else ctypes.c_void_p(stream),
                                     ctypes.byref(h)))
        self.h, self.params = h, {}

    def close(self):
        if self.h:
            lib().wg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, params, phi, psi, xy, frames, keep=False):
        a = np.ascontiguousarray(phi, np.float64).reshape(-1)
        b = np.ascontiguousarray(psi, np.float64).reshape(-1)
        m = np.ascontiguousarray(xy, np.int16).reshape(-1)
        rid = _I64()
        check(lib().wg_server_submit(self.h, ctypes.byref(params), a.ctypes.data, b.ctypes.data, m.ctypes.data,
                                     int(frames), int(keep), ctypes.byref(rid)))
        self.params[rid.value] = params.copy()
        return rid.value

    def tick(self):
        n = _I32()
        check(lib().wg_server_tick(self.h, ctypes.byref(n)))
        return n.value

    def drain(self):
        n = _I32()
        check(lib().wg_server_drain(self.h, ctypes.byref(n)))
        return n.value

    def cancel(self, rid):
        check(lib().wg_server_cancel(self.h, int(rid)))

    def state(self, rid):
        st, fd = _I32(), _I32()
        check(lib().wg_server_request_state(self.h, int(rid), ctypes.byref(st), ctypes.byref(fd)))
        return st.value, fd.value

    def frame(self, rid):
        """(frame index, RGB8 image) of the request's latest frame; read it before the next
        tick renders over the host buffer (wg_server_frame refuses a stale frame)."""
        w, h, idx = _I32(), _I32(), _I32()
        check(lib().wg_server_frame(self.h, int(rid), None, ctypes.byref(idx), ctypes.byref(w), ctypes.byref(h)))
        out = np.empty((h.value, w.value, 3), np.uint8)
        check(lib().wg_server_frame(self.h, int(rid), out.ctypes.data, ctypes.byref(idx), None, None))
        return idx.value, out

    def result(self, rid):
        p = self.params[rid]
        phi, psi = np.empty(p.nx * p.ny), np.empty(p.nx * p.ny)
        check(lib().wg_server_result(self.h, int(rid), phi.ctypes.data, psi.ctypes.data))
        return phi, psi

    def request_bytes(self, params):
        n = ctypes.c_uint64()
        check(lib().wg_server_request_bytes(self.h, ctypes.byref(params), ctypes.byref(n)))
        return n.value

    def stats(self):
        st = P.WgServerStats()
        check(lib().wg_server_get_stats(self.h, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in st._fields_}
