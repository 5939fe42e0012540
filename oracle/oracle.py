"""ctypes binding of the CPU oracle (oracle/wave_oracle.c).  TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module.  Arrays are numpy, flat [nx][ny] (j contiguous) as the reference's rows.
"""
import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _setup(_lib)
    return _lib


_D = ctypes.POINTER(ctypes.c_double)
_S = ctypes.POINTER(ctypes.c_int16)
_V = ctypes.c_void_p


def _setup(L):
    L.wo_oscillating_bc.restype = ctypes.c_double
    L.wo_oscillating_bc.argtypes = [_V, ctypes.c_int, ctypes.c_int]
    L.wo_evolve_wave_half.argtypes = [_V, ctypes.c_long, _V, _V, _V, _V, _V, _V, _V, _V, ctypes.c_int]
    L.wo_evolve_wave_half_energy.argtypes = [_V, ctypes.c_long, _V, _V, _V, _V]
    L.wo_run.restype = ctypes.c_int
    L.wo_run.argtypes = [_V, ctypes.POINTER(ctypes.c_long), ctypes.c_int, ctypes.POINTER(_V),
                         _V, _V, _V, _V, _V, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.wo_compute_energy.restype = ctypes.c_double
    L.wo_compute_energy.argtypes = [_V, _V, _V, _V, ctypes.c_int, ctypes.c_int]
    L.wo_energy_x.argtypes = [_V, _V, _V, _V, _V]
    L.wo_energy_tblr.argtypes = [_V, _V, _V, _V, ctypes.c_int, ctypes.c_int, _V]
    _D = ctypes.c_double
    L.wo_add_circular_wave.argtypes = [_V, _D, _D, _D, _D, _D, _D, _V, _V]
    L.wo_frame_cells.argtypes = [_V, _V, _V, _V, ctypes.c_int, _V, _V, _V, _V]
    L.wo_energy_total_naive.restype = ctypes.c_double
    L.wo_energy_total_naive.argtypes = [_V, _V, _V, _V]
    L.wo_energy_total_comp.restype = ctypes.c_double
    L.wo_energy_total_comp.argtypes = [_V, _V, _V, _V]
    L.wo_mask.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                          _V, ctypes.c_int, _V]
    L.wo_init_ior.argtypes = [_V, _V, _V, _V, _V]
    L.wo_init_neumann.restype = ctypes.c_int
    L.wo_init_neumann.argtypes = [_V, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                  _V, _V, ctypes.c_int]


def _p(a):
    return None if a is None else a.ctypes.data


def _pp(params):
    return ctypes.cast(ctypes.byref(params), _V)


def _f64(a, n):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    assert a.size == n
    return a


def oscillating_bc(params, time, j):
    return lib().wo_oscillating_bc(_pp(params), int(time), int(j))


def evolve_wave_half(params, time, phi_in, psi_in, phi_out, xy, tcc, tc, tgamma, nbc=None):
    n = params.nx * params.ny
    assert phi_out.flags.c_contiguous and phi_out.dtype == np.float64
    nrec = 0 if nbc is None else len(nbc)
    lib().wo_evolve_wave_half(_pp(params), int(time), _p(_f64(phi_in, n)), _p(_f64(psi_in, n)),
                              _p(phi_out), _p(np.ascontiguousarray(xy, np.int16)),
                              _p(_f64(tcc, n)), _p(_f64(tc, n)), _p(_f64(tgamma, n)),
                              _p(nbc), nrec)


def run(params, phi, psi, tmp, xy, tcc, tc, tgamma, nsteps, time=0, nbc=None):
    """nsteps updates with evolve_wave's rotation.  Returns (newest, previous, third, time)."""
    n = params.nx * params.ny
    bufs = [np.array(_f64(b, n)) for b in (phi, psi, tmp)]
    arr = (_V * 3)(*[b.ctypes.data for b in bufs])
    t = ctypes.c_long(time)
    prev = ctypes.c_int(0)
    keep = [np.ascontiguousarray(xy, np.int16), _f64(tcc, n), _f64(tc, n), _f64(tgamma, n)]
    nrec = 0 if nbc is None else len(nbc)
    cur = lib().wo_run(_pp(params), ctypes.byref(t), int(nsteps), arr, *[_p(k) for k in keep],
                       _p(nbc), nrec, ctypes.byref(prev))
    third = 3 - cur - prev.value
    return bufs[cur], bufs[prev.value], bufs[third], t.value


def evolve_wave_half_energy(params, time, phi_in, psi_in, phi_out, xy):
    n = params.nx * params.ny
    lib().wo_evolve_wave_half_energy(_pp(params), int(time), _p(_f64(phi_in, n)), _p(_f64(psi_in, n)),
                                     _p(phi_out), _p(np.ascontiguousarray(xy, np.int16)))


def compute_energy(params, phi, psi, xy, i, j):
    n = params.nx * params.ny
    return lib().wo_compute_energy(_pp(params), _p(_f64(phi, n)), _p(_f64(psi, n)),
                                   _p(np.ascontiguousarray(xy, np.int16)), i, j)


def energy_x(params, phi, psi, xy):
    n = params.nx * params.ny
    out = np.zeros(params.nx)
    lib().wo_energy_x(_pp(params), _p(_f64(phi, n)), _p(_f64(psi, n)),
                      _p(np.ascontiguousarray(xy, np.int16)), _p(out))
    return out


def energy_tblr(params, phi, psi, xy, ileft, iright):
    n = params.nx * params.ny
    out = np.zeros(6)
    lib().wo_energy_tblr(_pp(params), _p(_f64(phi, n)), _p(_f64(psi, n)),
                         _p(np.ascontiguousarray(xy, np.int16)), ileft, iright, _p(out))
    return out


def add_circular_wave(params, init_amp, factor, x, y, variance, wavelength, phi, xy):
    """add_circular_wave (wave_common.c:337-351) on a copy of phi; returns the new phi."""
    n = params.nx * params.ny
    out = np.array(_f64(phi, n), dtype=np.float64, copy=True)
    lib().wo_add_circular_wave(_pp(params), init_amp, factor, x, y, variance, wavelength, _p(out),
                               _p(np.ascontiguousarray(xy, np.int16)))
    return out


def energy_total(params, phi, psi, xy, compensated=True):
    n = params.nx * params.ny
    f = lib().wo_energy_total_comp if compensated else lib().wo_energy_total_naive
    return f(_pp(params), _p(_f64(phi, n)), _p(_f64(psi, n)), _p(np.ascontiguousarray(xy, np.int16)))


def mask(params, domain, lam, npoly=6, apoly=0.0, circles=None):
    circ = np.zeros((0, 4))
    if circles is not None and len(circles):
        c = np.asarray(circles, dtype=np.float64)
        circ = np.zeros((len(c), 4))
        circ[:, :3] = c[:, :3]
    # wo_circle is {double xc, yc, radius; int active} -> 32 bytes
    rec = np.zeros(len(circ), dtype=np.dtype([("xc", "f8"), ("yc", "f8"), ("r", "f8"), ("active", "i4")], align=True))
    if len(circ):
        rec["xc"], rec["yc"], rec["r"], rec["active"] = circ[:, 0], circ[:, 1], circ[:, 2], 1
    out = np.zeros(params.nx * params.ny, dtype=np.int16)
    lib().wo_mask(_pp(params), int(domain), float(lam), int(npoly), float(apoly),
                  _p(rec) if len(rec) else None, len(rec), _p(out))
    return out


def init_ior(params, xy, tcc=None, tc=None, tgamma=None):
    n = params.nx * params.ny
    tcc = np.zeros(n) if tcc is None else np.array(tcc, dtype=np.float64)
    tc = np.zeros(n) if tc is None else np.array(tc, dtype=np.float64)
    tgamma = np.zeros(n) if tgamma is None else np.array(tgamma, dtype=np.float64)
    lib().wo_init_ior(_pp(params), _p(np.ascontiguousarray(xy, np.int16)), _p(tcc), _p(tc), _p(tgamma))
    return tcc, tc, tgamma


def init_neumann(params, domain, lam, xy, npoly=6, apoly=0.0, max_records=80000):
    from_params = __import__("importlib").import_module("youtube_simulations_gb300.params")
    recs = np.zeros(max_records, dtype=from_params.NEUMANN_DTYPE)
    xy = np.array(xy, dtype=np.int16)
    n = lib().wo_init_neumann(_pp(params), int(domain), float(lam), int(npoly), float(apoly),
                              _p(xy), _p(recs), max_records)
    if n < 0:
        raise OverflowError("too many Neumann points")
    return xy, recs[:n].copy()


def frame_cells(params, phi, psi, xy, size):
    """compute_energy and the compute_energy_flux velocity / gradients at the sampled
    cells, arrays [row = j/size][col = i/size] (wo_frame_cells)."""
    n = params.nx * params.ny
    w, h = params.nx // size, params.ny // size
    out = [np.zeros(w * h) for _ in range(4)]
    lib().wo_frame_cells(_pp(params), _p(_f64(phi, n)), _p(_f64(psi, n)), _p(np.ascontiguousarray(xy, np.int16)),
                         int(size), *[_p(a) for a in out])
    return [a.reshape(h, w) for a in out]


_PI, _PID, _DPI = 3.141592654, 1.570796327, 6.283185307  # global_pdes.c:8-10


def _argument(x, y):
    """argument() of sub_wave.c:287-302, elementwise."""
    safe = np.where(x != 0.0, x, 1.0)
    a = np.arctan(y / safe) + np.where(x < 0.0, _PI, 0.0)
    return np.where(x != 0.0, a, np.where(y < 0.0, _PI * 1.5, _PID))


def frame_rgb8(params, phi, xy, lut, size=2, vshift=-0.2, vscale=1.0, slope=1.0, color_range=0.8, scale=1.0,
               fade=False, fade_value=1.0, fade_in_obstacle=False, tcc=None, plot=0, psi=None, state=None,
               log_shift=0.75, log_scale=0.75, flux_scale=250.0, avrg_e_factor=0.95, attenuation=0.0, time=0):
    """draw_wave_highres_palette (wave_common.c:1750-1848) with wave_value (wave_common.c:
    1053-1162) for the C_ONEDIM scheme (colors_waves.c:3-22, 161-258; colormaps.c:
    2449-2482) and the palette `lut` (256x3 bytes): rows j/size from the bottom, columns
    i/size.  `state` (a dict) carries the running sums of the mean, average and
    total-flux modes from one frame to the next."""
    nx, ny = params.nx, params.ny
    phi2 = np.asarray(phi, np.float64).reshape(nx, ny)
    xy2 = np.asarray(xy).reshape(nx, ny)
    w, h = nx // size, ny // size
    ii = np.arange(w) * size
    jj = np.arange(h) * size
    v = phi2[np.ix_(ii, jj)].T                      # [row = j][col = i]
    m = xy2[np.ix_(ii, jj)].T != 0
    drawn = m | bool(params.twospeeds)
    state = {} if state is None else state
    asym, linear, dim = False, False, np.ones_like(v)
    if plot != 0:
        energy, vel, gx, gy = frame_cells(params, phi, psi, xy, size)
    if plot == 0:
        value = vshift + vscale * v
    elif plot == 1:
        value, asym = energy, True
    elif plot == 2:
        value = np.where((jj > ny // 2)[:, None], v, energy)
    elif plot == 3:
        acc = state.setdefault("acc", np.zeros((h, w)))
        acc += energy
        value, asym = acc / float(time + 1), True
    elif plot == 4:
        value = log_shift + log_scale * np.log(np.where(energy < 1.0e-20, 1.0e-20, energy))
    elif plot == 5:
        acc = state.setdefault("acc", np.zeros((h, w)))
        acc += np.where(energy == 0.0, 1.0e-20, energy)
        value = log_shift + log_scale * np.log(acc / float(time + 1))
    elif plot == 6:
        mod = np.where(drawn, vel * np.sqrt(gx * gx + gy * gy), 0.0)
        value, asym = mod * flux_scale, True
    elif plot == 7:
        tx = state.setdefault("fx", np.zeros((h, w)))
        ty = state.setdefault("fy", np.zeros((h, w)))
        tx[...] = tx * 0.99 + np.where(drawn, vel * gx, 0.0)
        ty[...] = ty * 0.99 + np.where(drawn, vel * gy, 0.0)
        mod = np.sqrt(tx * tx + ty * ty)
        arg = _argument(tx, ty)
        arg = np.where(arg < 0.0, arg + _DPI, arg)
        value, linear, dim = arg / _DPI, True, np.tanh(mod * flux_scale)
    else:
        acc = state.setdefault("acc", np.zeros((h, w)))
        acc[...] = avrg_e_factor * acc + (1.0 - avrg_e_factor) * energy
        if plot == 8:
            value, asym = acc.copy(), True
        else:
            with np.errstate(divide="ignore"):
                value = np.where(acc == 0.0, log_shift - 10.0 * log_scale, log_shift + log_scale * np.log(acc))
    if linear:
        hh = slope * value
        hh = np.where(hh > 1.0, hh - 1.0, np.where(hh < 0.0, hh + 1.0, hh))
    else:
        amp = color_range * np.tanh(slope * value / scale)
        if attenuation != 0.0:
            amp = amp * np.exp(-(float(time) * attenuation))
        hh = amp if asym else 0.5 * (1.0 + amp)
    hv = 256.0 * hh
    hue = np.trunc(np.clip(hv, 0.0, 255.0)).astype(np.int64)
    f = dim.copy()
    if fade_in_obstacle:
        c2 = params.courant * params.courant
        if tcc is None:
            cc = np.where(m, c2, params.courantb * params.courantb)
        else:
            cc = np.asarray(tcc, np.float64).reshape(nx, ny)[np.ix_(ii, jj)].T
        f = f * np.power(cc / c2, 0.1)
    if fade:
        f = f * fade_value
    lut = np.asarray(lut, np.uint8).reshape(256, 3).astype(np.float64)
    rgb = lut[hue] * f[..., None]
    out = np.clip((rgb + 0.5).astype(np.int64), 0, 255).astype(np.uint8)
    out[~drawn] = 0
    return out
