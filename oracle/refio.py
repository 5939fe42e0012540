"""Runs the compiled reference (oracle/_ref/bin/ref_<variant>).  TEST INFRASTRUCTURE.

File layout read by oracle/ref_driver.c:
  int64[16]  magic 0x57415645, nx, ny, mode, nsteps, n_nbc, ncircles, ileft, iright,
             src_on, src_i, src_j, n_times, segments (TIME), report interval (STEP), 0
  double[4]  src_amp, src_period, 0, 0 (PULSE: factor, 0, x, y)
  double[3*ncircles] circles (xc, yc, r)
  mode OSC : int32[n_times]
  else     : double phi, psi, tmp, tcc, tc, tgamma [nx*ny each]; int16 xy [nx*ny];
             t_neumann_bc[n_nbc]
Output (non-OSC): the six arrays, xy, int64 n_nbc + records, energy total,
energy_x[nx], tblr[6], elapsed seconds, int64 threads, int64 n_reports + the total
energy after every `report` updates (STEP with report > 0).
"""
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BIN = HERE / "_ref" / "bin"
STEP, SETUP, TIME, OSC, PULSE, FRAME = 0, 1, 2, 3, 4, 5


def available(variant):
    return (BIN / f"ref_{variant}").exists()


def _neumann_dtype():
    import importlib
    return importlib.import_module("youtube_simulations_gb300.params").NEUMANN_DTYPE


def run(variant, nx, ny, mode=STEP, nsteps=0, fields=None, xy=None, nbc=None, circles=None,
        src=None, times=None, threads=None, timeout=600, pulse=None, report=0):
    circles = np.zeros((0, 3)) if circles is None else np.asarray(circles, np.float64)[:, :3]
    n_nbc = 0 if nbc is None else len(nbc)
    hdr = np.zeros(16, np.int64)
    hdr[:7] = [0x57415645, nx, ny, mode, nsteps, n_nbc, len(circles)]
    hd = np.zeros(4)
    if src is not None:
        hdr[9:12] = [1, src[0], src[1]]
        hd[0], hd[1] = src[2], src[3]
    if times is not None:
        hdr[12] = len(times)
    if pulse is not None:  # PULSE: (factor, x, y) of add_circular_wave
        hd[0], hd[2], hd[3] = pulse
    hdr[14] = int(report)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(hdr.tobytes())
            f.write(hd.tobytes())
            f.write(np.ascontiguousarray(circles).tobytes())
            if mode == OSC:
                f.write(np.asarray(times, np.int32).tobytes())
            else:
                n = nx * ny
                names = ["phi", "psi", "tmp", "tcc", "tc", "tgamma"]
                for k in names:
                    a = np.zeros(n) if fields is None or fields.get(k) is None else fields[k]
                    f.write(np.ascontiguousarray(a, np.float64).reshape(-1).tobytes())
                a = np.zeros(n, np.int16) if xy is None else xy
                f.write(np.ascontiguousarray(a, np.int16).reshape(-1).tobytes())
                if n_nbc:
                    f.write(np.ascontiguousarray(nbc).tobytes())
        env = dict(os.environ)
        if threads is not None:
            env["OMP_NUM_THREADS"] = str(threads)
        r = subprocess.run([str(BIN / f"ref_{variant}"), str(fin), str(fout)],
                           capture_output=True, text=True, env=env, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_{variant} failed ({r.returncode}): {r.stderr[-1000:]}")
        raw = fout.read_bytes()
    if mode == OSC:
        return np.frombuffer(raw, np.float64).reshape(len(times), ny)
    n = nx * ny
    off = 0
    out = {}
    for k in ["phi", "psi", "tmp", "tcc", "tc", "tgamma"]:
        out[k] = np.frombuffer(raw, np.float64, n, off).copy()
        off += 8 * n
    out["xy"] = np.frombuffer(raw, np.int16, n, off).copy()
    off += 2 * n
    nrec = int(np.frombuffer(raw, np.int64, 1, off)[0])
    off += 8
    dt = _neumann_dtype()
    out["nbc"] = np.frombuffer(raw, dt, nrec, off).copy()
    off += dt.itemsize * nrec
    out["energy"] = float(np.frombuffer(raw, np.float64, 1, off)[0])
    off += 8
    out["energy_x"] = np.frombuffer(raw, np.float64, nx, off).copy()
    off += 8 * nx
    out["tblr"] = np.frombuffer(raw, np.float64, 6, off).copy()
    off += 48
    out["elapsed"] = float(np.frombuffer(raw, np.float64, 1, off)[0])
    off += 8
    out["threads"] = int(np.frombuffer(raw, np.int64, 1, off)[0])
    off += 8
    nrep = int(np.frombuffer(raw, np.int64, 1, off)[0])
    off += 8
    out["reports"] = np.frombuffer(raw, np.float64, nrep, off).copy()
    return out


def frame(variant, nx, ny, phi, psi, xy, tcc, plot, size=2, frames=1, t0=0, scale=1.0, timeout=600):
    """FRAME mode: the reference's wave_value colours (palette COL_TURBO) of the cells
    draw_wave_highres_palette samples, after `frames` frames at times t0, t0+1, ...
    Returns (rgb [ny/size][nx/size][3] doubles, values [ny/size][nx/size], fade factors
    of init_fade_table at the same cells)."""
    hdr = np.zeros(16, np.int64)
    hdr[:7] = [0x57415645, nx, ny, FRAME, 0, 0, 0]
    hdr[7], hdr[8], hdr[12], hdr[13] = size, t0, plot, frames
    hd = np.zeros(4)
    hd[0] = scale
    n = nx * ny
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(hdr.tobytes())
            f.write(hd.tobytes())
            for a in (phi, psi, np.zeros(n), tcc, np.zeros(n), np.zeros(n)):
                f.write(np.ascontiguousarray(a, np.float64).reshape(-1).tobytes())
            f.write(np.ascontiguousarray(xy, np.int16).reshape(-1).tobytes())
        r = subprocess.run([str(BIN / f"ref_{variant}"), str(fin), str(fout)], capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_{variant} failed ({r.returncode}): {r.stderr[-1000:]}")
        raw = fout.read_bytes()
    w, h = nx // size, ny // size
    rgb = np.frombuffer(raw, np.float64, 3 * w * h, 0).reshape(h, w, 3).copy()
    vals = np.frombuffer(raw, np.float64, w * h, 24 * w * h).reshape(h, w).copy()
    fade = np.frombuffer(raw, np.float64, w * h, 32 * w * h).reshape(h, w).copy()
    return rgb, vals, fade


def time_reference(variant, nx, ny, nsteps, circles, centre, src=None, threads=None, timeout=900, segments=1):
    """TIME mode: the reference builds its own inputs (init_wave_flat, init_ior_2d,
    add_circular_wave) once and times `segments` runs of `nsteps` updates each.
    Returns (seconds, energy, threads), or with segments > 1 (per-segment seconds,
    energy, threads)."""
    circles = np.asarray(circles, np.float64)[:, :3]
    hdr = np.zeros(16, np.int64)
    hdr[:7] = [0x57415645, nx, ny, TIME, nsteps, 0, len(circles)]
    hdr[13] = segments
    hd = np.zeros(4)
    hd[2], hd[3] = centre
    if src is not None:
        hdr[9:12] = [1, src[0], src[1]]
        hd[0], hd[1] = src[2], src[3]
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(hdr.tobytes())
            f.write(hd.tobytes())
            f.write(np.ascontiguousarray(circles).tobytes())
        env = dict(os.environ)
        if threads is not None:
            env["OMP_NUM_THREADS"] = str(threads)
        r = subprocess.run([str(BIN / f"ref_{variant}"), str(fin), str(fout)],
                           capture_output=True, text=True, env=env, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_{variant} failed ({r.returncode}): {r.stderr[-1000:]}")
        raw = fout.read_bytes()
    el, e = np.frombuffer(raw, np.float64, 2, 0)
    th = int(np.frombuffer(raw, np.int64, 1, 16)[0])
    if segments > 1:
        return np.frombuffer(raw, np.float64, segments, 24).tolist(), float(e), th
    return float(el), float(e), th
