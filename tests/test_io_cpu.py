"""Frame files and time-series lines, on the CPU: wg_write_tiff against writetiff's
layout (sub_wave.c:62-122: baseline TIFF, 8-bit RGB, uncompressed, one row per strip,
ORIENTATION_BOTLEFT, scanline s = frame row height-1-s), wg_write_ppm, and the
SAVE_TIME_SERIES line format of wave_billiard.c:900-908 ("%019ld" of (long)(phi*1e16))."""
import struct

import numpy as np
import pytest

from youtube_simulations_gb300 import wavegpu as W


def parse_tiff(data):
    assert data[:4] == b"II*\x00"
    ifd = struct.unpack_from("<I", data, 4)[0]
    n = struct.unpack_from("<H", data, ifd)[0]
    tags = {}
    for k in range(n):
        tid, typ, cnt, val = struct.unpack_from("<HHII", data, ifd + 2 + 12 * k)
        if typ == 3 and cnt == 1:
            val &= 0xFFFF
        tags[tid] = (typ, cnt, val)
    assert struct.unpack_from("<I", data, ifd + 2 + 12 * n)[0] == 0
    return tags


@pytest.mark.parametrize("w,h", [(33, 22), (5, 1), (1, 7)])
def test_tiff_layout(tmp_path, w, h):
    rgb = np.random.default_rng(w * h).integers(0, 256, size=(h, w, 3), dtype=np.uint8)
    path = tmp_path / "frame.tif"
    W.write_tiff(path, rgb, description="wave billiard frame")
    data = path.read_bytes()
    t = parse_tiff(data)
    ids = list(t)
    assert ids == sorted(ids)
    assert t[256][2] == w and t[257][2] == h
    bps = struct.unpack_from("<3H", data, t[258][2])
    assert bps == (8, 8, 8)
    assert t[259][2] == 1 and t[262][2] == 2 and t[274][2] == 4 and t[277][2] == 3 and t[278][2] == 1
    assert t[284][2] == 1
    typ, cnt, off = t[270]
    assert data[off:off + cnt] == b"wave billiard frame\x00"
    offs = [t[273][2]] if h == 1 else list(struct.unpack_from("<%dI" % h, data, t[273][2]))
    cnts = [t[279][2]] if h == 1 else list(struct.unpack_from("<%dI" % h, data, t[279][2]))
    assert cnts == [3 * w] * h
    for s in range(h):
        line = np.frombuffer(data, np.uint8, 3 * w, offs[s]).reshape(w, 3)
        assert np.array_equal(line, rgb[h - 1 - s])


def test_ppm(tmp_path):
    rgb = np.random.default_rng(3).integers(0, 256, size=(4, 6, 3), dtype=np.uint8)
    path = tmp_path / "frame.ppm"
    W.write_ppm(path, rgb)
    data = path.read_bytes()
    head = b"P6\n6 4\n255\n"
    assert data[:len(head)] == head
    img = np.frombuffer(data, np.uint8, offset=len(head)).reshape(4, 6, 3)
    assert np.array_equal(img, rgb[::-1])


def test_time_series_lines(tmp_path):
    path = tmp_path / "series.txt"
    W.write_time_series(path, [1.234e-3, -5e-16, 0.0, -2.5e-2])
    assert path.read_text().split("\n")[:4] == ["0000012340000000000", "-000000000000000005",
                                                "0000000000000000000", "-000250000000000000"]
