"""CPU-side checks of the C ABI: the library builds for sm_103a, loads without a GPU
and exports every function include/*.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(wg_[a-z_0-9]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "wg_evolve_wave" in names and "wg_scene_step" in names and len(names) > 30


def test_library_exports_every_declared_symbol():
    from youtube_simulations_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_status_strings_without_gpu():
    from youtube_simulations_gb300 import wavegpu as W
    L = W.lib()
    assert L.wg_abi_version() == 3
    assert L.wg_status_string(-4) == b"HBM budget exceeded"
