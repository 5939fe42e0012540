"""GB300 (sm_103a) implementation of wave_billiard's leapfrog stepper and
wave_energy's energy diagnostics (nilsberglund-orleans/YouTube-simulations).

The compute path is libwavegpu.so (CUDA C++ behind the C ABI of include/wavegpu.h);
this package holds its build script, a ctypes binding that mirrors the reference's
function surface, and the host-side scene setup.
"""
from . import params  # noqa: F401
