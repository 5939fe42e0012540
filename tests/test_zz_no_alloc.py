"""wg_compute_energy_device_noalloc: the energy diagnostics for callers that cannot
allocate device memory when they need them (their device memory belongs to their own
arena, or they must not call cudaMalloc while serving).  The entry point takes fields
and output in the caller's device memory and keeps its per-column partial sums in a
fixed array inside the library.

Checked through the C ABI on two calls in a row (different fields each time) against
the existing entry points on the same data: the total against an FP64 scene's
wg_scene_energy, the six boxes against wg_compute_energy_tblr, the columns against
wg_compute_energy_x_all, all within 1e-12 relative.  The device buffers here are
allocated by the test (torch), not by the entry point, and the device's free memory is
the same before and after the calls: the entry point itself allocates nothing.  This
file is collected last."""
import ctypes

import numpy as np
import pytest

from helpers import variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


def existing(p, phi, psi, xy, ileft, iright):
    """Total, boxes and columns from the existing entry points."""
    with W.Scene(p, P.FP64, P.COEF_TABLE) as s:
        s.upload(phi, psi, xy, np.zeros_like(phi), np.zeros_like(phi), np.zeros_like(phi))
        total = s.total_energy()
    W.configure(p)
    rf = W.RowFields(p, phi, psi, np.zeros_like(phi), xy)
    return total, W.compute_energy_tblr(rf, ileft, iright), W.compute_energy_x(rf)


def close(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) <= TOL * max(np.max(np.abs(b)), 1e-300)


def test_noalloc_energy_matches_existing_entry_points_twice():
    torch = pytest.importorskip("torch")
    p, f, xy, _ = variant_inputs("s_abs", seed=12)
    nx, ny = p.nx, p.ny
    pitch = ny + 5  # a caller's own row pitch
    dev = torch.device("cuda", 0)
    d_phi = torch.zeros((nx, pitch), dtype=torch.float64, device=dev)
    d_psi = torch.zeros((nx, pitch), dtype=torch.float64, device=dev)
    d_xy = torch.zeros((nx, pitch), dtype=torch.int16, device=dev)
    d_out = torch.full((nx + 7,), float("nan"), dtype=torch.float64, device=dev)
    d_xy[:, :ny] = torch.from_numpy(xy.reshape(nx, ny)).to(dev)
    ileft, iright = nx // 5, (4 * nx) // 5
    L = W.lib()

    def call_noalloc():
        W.check(L.wg_compute_energy_device_noalloc(ctypes.byref(p), d_phi.data_ptr(), d_psi.data_ptr(),
                                                   d_xy.data_ptr(), pitch, ileft, iright, d_out.data_ptr(), None))

    # the first call in a process may load the library's device module (lazy loading);
    # after it, further calls leave the device's free memory exactly as it was
    call_noalloc()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(dev)[0]
    for _ in range(3):
        call_noalloc()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free_before
    for call, scale in enumerate((1.0, -2.5)):
        phi = f["phi"] * scale
        psi = f["psi"] * scale + 0.01 * call
        d_phi[:, :ny] = torch.from_numpy(phi.reshape(nx, ny)).to(dev)
        d_psi[:, :ny] = torch.from_numpy(psi.reshape(nx, ny)).to(dev)
        torch.cuda.synchronize()
        call_noalloc()
        torch.cuda.synchronize()
        out = d_out.cpu().numpy()
        total, boxes, cols = existing(p, phi, psi, xy, ileft, iright)
        assert close([out[0]], [total]), call
        assert close(out[1:7], boxes), call
        assert close(out[7:], cols), call


def test_noalloc_refuses_more_columns_than_its_scratch():
    torch = pytest.importorskip("torch")
    p = P.make_params(16385, 4)
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = W.lib().wg_compute_energy_device_noalloc(ctypes.byref(p), d.data_ptr(), d.data_ptr(), d.data_ptr(), 4,
                                                  0, 0, d.data_ptr(), None)
    assert st == -1
    assert b"16384" in W.lib().wg_last_error()
