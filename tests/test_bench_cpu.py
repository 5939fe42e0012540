"""bench.py's host-side accounting on CPU: the active-cell count (the cells the bulk rule
updates, wave_billiard.c:365) and the active-cell rate beside the all-cell rate."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402
from youtube_simulations_gb300 import scenes  # noqa: E402


def test_active_cells_twospeeds_counts_every_cell():
    sc = scenes.config2(seed=0, nx=64, ny=48)
    assert sc.params.twospeeds == 1
    assert bench.active_cells(sc.params, sc.xy) == 64 * 48


def test_active_cells_counts_the_inside_of_the_mask():
    sc = scenes.batch_member(np.random.default_rng(7), smin=(40, 40), smax=(80, 60))
    assert sc.params.twospeeds == 0
    n = bench.active_cells(sc.params, sc.xy)
    assert n == int(np.count_nonzero(sc.xy > 0))
    assert 0 < n < sc.params.nx * sc.params.ny


def test_active_rate_scales_the_all_cell_rate():
    res = bench.with_active_rate({"value": 100.0}, active=300, cells=400)
    assert res["active_cell_rate"] == 75.0 and res["value"] == 100.0


class FakeServer:
    """Host-only stand-in for W.Server: a request needs `frames` ticks once submitted."""

    def __init__(self):
        self.left, self.submit_times, self.t0, self.done = [], [], None, 0

    def submit(self, params, phi, psi, xy, frames):
        import time
        self.submit_times.append(time.perf_counter())
        self.left.append(frames)

    def stats(self):
        return {"resident": sum(1 for f in self.left if f > 0), "queued": 0, "completed": self.done,
                "cancelled": 0}

    def tick(self):
        for k, f in enumerate(self.left):
            if f > 0:
                self.left[k] = f - 1
                if f == 1:
                    self.done += 1
        return 0

    def drain(self):
        return 0


def test_serve_stream_submits_on_the_wall_clock():
    import time

    class M:
        params = phi = psi = xy = None
    reqs = [(M(), 3), (M(), 1), (M(), 2)]
    arrivals = np.array([0.0, 0.05, 0.12])
    srv = FakeServer()
    t0 = time.perf_counter()
    wall, max_q, max_res = bench.serve_stream(None, srv, reqs, arrivals)
    assert srv.done == 3 and len(srv.submit_times) == 3
    for t, a in zip(srv.submit_times, arrivals):
        assert t - t0 >= a - 1e-3  # never submitted before its arrival time
    assert wall >= 0.12 and max_q == 0 and max_res >= 1


def test_clock_summary_decodes_the_event_reasons():
    """NVML clock-event reason bits (sw power cap 0x4, hw slowdown 0x8, sw thermal 0x20, hw
    thermal 0x40) become the names the bench line reports; the clock is the median sample."""
    rows = [(2070.0, 0x0), (2070.0, 0x4), (1995.0, 0x4 | 0x8), (2070.0, 0x1)]
    out = bench.NvmlClocks.summary(rows, 2070.0)
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 4
    assert out["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert bench.NvmlClocks.summary([(1500.0, 0x40 | 0x20)], 2070.0)["reasons"] == ["hw_thermal_slowdown",
                                                                                   "sw_thermal_slowdown"]
    assert bench.NvmlClocks.summary([], 2070.0)["reasons"] == ["no samples"]


def test_clock_sampler_falls_back_without_nvml():
    """Where NVML cannot be loaded (this host has no GPU driver), the nvidia-smi sampler is used."""
    s = bench.clock_sampler(0)
    assert isinstance(s, (bench.Clocks, bench.NvmlClocks))
