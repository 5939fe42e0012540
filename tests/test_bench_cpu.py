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
