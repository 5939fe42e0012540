"""Drop-in surface on the GPU against the oracle: evolve_wave / evolve_wave_half
(wave_billiard.c:302-631) through the C ABI, FP64, bit for bit, for every boundary
rule, oscillation schedule, Neumann gather, FLOOR clamp and the point source.
The tolerance is zero except where a transcendental source (cos/exp/sin of
oscillating_bc or the point source) enters: CUDA's and glibc's last bits may differ
there, and the bar is 1e-12 relative to the field maximum."""
import numpy as np
import pytest

import oracle
import ref_variants
from helpers import params_of, rel_err, variant_inputs
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu

STEP_VARIANTS = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "wb_fn" and not v.get("dropin")]
ENERGY_VARIANTS = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "we_fn"]
TOL = 1e-12


def transcendental(p):
    return bool(p.oscillate_left or p.src_on)


def check_close(a, b, p):
    if transcendental(p):
        assert rel_err(a, b) <= TOL
    else:
        assert np.array_equal(a, b)


@pytest.mark.parametrize("variant", STEP_VARIANTS)
@pytest.mark.parametrize("resident", [False, True])
def test_evolve_wave_matches_oracle(variant, resident):
    p, f, xy, nbc = variant_inputs(variant, seed=7)
    nsteps = 30
    new, prev, third, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"],
                                     nsteps, nbc=nbc)
    W.configure(p)
    W.set_mode(resident)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    for _ in range(nsteps // 3):
        W.evolve_wave(rf, nbc=nbc)
    if resident:
        W.sync()
    check_close(rf.phi.reshape(-1), new, p)
    check_close(rf.psi.reshape(-1), prev, p)
    check_close(rf.tmp.reshape(-1), third, p)
    assert W.dropin_time() == nsteps
    W.set_mode(False)


@pytest.mark.parametrize("variant", ["s_dir", "s_vph", "s_neu_ts", "s_tiny"])
def test_evolve_wave_half_rotation(variant):
    """Single updates with the caller's own rotation, 7 updates (not a multiple of 3)."""
    p, f, xy, nbc = variant_inputs(variant, seed=11)
    new, prev, third, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], 7, nbc=nbc)
    W.configure(p)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    names = ["phi", "psi", "tmp"]
    cur, prv, fre = 0, 1, 2
    for _ in range(7):
        W.evolve_wave_half(rf, names[cur], names[prv], names[fre], nbc=nbc)
        cur, prv, fre = fre, cur, prv
    check_close(getattr(rf, names[cur]).reshape(-1), new, p)
    check_close(getattr(rf, names[prv]).reshape(-1), prev, p)


def test_point_source_dropin():
    p, f, xy, _ = variant_inputs("s_abs", seed=3)
    inside = np.argwhere(xy.reshape(p.nx, p.ny) > 0)[7]
    p.src_on, p.src_i, p.src_j, p.src_amp, p.src_period = 1, int(inside[0]), int(inside[1]), 0.05, 23.7
    new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], 42)
    W.configure(p)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    for _ in range(14):
        W.evolve_wave(rf)
    assert rel_err(rf.phi.reshape(-1), new) <= TOL
    assert rel_err(rf.psi.reshape(-1), prev) <= TOL


@pytest.mark.parametrize("variant", ENERGY_VARIANTS)
def test_wave_energy_stepper_matches_oracle(variant):
    p, f, xy, _ = variant_inputs(variant, seed=5)
    bufs = [f["phi"].copy(), f["psi"].copy(), f["tmp"].copy()]
    cur, prv, fre = 0, 1, 2
    for s in range(1, 31):
        oracle.evolve_wave_half_energy(p, s, bufs[cur], bufs[prv], bufs[fre], xy)
        cur, prv, fre = fre, cur, prv
    W.configure(p)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy)
    for _ in range(10):
        W.evolve_wave_energy(rf)
    check_close(rf.phi.reshape(-1), bufs[cur], p)
    check_close(rf.psi.reshape(-1), bufs[prv], p)
    check_close(rf.tmp.reshape(-1), bufs[fre], p)


@pytest.mark.parametrize("variant", ["e_dir", "e_per_osc", "s_abs"])
def test_energy_diagnostics(variant):
    p, f, xy, _ = variant_inputs(variant, seed=2)
    W.configure(p)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy)
    ex = W.compute_energy_x(rf)
    ref_x = oracle.energy_x(p, f["phi"], f["psi"], xy)
    assert np.max(np.abs(ex - ref_x)) <= 1e-12 * np.max(np.abs(ref_x))
    ileft, iright = p.nx // 4, (3 * p.nx) // 4
    tb = W.compute_energy_tblr(rf, ileft, iright)
    ref_tb = oracle.energy_tblr(p, f["phi"], f["psi"], xy, ileft, iright)
    assert np.max(np.abs(tb - ref_tb)) <= 1e-12 * np.max(np.abs(ref_tb))
    for (i, j) in [(0, 0), (p.nx - 1, p.ny - 1), (p.nx // 2, p.ny // 3), (1, p.ny - 1)]:
        assert W.compute_energy(rf, i, j) == oracle.compute_energy(p, f["phi"], f["psi"], xy, i, j)


def test_bad_records_rejected():
    p, f, xy, nbc = variant_inputs("s_neu", seed=1)
    bad = nbc.copy()
    bad["i"][0] = 0     # a boundary-line cell: outside what init_neumann_bc produces
    W.configure(p)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    with pytest.raises(W.WaveGpuError):
        W.evolve_wave(rf, nbc=bad)


class _ScatteredRows:
    """Row arrays whose rows are separate allocations starting 8 bytes past a 16-byte
    boundary (as rows from a general allocator may), for the row transfers' element path."""

    def __init__(self, rf):
        import ctypes
        self.rf = rf
        self._keep, self._r = [], {}
        for name in ("phi", "psi", "tmp", "xy", "tcc", "tc", "tgamma"):
            a = getattr(rf, name)
            rows = []
            for i in range(a.shape[0]):
                buf = np.zeros(a.shape[1] + 16, a.dtype)
                k = next(k for k in range(16) if (buf.ctypes.data + k * a.itemsize) % 16 == 8)
                v = buf[k:k + a.shape[1]]
                v[:] = a[i]
                rows.append(v)
            self._keep.append(rows)
            ptrs = (ctypes.c_void_p * len(rows))(*[r.ctypes.data for r in rows])
            self._r[name] = (ctypes.cast(ptrs, W._PP), ptrs, rows)

    def rows(self, name):
        return self._r[name][0]

    def field(self, name):
        return np.stack(self._r[name][2]).reshape(-1)


@pytest.mark.parametrize("rows_mode", [0, 1])  # WG_ROWS_AUTO (in place where the device can), WG_ROWS_PACKED
@pytest.mark.parametrize("variant,scattered", [("s_square", False), ("s_square", True), ("s_dir", True)])
def test_row_transfers(rows_mode, variant, scattered):
    """Strict evolve_wave with the rows moved in place by the device or packed by host
    threads: the oracle's fields either way, for rows of one buffer and for rows in separate
    allocations 8 bytes off a 16-byte boundary (even NY, and odd NY = 45)."""
    p, f, xy, nbc = variant_inputs(variant, seed=13)
    new, prev, third, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], 9, nbc=nbc)
    W.configure(p)
    W.set_mode(False)
    W.check(W.lib().wg_dropin_set_rows(rows_mode))
    try:
        rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
        target = _ScatteredRows(rf) if scattered else rf
        for _ in range(3):
            W.evolve_wave(target, nbc=nbc)
        get = (lambda n: target.field(n)) if scattered else (lambda n: getattr(rf, n).reshape(-1))
        check_close(get("phi"), new, p)
        check_close(get("psi"), prev, p)
        check_close(get("tmp"), third, p)
    finally:
        W.check(W.lib().wg_dropin_set_rows(0))
