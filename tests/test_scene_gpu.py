"""Native scenes (wg_scene_*) on the GPU against the oracle.

FP64 scenes run the reference's operation order and must match the oracle's values
(1e-12 relative where oscillating_bc or the point source brings cos/exp/sin); a term
left out for KAPPA = 0 or GAMMA = 0 may change only the sign of a zero result, and
test_fp64_bits_gpu.py compares the bits with every term present.
FP32 scenes are held to a field error <= 1e-5 relative to the field maximum and an
energy difference <= 1e-5 relative after the run."""
import numpy as np
import pytest

import oracle
import ref_variants
from helpers import equalize_unwritten, rel_err, variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu
STEP_VARIANTS = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "wb_fn" and not v.get("dropin")]


def run_oracle(p, f, xy, nsteps, nbc=None):
    new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], nsteps, nbc=nbc)
    return new, prev


def close(a, b, p, tol=1e-12):
    if p.oscillate_left or p.src_on:
        assert rel_err(a, b) <= tol
    else:
        assert np.array_equal(a, b)


@pytest.mark.parametrize("variant", STEP_VARIANTS)
def test_fp64_table_scene(variant):
    p, f, xy, nbc = variant_inputs(variant, seed=21)
    f = equalize_unwritten(p, f, xy, nbc)
    new, prev = run_oracle(p, f, xy, 23, nbc)
    with W.Scene(p, P.FP64, P.COEF_TABLE) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        if nbc is not None:
            s.set_neumann(nbc)
        s.step(23)
        phi, psi = s.download()
        assert s.time == 23
    close(phi, new, p)
    close(psi, prev, p)


@pytest.mark.parametrize("variant", [v for v in STEP_VARIANTS if not ref_variants.VARIANTS[v]["macros"]["BC_NEUMANN"]])
def test_fp64_mask_scene(variant):
    p, f, xy, _ = variant_inputs(variant, seed=22)
    tcc, tc, tg = scenes.tables(p, xy)
    f = dict(f, tcc=tcc, tc=tc, tgamma=tg)
    f = equalize_unwritten(p, f, xy)
    new, prev = run_oracle(p, f, xy, 31)
    with W.Scene(p, P.FP64, P.COEF_MASK) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy)
        s.step(31)
        phi, psi = s.download()
    close(phi, new, p)
    close(psi, prev, p)


@pytest.mark.parametrize("variant", ["s_dir", "s_per", "s_abs", "s_vph", "s_topbot", "s_neu"])
@pytest.mark.parametrize("coef", [P.COEF_MASK, P.COEF_TABLE])
def test_fp32_scene_tolerance(variant, coef):
    p, f, xy, nbc = variant_inputs(variant, seed=23, smooth=True)
    if coef == P.COEF_MASK and nbc is not None:
        pytest.skip("Neumann ghosts need tables")
    if coef == P.COEF_MASK:
        tcc, tc, tg = scenes.tables(p, xy)
        f = dict(f, tcc=tcc, tc=tc, tgamma=tg)
    f = equalize_unwritten(p, f, xy, nbc)
    new, prev = run_oracle(p, f, xy, 60, nbc)
    with W.Scene(p, P.FP32, coef) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        if nbc is not None:
            s.set_neumann(nbc)
        s.step(60)
        phi, psi = s.download()
        e32 = s.total_energy()
    assert rel_err(phi, new) <= 1e-5
    assert rel_err(psi, prev) <= 1e-5
    e64 = oracle.energy_total(p, new, prev, xy)
    assert abs(e32 - e64) <= 1e-5 * abs(e64)


@pytest.mark.parametrize("prec", [P.FP64, P.FP32])
def test_scene_energy_matches_oracle(prec):
    p, f, xy, _ = variant_inputs("s_abs", seed=4)
    with W.Scene(p, prec, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        total, cols, boxes = s.energy(ileft=10, iright=50)
        phi, psi = s.download()
    # the oracle on the values the scene holds (FP32-rounded for an FP32 scene); an FP32
    # scene evaluates each cell's energy in FP32 (sums in FP64), hence 1e-6 there
    tol_t, tol_c = (1e-13, 1e-12) if prec == P.FP64 else (1e-6, 1e-6)
    ref_total = oracle.energy_total(p, phi, psi, xy, compensated=True)
    assert abs(total - ref_total) <= tol_t * abs(ref_total)
    ref_cols = oracle.energy_x(p, phi, psi, xy)
    assert np.max(np.abs(cols - ref_cols)) <= tol_c * np.max(np.abs(ref_cols))
    ref_boxes = oracle.energy_tblr(p, phi, psi, xy, 10, 50)
    assert np.max(np.abs(boxes - ref_boxes)) <= tol_c * np.max(np.abs(ref_boxes))


def test_state_roundtrip_and_time():
    """An FP32 scene stores phi and the velocity v = phi - psi (each rounded once from the
    FP64 difference); psi comes back as phi - v, within an FP32 rounding of |v| of the
    uploaded psi, and phi exactly."""
    p, f, xy, _ = variant_inputs("s_per", seed=9)
    with W.Scene(p, P.FP32, P.COEF_MASK) as s:
        s.upload(f["phi"], f["psi"], xy)
        a = np.random.default_rng(0).standard_normal(p.nx * p.ny).astype(np.float32)
        b = np.random.default_rng(1).standard_normal(p.nx * p.ny).astype(np.float32)
        s.upload_state(a, b)
        x, y = s.download(native=True)
        v = (a.astype(np.float64) - b.astype(np.float64)).astype(np.float32)
        assert np.array_equal(x, a)
        assert np.array_equal(y, (a.astype(np.float64) - v.astype(np.float64)).astype(np.float32))
        assert np.max(np.abs(y.astype(np.float64) - b)) <= 2 * np.finfo(np.float32).eps * np.max(np.abs(v))
        x64, y64 = s.download()
        assert np.array_equal(x64, a.astype(np.float64))
        assert np.array_equal(y64, a.astype(np.float64) - v.astype(np.float64))
        s.time = 100
        s.step(3)
        assert s.time == 103


def _special_pairs(n, seed):
    """FP32 (phi, psi) rows: normals, then signed zeros, subnormals, differences that
    overflow FP32 and exponent gaps wider than FP32 can hold in one difference."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(n).astype(np.float32)
    b = rng.standard_normal(n).astype(np.float32)
    tiny = np.float32(1.4e-45)
    sa = np.array([0.0, -0.0, 0.0, -0.0, tiny, -tiny, 3 * tiny, 1.2e-38, 3.0e38, -3.0e38, 1.0e30, 1.0e-30,
                   1.0, 16777217.0, 1.0e8], np.float32)
    sb = np.array([0.0, 0.0, -0.0, -0.0, tiny, 2 * tiny, -tiny, 1.1e-38, -3.0e38, 3.0e38, 1.0e-30, 1.0e30,
                   5.9604645e-08, 1.0, -3.0e-8], np.float32)
    a[:len(sa)] = sa
    b[:len(sb)] = sb
    return a, b


def test_state_special_values():
    """The velocity phi - psi and psi = phi - v are formed by the FP32 subtraction for FP32
    host rows; they must equal the FP64 difference rounded once to FP32, bit for bit, on
    signed zeros, subnormals, overflow and wide exponent gaps."""
    p, f, xy, _ = variant_inputs("s_per", seed=9)
    n = p.nx * p.ny
    a, b = _special_pairs(n, 3)
    with W.Scene(p, P.FP32, P.COEF_MASK) as s:
        s.upload(f["phi"], f["psi"], xy)
        s.upload_state(a, b)
        x, y = s.download(native=True)
        with np.errstate(over="ignore"):
            v = (a.astype(np.float64) - b.astype(np.float64)).astype(np.float32)
            want = (a.astype(np.float64) - v.astype(np.float64)).astype(np.float32)
        assert np.array_equal(x.view(np.uint32), a.view(np.uint32))
        assert np.array_equal(y.view(np.uint32), want.view(np.uint32))


def test_state_in_place_page_locked():
    """Page-locked host rows are read and written by the device in place (no staging copy):
    the same bits as pageable rows, from and to FP32 and FP64 host arrays."""
    torch = pytest.importorskip("torch")
    p, f, xy, _ = variant_inputs("s_per", seed=9)
    n = p.nx * p.ny
    a32, b32 = _special_pairs(n, 4)
    lib = W.lib()
    with W.Scene(p, P.FP32, P.COEF_MASK) as s:
        s.upload(f["phi"], f["psi"], xy)
        for prec, dt in ((P.FP32, np.float32), (P.FP64, np.float64)):
            a, b = a32.astype(dt), b32.astype(dt)
            if dt == np.float64:
                a[len(a) // 2:] += 1e-12 * b[len(a) // 2:]  # values FP32 cannot hold
            W.check(lib.wg_scene_upload_state(s.h, a.ctypes.data, b.ctypes.data, prec))
            W.check(lib.wg_scene_sync(s.h))
            x0, y0 = np.empty(n, dt), np.empty(n, dt)
            W.check(lib.wg_scene_download(s.h, x0.ctypes.data, y0.ctypes.data, prec))
            ha, hb = torch.from_numpy(a).pin_memory(), torch.from_numpy(b).pin_memory()
            hx, hy = torch.empty(n, dtype=ha.dtype).pin_memory(), torch.empty(n, dtype=ha.dtype).pin_memory()
            W.check(lib.wg_scene_upload_state(s.h, ha.data_ptr(), hb.data_ptr(), prec))
            W.check(lib.wg_scene_download(s.h, hx.data_ptr(), hy.data_ptr(), prec))
            x1, y1 = hx.numpy(), hy.numpy()
            assert np.array_equal(x0.view(np.uint8), x1.view(np.uint8))
            assert np.array_equal(y0.view(np.uint8), y1.view(np.uint8))
            # phi alone, into a view that starts 4 elements into its page-locked allocation
            big = torch.zeros(n + 4, dtype=ha.dtype).pin_memory()
            W.check(lib.wg_scene_download(s.h, big.data_ptr() + 4 * big.element_size(), None, prec))
            assert np.array_equal(big.numpy()[4:].view(np.uint8), x0.view(np.uint8))
            assert not big.numpy()[:4].any()


def test_state_copies_are_stream_ordered():
    """wg_scene_upload_state returns before its copies and repacks finish: a state upload
    followed at once, with no sync, by a step and a download (the end-to-end step) gives
    the fields of the same state uploaded in FP64 and stepped (bit for bit, the same
    skewed passes on both), twice in a row on one scene."""
    sc = scenes.config2(seed=5, nx=1536, ny=1024)
    lib = W.lib()
    out = []
    for fast in (False, True):
        with W.Scene(sc.params, P.FP32, P.COEF_TABLE) as s:
            s.upload(sc.phi, sc.psi, sc.xy, sc.tcc, sc.tc, sc.tgamma)
            s.set_blocking(4, 16, 1)
            for rep in range(2):
                s.time = 0
                if fast:
                    a = np.ascontiguousarray(sc.phi, np.float32)
                    b = np.ascontiguousarray(sc.psi, np.float32)
                    W.check(lib.wg_scene_upload_state(s.h, a.ctypes.data, b.ctypes.data, P.FP32))
                    W.check(lib.wg_scene_step(s.h, 40))
                    x, y = np.empty_like(a), np.empty_like(b)
                    W.check(lib.wg_scene_download(s.h, x.ctypes.data, y.ctypes.data, P.FP32))
                else:
                    s.upload(sc.phi, sc.psi, sc.xy, sc.tcc, sc.tc, sc.tgamma)
                    s.step(40)
                    x, y = s.download(native=True)
            out.append((x, y))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_nonfinite_detector():
    """Blow-up detection through a host-side injected NaN (no device fault)."""
    p, f, xy, _ = variant_inputs("s_dir", seed=9)
    phi = f["phi"].copy()
    phi[p.ny * 10 + 10] = np.nan
    with W.Scene(p, P.FP32, P.COEF_TABLE) as s:
        s.upload(phi, f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        assert s.nonfinite() == 1
        s.step(2)
        assert s.nonfinite() > 1


def test_mask_mode_rejects_ghost_values():
    p, f, xy, nbc = variant_inputs("s_neu", seed=1)
    with W.Scene(p, P.FP32, P.COEF_MASK) as s:
        with pytest.raises(W.WaveGpuError):
            s.upload(f["phi"], f["psi"], xy)
