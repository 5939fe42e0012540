"""FP64 steppers bit for bit, signs of zero included.

The FP64 update fuses its two exact products with their adds (-y + 2x and delta - 4x
are one __fma_rn each), which rounds the same exact value once, as the reference's
separate multiply and add do.  With every term of the update present (KAPPA != 0 and a
varying GAMMA table) the fields must therefore equal the oracle's in every bit, not only
in value.  A checkerboard patch of +0 and -0 cells inside the domain exercises the
zero-sign rule of IEEE 754 for both forms.  (With KAPPA = 0 or GAMMA = 0 the native
scenes leave the zero term out; a zero may then change sign, and the other tests compare
values.)"""
import numpy as np
import pytest

import oracle
from helpers import equalize_unwritten, variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu


def signed_zero_inputs(seed):
    p, f, xy, nbc = variant_inputs("s_dir", seed=seed)  # KAPPA = 0.001, per-cell GAMMA table
    assert p.kappa != 0.0 and nbc is None
    grid = xy.reshape(p.nx, p.ny)
    inside = np.argwhere(grid[5:-5, 5:-5] > 0) + 5
    ci, cj = inside[len(inside) // 3]
    ii, jj = np.meshgrid(np.arange(-3, 4), np.arange(-3, 4), indexing="ij")
    f = dict(f)
    for k, par in (("phi", 0), ("psi", 1), ("tmp", 0)):
        a = f[k].reshape(p.nx, p.ny).copy()
        a[ci - 3:ci + 4, cj - 3:cj + 4] = np.where((ii + jj + par) % 2 == 0, 0.0, -0.0)
        f[k] = a.reshape(-1)
    return p, f, xy


def bits(a):
    return np.ascontiguousarray(a, np.float64).reshape(-1).view(np.uint64)


@pytest.mark.parametrize("nsteps", [1, 2, 23])
def test_fp64_scene_bitwise(nsteps):
    p, f, xy = signed_zero_inputs(seed=41)
    f = equalize_unwritten(p, f, xy)
    new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], nsteps)
    assert np.any(bits(f["phi"]) == np.uint64(1 << 63))  # the patch holds -0 cells
    with W.Scene(p, P.FP64, P.COEF_TABLE) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.step(nsteps)
        phi, psi = s.download()
    assert np.array_equal(bits(phi), bits(new))
    assert np.array_equal(bits(psi), bits(prev))


@pytest.mark.parametrize("nsteps", [3, 24])
def test_fp64_dropin_bitwise(nsteps):
    p, f, xy = signed_zero_inputs(seed=43)
    new, prev, third, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], nsteps)
    W.configure(p)
    W.set_mode(False)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    for _ in range(nsteps // 3):
        W.evolve_wave(rf)
    assert np.array_equal(bits(rf.phi), bits(new))
    assert np.array_equal(bits(rf.psi), bits(prev))
    assert np.array_equal(bits(rf.tmp), bits(third))
