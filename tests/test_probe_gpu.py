"""SAVE_TIME_SERIES probes (wave_billiard.c:667-672, 900-908) on the GPU: phi at the
probe cells after every update, against the oracle stepped one update at a time
(FP64 bit for bit, FP32 within 1e-5 of the field maximum); the buffer refuses to
overflow and partial reads keep the rest; the drop-in's resident cell read."""
import numpy as np
import pytest

import oracle
from helpers import variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu

CELLS = [(10, 20), (33, 22), (60, 40), (0, 5)]


def oracle_series(p, f, xy, n):
    phi, psi, tmp = f["phi"], f["psi"], f["tmp"]
    out = []
    for _ in range(n):
        phi, psi, tmp, _ = oracle.run(p, phi, psi, tmp, xy, f["tcc"], f["tc"], f["tgamma"], 1)
        out.append([phi.reshape(p.nx, p.ny)[i, j] for i, j in CELLS])
    return np.array(out), phi


@pytest.mark.parametrize("prec", [P.FP64, P.FP32])
def test_probes_match_oracle_every_update(prec):
    p, f, xy, _ = variant_inputs("s_abs", seed=8)
    n = 12
    ref, final = oracle_series(p, f, xy, n)
    with W.Scene(p, prec, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.set_probes(CELLS, capacity=n)
        s.step(5)
        first = s.read_probes(max_updates=3)   # partial read: updates 1-3
        s.step(7)
        rest = s.read_probes()                  # updates 4-12
        got = np.vstack([first, rest])
        with pytest.raises(W.WaveGpuError):
            s.step(n + 1)                       # would overflow the buffer
    assert got.shape == (n, len(CELLS))
    if prec == P.FP64:
        assert np.array_equal(got, ref)
    else:
        assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(final))


def test_probe_out_of_grid_refused():
    p, f, xy, _ = variant_inputs("s_abs", seed=8)
    with W.Scene(p, P.FP64, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        with pytest.raises(W.WaveGpuError):
            s.set_probes([(p.nx, 0)], capacity=4)


def test_dropin_resident_cell():
    p, f, xy, _ = variant_inputs("s_dir", seed=4)
    new, _, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], 9)
    W.configure(p)
    W.set_mode(True)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    for _ in range(3):
        W.evolve_wave(rf)
    for i, j in [(5, 7), (30, 20), (66, 44)]:
        assert W.dropin_cell(rf, i, j) == new.reshape(p.nx, p.ny)[i, j]
    W.set_mode(False)
