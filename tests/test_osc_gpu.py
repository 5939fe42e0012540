"""Every oscillating_bc schedule (sub_wave.c:11965-12162) on the GPU.

The oracle's oscillating_bc is pinned bit for bit to the reference for each of the 15
schedules and the two negative-y-shift builds (test_oracle_vs_reference.py, one
compiled reference build per schedule).  Here each of those 17 macro sets drives an
OSCILLATE_LEFT stepper on a 67x45 ellipse, Dirichlet, through the drop-in evolve_wave
and through an FP64 scene, against the oracle: <= 1e-12 relative to the field maximum
(CUDA's and glibc's cos/exp/sin may differ in the last bit).  The FP32 scene is held to
the FP32 bar, 1e-5 relative."""
import numpy as np
import pytest

import oracle
import ref_variants
from helpers import equalize_unwritten, rel_err, variant_inputs
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu

OSC = [n for n, v in ref_variants.VARIANTS.items() if v["kind"] == "osc"]
NSTEPS = 45


def inputs(variant, seed):
    p, f, xy, _ = variant_inputs(variant, seed=seed, oscillate_left=1)
    assert p.oscillate_left == 1 and p.b_cond == P.BC_DIRICHLET
    return p, f, xy


@pytest.mark.parametrize("variant", OSC)
def test_schedule_dropin(variant):
    p, f, xy = inputs(variant, 51)
    new, prev, third, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], NSTEPS)
    W.configure(p)
    W.set_mode(False)
    W.set_dropin_time(0)
    rf = W.RowFields(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"])
    for _ in range(NSTEPS // 3):
        W.evolve_wave(rf)
    # the left column carries the schedule's values (not all zero over the run)
    assert np.any(rf.phi[0, 1:-1] != f["phi"].reshape(p.nx, p.ny)[0, 1:-1])
    assert rel_err(rf.phi.reshape(-1), new) <= 1e-12
    assert rel_err(rf.psi.reshape(-1), prev) <= 1e-12
    assert rel_err(rf.tmp.reshape(-1), third) <= 1e-12


@pytest.mark.parametrize("variant", OSC)
@pytest.mark.parametrize("prec", [P.FP64, P.FP32])
def test_schedule_scene(variant, prec):
    p, f, xy = inputs(variant, 52)
    f = equalize_unwritten(p, f, xy)
    new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, f["tcc"], f["tc"], f["tgamma"], NSTEPS)
    with W.Scene(p, prec, P.COEF_TABLE) as s:
        s.upload(f["phi"], f["psi"], xy, f["tcc"], f["tc"], f["tgamma"])
        s.step(NSTEPS)
        phi, psi = s.download()
    tol = 1e-12 if prec == P.FP64 else 1e-5
    assert rel_err(phi, new) <= tol
    assert rel_err(psi, prev) <= tol
