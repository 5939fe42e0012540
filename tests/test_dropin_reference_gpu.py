"""The reference's own code with its stepper replaced by include/wavegpu_dropin.h.

oracle/build_ref.py builds each small configuration twice from the reference's
sources: once as is (CPU) and once with evolve_wave / evolve_wave_half replaced by the
drop-in header linked to libwavegpu.so.  Both binaries run the reference's driver loop
on identical inputs; the fields must agree bit for bit (1e-12 relative where
oscillating_bc's cos/exp enter)."""
import numpy as np
import pytest

import ref_variants
import refio
from helpers import rel_err, variant_inputs

pytestmark = pytest.mark.gpu

DROPIN = [n for n, v in ref_variants.VARIANTS.items() if v.get("dropin")]


@pytest.mark.parametrize("variant", DROPIN)
@pytest.mark.parametrize("nsteps", [6, 7])
def test_reference_driver_on_gpu_stepper(variant, nsteps):
    base = variant[: -len("__dropin")]
    if not (refio.available(base) and refio.available(variant)):
        pytest.skip("compiled reference or drop-in build absent")
    p, f, xy, nbc = variant_inputs(base, seed=31)
    cpu = refio.run(base, p.nx, p.ny, refio.STEP, nsteps, fields=f, xy=xy, nbc=nbc)
    gpu = refio.run(variant, p.nx, p.ny, refio.STEP, nsteps, fields=f, xy=xy, nbc=nbc)
    for k in ("phi", "psi", "tmp"):
        if p.oscillate_left:
            assert rel_err(gpu[k], cpu[k]) <= 1e-12, k
        else:
            assert np.array_equal(gpu[k], cpu[k]), k
    assert abs(gpu["energy"] - cpu["energy"]) <= 1e-12 * max(1.0, abs(cpu["energy"]))
