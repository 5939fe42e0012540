"""The batch instance with the largest FP32 energy difference in the uneven-batch
workload (instance 221 of the seeded batch: 1028x718, periodic, COURANT 0.052, a disc
array, pulse sigma about 9 cells), stepped in an FP32 batch (skewed passes at the tuned
depth) against the FP64 oracle.

Why this instance: with (phi, psi) stored in FP32 the velocity phi - psi carries the
6e-8 relative rounding of phi, and a small COURANT number makes the velocity small next
to phi (the increments per update are small), so its relative error, and the energy's,
is larger than for fast waves.  A numpy emulation that rounds only the stored levels to
FP32 (every operation in FP64) shows the same energy difference, so the kernels'
arithmetic is not the cause.  The test holds the field to 1e-5 of the initial field
maximum and the energy to 1e-5 after 2000 updates, and prints the measured values."""
import numpy as np
import pytest

import oracle
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu
UPDATES = 2000


def worst_member():
    rng = np.random.default_rng(1000)  # the uneven batch's seed (bench.py run_batch, rank 0)
    for k in range(222):
        m = scenes.batch_member(rng)
    assert (m.params.nx, m.params.ny, m.params.b_cond) == (1028, 718, P.BC_PERIODIC)
    return m


def test_worst_batch_instance_fp32_vs_oracle():
    m = worst_member()
    p = m.params
    new, prev, _, _ = oracle.run(p, m.phi, m.psi, np.zeros_like(m.phi), m.xy, m.tcc, m.tc, m.tgamma, UPDATES)
    with W.Batch(P.FP32) as b:
        slot = b.add(p, m.phi, m.psi, m.xy)
        for _ in range(UPDATES // 10):
            b.step(10)
        phi, psi = b.download(slot)
        e32 = b.energy(slot)
    e64 = oracle.energy_total(p, new, prev, m.xy, compensated=True)
    ferr = float(np.max(np.abs(phi - new)) / np.max(np.abs(m.phi)))
    derr = abs(e32 - e64) / abs(e64)
    print(f"\nworst batch instance, {UPDATES} updates, FP32 vs the FP64 oracle: field {ferr:.2e} of the initial "
          f"maximum, energy {derr:.2e}")
    assert ferr <= 1e-5
    assert derr <= 1e-5
