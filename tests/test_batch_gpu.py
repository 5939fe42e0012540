"""Batches of uneven scenes (wg_batch_*): one persistent kernel per update over a
device-side tile work queue, frames replayed as CUDA graphs.

Batch invariance: every instance gives bit-identical fields in a batch (with other
instances admitted and removed around it) and alone (a native scene on the
single-step kernels), in FP32 and FP64.  FP64 batches also match the oracle's values
(1e-12 relative where cos/exp/sin sources enter)."""
import numpy as np
import pytest

import oracle
from helpers import equalize_unwritten, rel_err
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu


def members(seed, count=10):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        sc = scenes.batch_member(rng, smin=(40, 40), smax=(300, 200),
                                 bconds=(P.BC_DIRICHLET, P.BC_PERIODIC, P.BC_ABSORBING, P.BC_VPER_HABS))
        p = sc.params
        if k % 3 == 0:
            p.oscillate_left, p.omega = 1, 0.07
        if k % 4 == 1:
            inside = np.argwhere(sc.xy.reshape(p.nx, p.ny) > 0)
            si, sj = inside[len(inside) // 2]
            p.src_on, p.src_i, p.src_j, p.src_amp, p.src_period = 1, int(si), int(sj), 0.05, 23.0
        if k % 5 == 2:
            p.twospeeds, p.courantb, p.gammab = 1, p.courant / 1.5, 1e-4
        if k % 7 == 3:
            p.kappa = 1e-3  # every term of the update present (FP64: no zero-term form)
        f = dict(phi=sc.phi, psi=sc.psi * 0.99, tmp=np.zeros_like(sc.phi))
        f = equalize_unwritten(p, f, sc.xy)
        out.append((p, f, sc.xy))
    return out


def solo(p, f, xy, prec, n):
    with W.Scene(p, prec, P.COEF_MASK) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy)
        s.step(n)
        return s.download()


@pytest.mark.parametrize("prec", [P.FP32, P.FP64])
def test_batch_invariance_with_admission_and_removal(prec):
    ms = members(1)
    frames = [10, 10, 7]
    with W.Batch(prec) as b:
        slots = [b.add(p, f["phi"], f["psi"], xy) for (p, f, xy) in ms[:6]]
        b.step(frames[0])
        # continuous batching: one leaves, four arrive between frames
        b.remove(slots[2])
        late = [b.add(p, f["phi"], f["psi"], xy) for (p, f, xy) in ms[6:]]
        b.step(frames[1])
        b.step(frames[2])
        n_active, cells = b.count()
        assert n_active == 9
        done = {}
        for k, sl in enumerate(slots):
            if k != 2:
                done[k] = (b.download(sl), sum(frames))
        for k, sl in enumerate(late):
            done[6 + k] = (b.download(sl), frames[1] + frames[2])
        assert b.launches() >= sum(frames)
    for k, ((phi, psi), n) in done.items():
        p, f, xy = ms[k]
        phi1, psi1 = solo(p, f, xy, prec, n)
        assert np.array_equal(phi, phi1), k
        assert np.array_equal(psi, psi1), k


def test_fp64_batch_matches_oracle():
    ms = members(2, count=6)
    with W.Batch(P.FP64) as b:
        slots = [b.add(p, f["phi"], f["psi"], xy) for (p, f, xy) in ms]
        b.step(12)
        for sl, (p, f, xy) in zip(slots, ms):
            tcc, tc, tg = scenes.tables(p, xy)
            new, prev, _, _ = oracle.run(p, f["phi"], f["psi"], f["tmp"], xy, tcc, tc, tg, 12)
            phi, psi = b.download(sl)
            if p.oscillate_left or p.src_on:
                assert rel_err(phi, new) <= 1e-12 and rel_err(psi, prev) <= 1e-12
            else:
                assert np.array_equal(phi, new) and np.array_equal(psi, prev)
            e = b.energy(sl)
            assert abs(e - oracle.energy_total(p, new, prev, xy)) <= 1e-12 * max(1.0, abs(e))


def test_graph_reuse_and_empty_batch():
    ms = members(3, count=3)
    with W.Batch(P.FP32) as b:
        b.step(5)  # empty: nothing to do
        s0 = b.add(*[ms[0][0], ms[0][1]["phi"], ms[0][1]["psi"], ms[0][2]])
        for _ in range(4):
            b.step(10)  # the same graph, replayed
        b.remove(s0)
        b.step(10)
        assert b.count()[0] == 0
        with pytest.raises(W.WaveGpuError):
            b.download(s0)
