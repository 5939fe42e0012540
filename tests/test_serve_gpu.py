"""Serving loop (wg_server_*): continuous batching under an HBM budget.

Requests arrive while others are resident; each tick admits what the budget allows
(first come first served), advances every resident scene by one frame of updates in one
graph launch, and returns RGB8 frames.  The final state of every request must be
bit-identical to the same scene run alone (a native scene on the single-step kernels),
and each returned frame to the solo scene's frame at the same step."""
import numpy as np
import pytest

from helpers import equalize_unwritten, frame_lut
from youtube_simulations_gb300 import params as P
from youtube_simulations_gb300 import scenes
from youtube_simulations_gb300 import wavegpu as W

pytestmark = pytest.mark.gpu
LUT = frame_lut(7)


def requests(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        sc = scenes.batch_member(rng, smin=(48, 48), smax=(260, 180),
                                 bconds=(P.BC_DIRICHLET, P.BC_PERIODIC, P.BC_ABSORBING))
        p = sc.params
        if k % 3 == 1:
            p.twospeeds, p.courantb, p.gammab = 1, p.courant / 1.5, 1e-4
        f = equalize_unwritten(p, dict(phi=sc.phi, psi=sc.psi, tmp=np.zeros_like(sc.phi)), sc.xy)
        frames = int(rng.integers(2, 7))
        out.append((p, f, sc.xy, frames))
    return out


def solo(p, f, xy, prec, n, want_frame=False):
    with W.Scene(p, prec, P.COEF_MASK) as s:
        s.set_blocking(1)
        s.upload(f["phi"], f["psi"], xy)
        s.step(n)
        img = s.frame_rgb8(LUT) if want_frame else None
        return s.download() + (img,)


@pytest.mark.parametrize("prec", [P.FP32, P.FP64])
def test_results_identical_alone_and_in_the_mix(prec):
    reqs = requests(3, 9)
    steps = 5
    one = W.scene_bytes(reqs[0][0], prec) * 2
    with W.Server(LUT, precision=prec, steps_per_frame=steps) as probe:
        budget = int(3.2 * max(probe.request_bytes(p) for (p, _, _, _) in reqs))
    with W.Server(LUT, precision=prec, steps_per_frame=steps, hbm_budget=budget, max_scenes=64) as srv:
        ids = []
        # arrivals spread over the first ticks: later requests join a running batch
        pending = list(reqs)
        ticks = 0
        while pending or any(srv.state(r)[0] != 2 for r in ids):
            for _ in range(2):
                if pending:
                    p, f, xy, frames = pending.pop(0)
                    ids.append(srv.submit(p, f["phi"], f["psi"], xy, frames, keep=True))
            srv.tick()
            ticks += 1
            assert ticks < 200
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["queued"] == 0 and st["resident"] == 0
        assert st["bytes_peak"] <= budget
        assert st["frame_latency_p99_ms"] >= st["frame_latency_p50_ms"] > 0
        for rid, (p, f, xy, frames) in zip(ids, reqs):
            phi, psi = srv.result(rid)
            phi1, psi1, _ = solo(p, f, xy, prec, frames * steps)
            assert np.array_equal(phi, phi1), rid
            assert np.array_equal(psi, psi1), rid
    assert one > 0


def test_frames_match_solo_scene():
    reqs = requests(4, 3)
    steps = 4
    with W.Server(LUT, precision=P.FP32, steps_per_frame=steps) as srv:
        ids = [srv.submit(p, f["phi"], f["psi"], xy, 3) for (p, f, xy, _) in reqs]
        for t in range(3):
            srv.tick()
            for rid, (p, f, xy, _) in zip(ids, reqs):
                idx, img = srv.frame(rid)
                assert idx == t
                _, _, ref = solo(p, f, xy, P.FP32, (t + 1) * steps, want_frame=True)
                assert np.array_equal(img, ref)


def test_budget_refusal_and_queueing():
    reqs = requests(5, 4)
    with W.Server(LUT, precision=P.FP32, steps_per_frame=2) as probe:
        sizes = [probe.request_bytes(p) for (p, _, _, _) in reqs]
    budget = max(sizes) + min(sizes) // 2   # room for one request at a time
    with W.Server(LUT, precision=P.FP32, steps_per_frame=2, hbm_budget=budget) as srv:
        ids = [srv.submit(p, f["phi"], f["psi"], xy, 2) for (p, f, xy, _) in reqs]
        srv.tick()
        st = srv.stats()
        assert st["resident"] == 1 and st["queued"] == len(reqs) - 1
        while srv.stats()["completed"] < len(reqs):
            srv.tick()
        p = P.make_params(2000, 2000)
        z = np.zeros(2000 * 2000)
        with pytest.raises(W.WaveGpuError):
            srv.submit(p, z, z, np.zeros(2000 * 2000, np.int16), 1)


def test_pipelined_ticks_give_the_same_frames_and_results():
    """pipeline=1: tick t enqueues its device work and then completes tick t-1, whose
    frames are then readable; drain() completes the last tick.  Every frame and every
    final state equal those of the synchronous server and of the scene run alone."""
    reqs = requests(6, 4)
    steps = 3
    with W.Server(LUT, precision=P.FP32, steps_per_frame=steps, pipeline=True) as srv:
        ids = [srv.submit(p, f["phi"], f["psi"], xy, frames, keep=True) for (p, f, xy, frames) in reqs]
        seen = {rid: [] for rid in ids}
        ticks = 0
        while any(srv.state(r)[0] != P.REQ_DONE for r in ids):
            got = srv.tick() if ticks < 40 else srv.drain()
            ticks += 1
            assert ticks < 60
            for rid in ids:
                try:
                    idx, img = srv.frame(rid)
                except W.WaveGpuError:
                    continue
                if not seen[rid] or seen[rid][-1][0] != idx:
                    seen[rid].append((idx, img))
            if got == 0 and srv.stats()["resident"] == 0 and srv.stats()["queued"] == 0:
                srv.drain()
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["tick_device_p50_ms"] > 0
        for rid, (p, f, xy, frames) in zip(ids, reqs):
            assert [i for i, _ in seen[rid]] == list(range(frames)), rid
            for idx, img in seen[rid]:
                _, _, ref = solo(p, f, xy, P.FP32, (idx + 1) * steps, want_frame=True)
                assert np.array_equal(img, ref), (rid, idx)
            phi, psi = srv.result(rid)
            phi1, psi1, _ = solo(p, f, xy, P.FP32, frames * steps)
            assert np.array_equal(phi, phi1) and np.array_equal(psi, psi1), rid


@pytest.mark.parametrize("pipeline", [False, True])
def test_cancellation(pipeline):
    """A queued request cancelled leaves the queue at once; a resident one leaves the
    batch at the next tick and returns its bytes to the budget; a finished one cannot be
    cancelled.  The other requests' results are unaffected."""
    reqs = requests(8, 4)
    with W.Server(LUT, precision=P.FP32, steps_per_frame=2) as probe:
        order = sorted(range(len(reqs)), key=lambda k: -probe.request_bytes(reqs[k][0]))
        reqs = [reqs[k] for k in order]  # the two largest first
        sizes = [probe.request_bytes(p) for (p, _, _, _) in reqs]
    budget = sizes[0] + sizes[1]  # the first two fit together, a third does not
    with W.Server(LUT, precision=P.FP32, steps_per_frame=2, hbm_budget=budget, pipeline=pipeline) as srv:
        ids = [srv.submit(p, f["phi"], f["psi"], xy, 6, keep=True) for (p, f, xy, _) in reqs]
        srv.tick()
        assert srv.state(ids[0])[0] == P.REQ_RESIDENT and srv.state(ids[3])[0] == P.REQ_QUEUED
        srv.cancel(ids[3])                       # queued
        assert srv.state(ids[3])[0] == P.REQ_CANCELLED
        srv.tick()
        srv.cancel(ids[1])                       # resident
        with pytest.raises(W.WaveGpuError):
            srv.cancel(ids[1])                   # already cancelled
        srv.tick()
        assert srv.state(ids[1])[0] == P.REQ_CANCELLED
        ticks = 0
        while srv.state(ids[0])[0] != P.REQ_DONE or srv.state(ids[2])[0] != P.REQ_DONE:
            srv.tick()
            ticks += 1
            assert ticks < 40
        srv.drain()
        with pytest.raises(W.WaveGpuError):
            srv.cancel(ids[0])                   # finished
        st = srv.stats()
        assert st["cancelled"] == 2 and st["completed"] == 2 and st["resident"] == 0
        assert st["bytes_resident"] == 0
        for k in (0, 2):
            p, f, xy, _ = reqs[k]
            phi, psi = srv.result(ids[k])
            phi1, psi1, _ = solo(p, f, xy, P.FP32, 12)
            assert np.array_equal(phi, phi1) and np.array_equal(psi, psi1), k
