"""The N > 1 path of bench.py on CPU: replicas only (every rank advances its own seeded
instance, no collective on the data path), the job's time is the slowest rank's (one
all-reduce MAX over gloo, world size 2), and the whole-job rate sums the replicas."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, _ = bench.dist_env()
        t = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")  # rank 1 is the slow one
        bench._package()
        from youtube_simulations_gb300 import scenes
        sc = scenes.config2(seed=r, nx=64, ny=48, ndiscs=4)
        q.put((r, t, float(np.sum(sc.phi)), tuple(sc.meta["source"])))
    except Exception as e:  # report instead of leaving the parent waiting
        q.put((rank, repr(e), None, None))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_seeds():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [15.0, 15.0]           # both ranks see the slowest time
    assert out[0][2] != out[1][2] or out[0][3] != out[1][3]  # seed = rank: different replicas


def test_whole_job_rate_sums_replicas():
    one = bench.whole_job_rate(1, 8_294_400, 100, 12.0)
    assert abs(bench.whole_job_rate(2, 8_294_400, 100, 12.0) - 2 * one) < 1e-9
    assert abs(one - 8_294_400 * 100 / 0.012 / 1e9) < 1e-9
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
