"""Multi-rank replicas on CPU (gloo, world size 2): bench.py's N>1 logic.

On N GPUs every rank encodes its own stream (no data-path collective); the
only cross-rank steps are the barrier around the timed region and the max of
the ranks' times, from which the whole-job rate follows."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        t = bench.max_over_ranks(1.5 + rank, dist, torch.device("cpu"))
        rate = bench.whole_job_rate(120, world, t)
        from mptc_gb300.synth import FHD1080, StreamSpec
        seed = StreamSpec(**{**FHD1080.__dict__, "seed": FHD1080.seed + rank}).seed
        out.put((rank, t, rate, seed))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]            # max over ranks, on every rank
    assert [r[2] for r in res] == [2 * 120 / 2.5] * 2   # whole-job rate
    assert res[0][3] != res[1][3]                       # each replica encodes its own stream


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.0, None, None) == 3.0
    assert bench.whole_job_rate(120, 1, 0.1) == pytest.approx(1200.0)
