"""Replica bookkeeping of multi-GPU runs (bench.py under torchrun), on CPU with gloo: the
maximum over ranks and the whole-job rate, world size 2."""
import os
import socket
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "lpm-v2_gb300"))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from replicas import max_over_ranks, replica_rate
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds = [2.0, 3.0][rank]  # rank 1 is the slower replica
    m = max_over_ranks(seconds, dist)
    rate = replica_rate(100.0, seconds, dist)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, m, rate))


def test_replica_rate_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, rate in res:
        assert m == 3.0                      # the slowest rank's time
        assert rate == pytest.approx(200.0 / 3.0)  # both ranks' work over that time


def test_replica_rate_single_process():
    from replicas import max_over_ranks, replica_rate
    assert max_over_ranks(1.5) == 1.5
    assert replica_rate(10.0, 2.0) == 5.0
