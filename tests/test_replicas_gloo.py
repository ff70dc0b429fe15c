"""CPU: the multi-GPU path of bench.py (independent replicas, no data-path
collective) reduced over two gloo ranks: job time = slowest rank, work = sum."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    ms = [10.0, 12.5][rank]
    units = [3663, 3600][rank]
    out = bench.reduce_over_ranks(ms, units, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_replicas_reduce_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    [p.start() for p in ps]
    [p.join(timeout=120) for p in ps]
    assert all(p.exitcode == 0 for p in ps)
    res = dict(q.get(timeout=5) for _ in range(2))
    for r in range(2):
        ms, units, rate = res[r]
        assert ms == 12.5 and units == 3663 + 3600
        assert rate == pytest.approx((3663 + 3600) / 0.0125)
