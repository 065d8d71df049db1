"""Replica aggregation over world_size 2 with gloo, on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from npbench_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, lr = replicas.dist_info()
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slowest
        slowest = replicas.max_over_ranks(local_ms)
        q.put((r, w, slowest, replicas.job_throughput(1000, w, slowest / 1e3)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_slowest_rank_and_total_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, slowest, thr in out:
        assert w == 2 and slowest == 15.0
        assert thr == pytest.approx(1000 * 2 / 0.015)


def test_single_process_is_identity():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_throughput(10, 1, 2.0) == 5.0
    with pytest.raises(ValueError):
        replicas.job_throughput(10, 1, 0.0)
