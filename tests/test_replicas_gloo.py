"""The replica harness with two gloo ranks on CPU: disjoint seeds, max-over-ranks
timing and whole-job throughput, as bench.py uses them under torchrun."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from pybella_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = replicas.seeds_for_rank(rank, 5)
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        slow = replicas.max_over_ranks(0.5 + rank)          # rank 1 is the slowest
        rate = replicas.aggregate_rate(5, world, slow)
        out.put((rank, gathered, slow, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, slow, rate in res:
        assert set(gathered[0]).isdisjoint(gathered[1])
        assert slow == 1.5
        assert rate == pytest.approx(10 / 1.5)


def test_single_process_fallbacks():
    from pybella_gb300 import replicas
    assert replicas.max_over_ranks(2.5) == 2.5
    assert replicas.seeds_for_rank(0, 3) == [0, 1, 2]
    with pytest.raises(ValueError):
        replicas.seeds_for_rank(0, 2000)
