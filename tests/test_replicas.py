"""Replica sharding and max-over-ranks timing with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from wsclean_gb300 import replicas


def test_shard_units_partition():
    for world in (1, 2, 3, 8):
        seen = []
        for r in range(world):
            seen += replicas.shard_units(37 * 8, r, world)
        assert sorted(seen) == list(range(37 * 8))
    with pytest.raises(ValueError):
        replicas.shard_units(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units = replicas.shard_units(10, rank, world)
    # rank r pretends its step took (r + 1) seconds
    slowest = replicas.max_over_ranks(float(rank + 1))
    dist.barrier()
    out[rank] = (len(units), slowest)
    dist.destroy_process_group()


def test_two_rank_gloo_replicas():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0][1] == 2.0 and out[1][1] == 2.0
    assert out[0][0] + out[1][0] == 10
    assert replicas.aggregate_rate([out[0][0], out[1][0]], out[0][1]) == 5.0
