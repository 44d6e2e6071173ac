"""Multi-GPU is replicas only: no collective on the data path, a barrier and a
max over ranks of the timings.  Covered here with two gloo ranks on CPU."""
import os
import socket

import torch.multiprocessing as mp

from graphitethree_gb300.replicas import max_over_ranks, shard


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
    dist.barrier()
    got = max_over_ranks([1.0 + rank, 10.0 - rank, 3.0], dist)
    out[rank] = got
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0] == out[1] == [2.0, 10.0, 3.0]


def test_single_rank_is_identity_and_shards_partition():
    assert max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
    items = list(range(11))
    parts = [shard(items, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == items
    assert all(set(a).isdisjoint(b) for i, a in enumerate(parts) for b in parts[i + 1:])
