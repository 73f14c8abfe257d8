"""Replica (multi-GPU) host logic with the gloo backend on CPU, world size 2:
gradient averaging, max-over-ranks timing, segment sharding and seeds."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "diffeqflux.jl_gb300"))
    import torch.distributed as dist

    from gbnde import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = np.full(5, float(rank + 1), dtype=np.float32)
    avg = replicas.average_gradients(g)
    t = replicas.max_over_ranks(0.1 * (rank + 1))
    seg = list(replicas.shard_segments(11, rank, world))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, avg.tolist(), t, seg, replicas.replica_seed(7, rank)))


def test_replica_helpers_gloo_world2():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert out[0][1] == out[1][1] == [1.5] * 5
    assert out[0][2] == out[1][2] == pytest.approx(0.2)
    assert out[0][3] + out[1][3] == list(range(11))
    assert out[0][4] != out[1][4]


def test_single_process_is_identity():
    from gbnde import replicas
    g = np.arange(3, dtype=np.float32)
    assert np.array_equal(replicas.average_gradients(g), g)
    assert replicas.max_over_ranks(2.5) == 2.5
