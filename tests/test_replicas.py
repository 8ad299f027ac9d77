"""Multi-rank (replica) aggregation on CPU with the gloo backend, world size 2."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from piquassoboost_gb300.replicas import replica_throughput, shard_seeds
    # rank r did (r + 1) * 3 units in (r + 1) seconds
    v, tmax = replica_throughput((rank + 1) * 3, float(rank + 1))
    seeds = shard_seeds(36, rank, 3)
    q.put((rank, v, tmax, seeds))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_gloo_world2():
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
    # 3 + 6 units over max(1, 2) seconds on every rank
    for rank, v, tmax, seeds in res:
        assert abs(v - 4.5) < 1e-12 and tmax == 2.0
    assert set(res[0][3]).isdisjoint(res[1][3])


def test_replica_throughput_single_process():
    from piquassoboost_gb300.replicas import replica_throughput
    assert replica_throughput(10, 2.0) == (5.0, 2.0)
