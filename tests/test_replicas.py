"""Replica host logic with two gloo ranks on CPU: max-over-ranks timing, distinct
per-rank seeds, whole-job throughput."""
import os
import socket

import torch.multiprocessing as mp

from qml_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, lr = replicas.rank_info()
    t = replicas.max_over_ranks(10.0 + 5.0 * r)
    out.put((r, w, t, replicas.replica_seed(2024, r)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 15.0 for r in res)          # every rank sees the slowest time
    assert res[0][3] != res[1][3]                  # each replica fits its own problem


def test_single_process_and_throughput():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.rank_info()[0] >= 1
    assert replicas.job_throughput(1.0, 0.5, 4) == 8.0
