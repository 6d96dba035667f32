"""Replica (N > 1) host path of bench.py on CPU: two gloo ranks on 127.0.0.1 run dist_init,
barrier and the max-over-ranks timing reduction that the multi-GPU run uses (each rank solves
its own copy; the job's value counts every rank's solves over the slowest rank's time)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, w, dist = bench.dist_init()
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 10.0 * (r + 1))     # rank r "took" 10 (r + 1) ms
    value = bench.replica_value(1e6, 3, w, t)
    q.put((r, w, t, value))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest_rank():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(ws))
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == 20.0 for o in out)                       # max over ranks
    assert all(abs(o[3] - 1e6 * 3 * 2 / 0.020) < 1e-3 for o in out)   # all ranks' work / slowest time
