"""Replica aggregation of bench.py across ranks (world size 2, gloo, CPU only): barrier and
max-over-ranks of the timed region, whole-job ms/proof."""
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


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist()
    d.barrier()
    local_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
    total = d.max(local_ms)
    q.put((rank, total, bench.aggregate_ms_per_proof(total, d.world, 10)))
    d.close()


def test_two_rank_max_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [200.0, 200.0]
    assert got[0][2] == pytest.approx(10.0)   # 200 ms for 2 ranks x 10 proofs
