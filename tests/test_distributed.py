"""Multi-process host logic of bench.py on CPU (gloo, world size 2): every rank
runs its own independently seeded batch ("replicas only", no data-path
collective); ranks meet only for the barrier and the max/sum reductions of
the timing."""
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "upside2-md_gb300"))
    import bench
    d = bench.Dist()
    t = d.max(1.0 + rank)          # max over ranks of the per-rank time
    units = d.sum(100 * (rank + 1))  # units all ranks processed
    d.barrier()
    import workloads
    w = workloads.workload("C1", seed=1 + rank)  # per-rank seeds: independent replicas
    q.put((rank, t, units, w["seeds"][0]))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_gloo_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert all(r[1] == 2.0 for r in res)      # max of 1.0, 2.0
    assert all(r[2] == 300.0 for r in res)    # 100 + 200
    assert res[0][3] != res[1][3]             # ranks run distinct replicas
