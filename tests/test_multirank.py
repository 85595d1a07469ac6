"""Multi-rank logic of the benchmark on CPU (gloo, world size 2).

Each rank searches its own template set against the same data (weak
scaling); the only cross-rank operations are a barrier and the max of the
per-rank times.  Runs without a GPU.
"""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, local = bench.dist_info()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    t = bench.dist_max(1.5 + rank, w)
    cfg = bench.make_workload("config0", rank)
    out.put((rank, t, float(cfg["templates"][0, 0, 0, 5]), float(cfg["data"][0, 0, 7])))
    dist.destroy_process_group()


def test_two_ranks_max_time_and_distinct_template_sets():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == res[1][1] == 2.5  # max over ranks
    assert res[0][2] != res[1][2]          # each rank its own templates
    assert np.isfinite(res[0][3]) and np.isfinite(res[1][3])
