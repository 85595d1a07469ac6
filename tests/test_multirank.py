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


def test_template_blocks_partition_the_templates():
    from fast_matched_filter_gb300.sharding import template_block
    for T in (1, 2, 7, 100, 501):
        for world in (1, 2, 3, 8):
            blocks = [template_block(T, world, r) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == T
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
            sizes = [t1 - t0 for t0, t1 in blocks]
            assert max(sizes) - min(sizes) <= 1 and min(sizes) >= 0


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist

    from oracle import cpu
    from fast_matched_filter_gb300.sharding import matched_filter_sharded
    from tests._cases import random_search

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    tp, mo, w, d = random_search(11, 5, 3, 2, 64, 3000, -20, 80, zero_weights=1)
    oracle = lambda t, m, ww, dd, s: cpu.run_oracle(t, m, ww, dd, s)  # noqa: E731
    full = matched_filter_sharded(tp, mo, w, d, 1, search=oracle)
    rows, (t0, t1) = matched_filter_sharded(tp, mo, w, d, 1, search=oracle, gather=False)
    out.put((rank, full, rows, t0, t1))
    dist.destroy_process_group()


def test_two_ranks_reproduce_the_single_process_search(oracle_built):
    """Two gloo ranks each search their own block of one search's templates
    (the reference's template-parallel split over GPUs, matched_filter.cu:261-280);
    the gathered rows equal the single-process result bit for bit.  The CPU
    oracle stands in for the per-rank GPU search."""
    torch = pytest.importorskip("torch")
    from tests._cases import random_search
    tp, mo, w, d = random_search(11, 5, 3, 2, 64, 3000, -20, 80, zero_weights=1)
    single = oracle_built.run_oracle(tp, mo, w, d, 1)
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=120) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r[3], r[4]) for r in res] == [(0, 3), (3, 5)]
    for rank, full, rows, t0, t1 in res:
        assert np.array_equal(full, single)
        assert np.array_equal(rows, single[t0:t1])
