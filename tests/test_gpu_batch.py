"""Batches of uneven searches in one graph (fmf_batch_*), needs a GB300.

Every search of a batch must equal the same search run alone, and the
oracle, at the suite's tolerance; re-running the graph after refilling an
input must see the new input.
"""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from tests._cases import random_search
from tests.test_gpu_parity import TOL, assert_parity, oracle_of

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPES = [  # (T, S, C, L, N, step, normalize, network_sum)
    (3, 4, 3, 200, 30000, 1, "short", True),
    (2, 2, 1, 610, 50000, 2, "full", True),
    (5, 3, 3, 64, 12000, 1, "full", True),
    (1, 6, 1, 1200, 40000, 1, "short", True),
    (2, 2, 3, 97, 9000, 3, "short", False),
    (4, 5, 1, 333, 20001, 2, "short", True),
]


def _dev(seed, T, S, C, L, N, step, normalize, network_sum):
    tp, mo, w, d = random_search(seed, T, S, C, L, N, -20, 250,
                                 dc=2.0 if normalize == "full" else 0.0, zero_weights=1)
    n_corr = (N - L) // step + 1
    shape = (T, n_corr) if network_sum else (T, n_corr, S, C)
    g = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in
         (tp, np.sum(tp ** 2, axis=-1).astype(np.float32), mo, w, d)]
    out = torch.full(shape, 5.0, dtype=torch.float32, device="cuda")
    return (tp, mo, w, d), g, out


@pytest.mark.parametrize("precision", ["split_bf16", "fp32"])
def test_batch_matches_single_searches_and_oracle(oracle_built, precision):
    b = fmf.Batch(precision)
    cases = []
    for i, sh in enumerate(SHAPES):
        host, g, out = _dev(100 + i, *sh)
        b.add(*g, sh[5], out, sh[6], sh[7])
        cases.append((sh, host, g, out))
    n_launch = b.run()
    torch.cuda.synchronize()
    assert n_launch > 0
    for sh, host, g, out in cases:
        T, S, C, L, N, step, normalize, network_sum = sh
        single = torch.empty_like(out)
        fmf.matched_filter_device(*g, step, single, normalize, network_sum, precision)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.abs(got - single.cpu().numpy()).max() <= TOL
        assert_parity(got, oracle_of(oracle_built, *host, step, normalize, network_sum))
    b.close()


def test_batch_graph_replay_reads_new_inputs(oracle_built):
    b = fmf.Batch("split_bf16")
    sh = SHAPES[0]
    host, g, out = _dev(7, *sh)
    b.add(*g, sh[5], out, sh[6], sh[7])
    b.run()
    torch.cuda.synchronize()
    first = out.cpu().numpy().copy()
    rng = np.random.default_rng(8)
    d2 = rng.standard_normal(host[3].shape).astype(np.float32)
    g[4].copy_(torch.from_numpy(d2))
    b.run()
    torch.cuda.synchronize()
    second = out.cpu().numpy()
    assert not np.array_equal(first, second)
    assert_parity(second, oracle_of(oracle_built, host[0], host[1], host[2], d2, sh[5], sh[6], sh[7]))
    b.close()


def test_many_searches_span_several_persistent_launches():
    """More than 64 searches: one persistent launch per 64."""
    b = fmf.Batch("split_bf16")
    outs = []
    for i in range(70):
        host, g, out = _dev(300 + i, 1, 2, 1, 40, 3000, 1, "short", True)
        b.add(*g, 1, out)
        outs.append((g, out))
    b.run()
    torch.cuda.synchronize()
    for g, out in outs[::7]:
        single = torch.empty_like(out)
        fmf.matched_filter_device(*g, 1, single, "short", True, "split_bf16")
        torch.cuda.synchronize()
        assert np.abs(out.cpu().numpy() - single.cpu().numpy()).max() <= TOL
    b.close()
