"""The benchmark workloads at their full sizes, per workload (needs a GB300).

* continuous record (S=20, C=3, N=1,080,000, T=100, L=800; channel sigma
  log-U[1e-2, 1e2], zeroed gaps on 4 stations; 'short'): the first two
  templates over the whole trace against the oracle's 'cpu' arch (the
  reference's matched_filter.c:22-96) in both forms; FP64 windows at the
  start, middle and end of the valid range and around the zeroed gaps; the
  two forms over all 100 templates;
* DC offset + full (S=16, C=3, N=2,160,000, T=200, L=600, step 2, DC 1e3):
  max and p99.9 |cc - FP64| on two templates x 200,000 lags for the plain,
  split-bf16 and single-bf16 forms (the first two held to 1e-5), with the
  reference 'precise' arch's own error beside them (matched_filter.c:98-168);
* 64 uneven searches in one batch (T 10-500, S 4-40, C 1/3, L 200-1200,
  N 1e5-4.32M, step 1/2, half 'full'): every search's first template on
  1,024 lags in the middle of its range against FP64.
"""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import synthetic
from oracle import fp64
from tests.test_gpu_parity import TOL, assert_parity

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _device(tp, mo, w, d):
    return [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in
            (tp, np.sum(tp ** 2, axis=-1).astype(np.float32), mo, w, d)]


@pytest.fixture(scope="module")
def continuous():
    cfg = synthetic.config1(seed=101)
    tp, mo, w, d = cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"]
    T, S, C, L = tp.shape
    N = d.shape[-1]
    g = _device(tp, mo, w, d)
    outs = {}
    for precision in ("fp32", "split_bf16"):
        out = torch.empty((T, N - L + 1), dtype=torch.float32, device="cuda")
        fmf.matched_filter_device(*g, 1, out, precision=precision)
        outs[precision] = out
    torch.cuda.synchronize()
    return cfg, outs


def test_continuous_record_against_the_oracle(oracle_built, continuous):
    cfg, outs = continuous
    tp, mo, w, d = cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"]
    ref = oracle_built.run_oracle(tp[:2], mo[:2], w[:2], d, 1, "cpu", "short", True)
    for precision, out in outs.items():
        assert_parity(out[:2].cpu().numpy(), ref, TOL)


def _gap_edges(d):
    """Sample indices where a zeroed segment of some channel starts or ends
    (the noise itself is never exactly 0)."""
    zero = np.any(d.reshape(-1, d.shape[-1]) == 0.0, axis=0)
    return np.flatnonzero(np.diff(zero.astype(np.int8)) != 0)


def test_continuous_record_fp64_windows(continuous):
    cfg, outs = continuous
    tp, mo, w, d = cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"]
    T, S, C, L = tp.shape
    N = d.shape[-1]
    edges = _gap_edges(d)
    assert edges.size > 0
    worst = {p: 0.0 for p in outs}
    for t in (0, 41, 99):
        k0, k1 = fp64.valid_range(mo[t].reshape(-1), 1, L, N)
        starts = [k0, (k0 + k1) // 2, k1 - 600]
        # windows whose data cross the start or end of a zeroed gap
        for e in edges[:: max(1, edges.size // 4)][:4]:
            a = int(e) - L - int(mo[t].max())
            if k0 <= a and a + 600 <= k1:
                starts.append(a)
        for a in starts:
            ref = fp64.fp64_matched_filter(tp, mo, w, d, 1, "short", True, k_range=(a, a + 600),
                                           t_index=[t])[0]
            for p, out in outs.items():
                got = out[t, a:a + 600].cpu().numpy().astype(np.float64)
                worst[p] = max(worst[p], float(np.abs(got - ref).max()))
    print("continuous record, max |cc - FP64| over the windows:", worst)
    assert max(worst.values()) <= TOL, worst


def test_continuous_record_forms_agree_everywhere(continuous):
    _, outs = continuous
    a, b = outs["fp32"], outs["split_bf16"]
    assert torch.equal(a == 0, b == 0)
    diff = (a - b).abs().max().item()
    assert diff <= TOL, diff


def _crop(d, step, k0, K, L, max_mo):
    """The data a search needs for output indices [k0, k0 + K)."""
    a = k0 * step
    return np.ascontiguousarray(d[..., a:a + (K - 1) * step + L + max_mo])


def test_dc_offset_full_precision_vs_fp64(oracle_built):
    cfg = synthetic.config2(seed=102)
    tp, mo, w, d = cfg["templates"][:2], cfg["moveouts"][:2], cfg["weights"][:2], cfg["data"]
    T, S, C, L = tp.shape
    N, step = d.shape[-1], cfg["step"]
    k0, K = 400000, 200000
    ref = fp64.fp64_matched_filter(tp, mo, w, d, step, "full", True, k_range=(k0, k0 + K))
    g = _device(tp, mo, w, d)
    n_corr = (N - L) // step + 1
    rows = {}
    for precision in ("fp32", "split_bf16", "bf16"):
        out = torch.empty((T, n_corr), dtype=torch.float32, device="cuda")
        fmf.matched_filter_device(*g, step, out, "full", True, precision)
        torch.cuda.synchronize()
        rows[precision] = out[:, k0:k0 + K].cpu().numpy().astype(np.float64)
    # the reference's own 'precise' arch (FP32 sums) on the data of these lags
    crop = _crop(d, step, k0, K, L, int(mo.max()))
    rows["reference_precise"] = oracle_built.run_oracle(tp, mo, w, crop, step, "precise", "full",
                                                        True)[:, :K].astype(np.float64)
    stats = {}
    for name, got in rows.items():
        err = np.abs(got - ref)
        stats[name] = (float(err.max()), float(np.quantile(err, 0.999)))
    print("DC offset + full, |cc - FP64| (max, p99.9) on 2 x 200,000 outputs:")
    for name, (mx, q) in stats.items():
        print("  %-18s %.3g  %.3g" % (name, mx, q))
    assert stats["fp32"][0] <= TOL and stats["split_bf16"][0] <= TOL, stats
    assert stats["bf16"][0] > stats["split_bf16"][0]  # the single product loses digits


def test_uneven_batch_at_size_against_the_oracle():
    shapes = synthetic.config3_shapes(seed=103)
    b = fmf.Batch("split_bf16")
    checks = []
    for sh in shapes:
        p = synthetic.config3_problem(sh)
        tp, mo, w, d = p["templates"], p["moveouts"], p["weights"], p["data"]
        T, S, C, L = tp.shape
        N, step = d.shape[-1], p["step"]
        k0, k1 = fp64.valid_range(mo[0].reshape(-1), step, L, N)
        a = max(k0, (k0 + k1) // 2 - 512)
        n = min(1024, k1 - a)
        ref = fp64.fp64_matched_filter(tp, mo, w, d, step, p["normalize"], True,
                                       k_range=(a, a + n), t_index=[0])[0]
        g = _device(tp, mo, w, d)
        out = torch.empty((T, (N - L) // step + 1), dtype=torch.float32, device="cuda")
        b.add(*g, step, out, p["normalize"], True)
        checks.append((g, out, a, n, ref))
        del tp, mo, w, d, p
    assert b.run() > 0
    torch.cuda.synchronize()
    worst = 0.0
    for g, out, a, n, ref in checks:
        got = out[0, a:a + n].cpu().numpy().astype(np.float64)
        worst = max(worst, float(np.abs(got - ref).max()))
    b.close()
    print("64 uneven searches, max |cc - FP64| on the checked windows: %.3g" % worst)
    assert worst <= TOL, worst
