"""The full-day search at its benchmark size (S=20, C=3, N=4,320,000, T=500,
L=600: 8.6 GB of cc_sums) on the GPU, checked through properties that do not
depend on size (needs a GB300):

* no NaN, |cc_sum| <= 1 (weights sum to 1 per template);
* outputs outside each template's valid lag range exactly 0, inside rarely 0;
* FP64 spot checks: windows of lags at the start, middle and end of the valid
  range of several templates against the FP64 oracle, within TOL;
* the two forms agree within TOL everywhere (max over the whole array).
"""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import synthetic
from oracle import fp64
from tests.test_gpu_parity import TOL

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def day():
    cfg = synthetic.config4(seed=104)
    tp, mo, w, d = cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"]
    T, S, C, L = tp.shape
    N = d.shape[-1]
    n_corr = (N - L) + 1
    g = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in
         (tp, np.sum(tp ** 2, axis=-1).astype(np.float32), mo, w, d)]
    outs = {}
    for precision in ("split_bf16", "fp32"):
        out = torch.empty((T, n_corr), dtype=torch.float32, device="cuda")
        fmf.matched_filter_device(*g, 1, out, precision=precision)
        outs[precision] = out
    torch.cuda.synchronize()
    ranges = np.array([fp64.valid_range(mo[t].reshape(-1), 1, L, N) for t in range(T)])
    return cfg, outs, ranges


@pytest.mark.parametrize("precision", ["split_bf16", "fp32"])
def test_fullday_bounds_and_zero_ranges(day, precision):
    cfg, outs, ranges = day
    out = outs[precision]
    assert not torch.isnan(out).any().item()
    assert out.abs().max().item() <= 1.0 + 1e-6
    T, n_corr = out.shape
    k = torch.arange(n_corr, device="cuda")
    lo = torch.from_numpy(ranges[:, 0]).cuda()[:, None]
    hi = torch.from_numpy(ranges[:, 1]).cuda()[:, None]
    inside = (k[None, :] >= lo) & (k[None, :] < hi)
    assert (out[~inside] == 0).all().item()
    zeros_inside = ((out == 0) & inside).sum().item()
    assert zeros_inside < 1e-4 * inside.sum().item()  # zeroed data gaps only


@pytest.mark.parametrize("precision", ["split_bf16", "fp32"])
def test_fullday_fp64_spot_checks(day, precision):
    cfg, outs, ranges = day
    out = outs[precision]
    tp, mo, w, d = cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"]
    worst = 0.0
    for t in (0, 137, 499):
        k0, k1 = (int(v) for v in ranges[t])
        mid = (k0 + k1) // 2
        for a in (k0, mid, k1 - 400):
            ref = fp64.fp64_matched_filter(tp, mo, w, d, 1, "short", True, k_range=(a, a + 400),
                                           t_index=[t])[0]
            got = out[t, a:a + 400].cpu().numpy().astype(np.float64)
            worst = max(worst, float(np.abs(got - ref).max()))
    assert worst <= TOL, worst


def test_fullday_forms_agree(day):
    _, outs, _ = day
    diff = (outs["split_bf16"] - outs["fp32"]).abs().max().item()
    assert diff <= TOL, diff


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_variable_lengths_fullsize_first_template(oracle_built, precision):
    """Per-channel lengths at the benchmark size (S=20, C=3, N=1,080,000, T=100,
    lengths 400-800): the first template's whole row against the oracle (the
    running sums span the whole trace; the first template's scale is its own
    weight sum, as in a search of that template alone)."""
    cfg = synthetic.variable(seed=105)
    tp, mo, w, d, nt = (cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"],
                        cfg["n_samples_template"])
    got = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                             precision=precision)[0]
    ref = oracle_built.run_oracle_variable(tp[:1], nt[:1], mo[:1], w[:1], d, 1)[0]
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.abs(got[ok].astype(np.float64) - ref[ok]).max() <= TOL
