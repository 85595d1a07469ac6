"""GPU parity of per-channel template lengths (the reference's arch
'variable_precise', matched_filter.c:321-412) against the oracle and the
golden fixtures made by the reference itself (needs a GB300).

Outputs are scaled by the reference's template-cumulative weight sum, so the
bar is TOL relative to that scale."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from tests._cases import canonical, golden_names_variable, load_golden, random_search
from tests.test_gpu_parity import TOL

pytestmark = pytest.mark.gpu


# Tensor-core numerators (split bf16, FP32 accumulation) carry a relative error
# of about 2^-16 per coefficient; the Fisher-z sum passes it through
# atanh, whose slope 1 / (1 - cc^2) grows near |cc| = 1, so their bar is wider.
TOL_TC = 1e-4


def _check(got, ref, scale, tol=TOL):
    assert got.shape == ref.shape
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    err = np.abs(got[ok].astype(np.float64) - ref[ok]).max()
    assert err <= tol * max(1.0, scale), "max |diff| %.3g" % err


def _tol(precision):
    return TOL if precision == "fp32" else TOL_TC


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("name", golden_names_variable())
def test_variable_golden(name, precision):
    inputs, opts, expected = load_golden(name)
    got = fmf.matched_filter(check_zeros=False, arch="variable_precise",
                             normalize=opts["normalize"], precision=precision, **inputs)
    _check(got, expected.reshape(got.shape), float(np.sum(inputs["weights"])), _tol(precision))


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("step", [1, 2, 3])
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_variable_random_vs_oracle(oracle_built, step, normalize, precision):
    rng = np.random.default_rng(60 + step)
    tp, mo, w, d = random_search(70 + step, 3, 3, 2, 160, 8000, -30, 200,
                                 dc=3.0 if normalize == "full" else 0.0, zero_weights=2)
    nt = rng.integers(60, 161, mo.shape).astype(np.int32)
    tp = np.ascontiguousarray(tp[..., :int(nt.max())])
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    got = fmf.matched_filter(tp, mo, w, d, step, n_samples_template=nt, arch="gpu",
                             check_zeros=False, normalize=normalize, precision=precision)
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, step, normalize)
    _check(got, ref, float(np.sum(w)), _tol(precision))


def _bf16(x):
    """Round float32 to bfloat16 (nearest, ties to even), kept as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(
        np.float32).astype(np.float64)


def _split_bf16_shift(tp, nt, mo, w, d, step):
    """What the split-bf16 numerators (t_hi d_hi + t_hi d_lo + t_lo d_hi, the
    lo*lo product dropped) change in each 'short' output, computed in FP64:
    (tanh(sum_ch atanh(cc_split) z / sum z) - the same with exact cc) times
    the template's scale.  Only the valid lags of the reference's
    'variable_precise' range (matched_filter.c:384-385) are non-zero."""
    T, S, C, L = tp.shape
    N = d.shape[-1]
    n_corr = (N - L) // step + 1
    eps = float(np.finfo(np.float32).eps)
    out = np.zeros((T, n_corr))
    scale = np.cumsum(w.reshape(T, -1).astype(np.float64).sum(axis=1))
    for t in range(T):
        lo, hi = min(0, int(mo[t].min())), max(0, int(mo[t].max()))
        start = -(-abs(lo) // step) * step
        ks = np.arange(start, N - L - hi - step, step) // step
        exact, split, zsum = np.zeros(ks.size), np.zeros(ks.size), 0.0
        for s in range(S):
            for c in range(C):
                n, wt = int(nt[t, s, c]), float(w[t, s, c])
                z = np.sqrt(n - 3.0) * wt
                zsum += z
                if wt == 0.0:
                    continue
                tt = tp[t, s, c, :n]
                win = d[s, c][ks[:, None] * step + mo[t, s, c] + np.arange(n)[None, :]]
                th, wh = _bf16(tt), _bf16(win)
                tl, wl = _bf16(tt - th), _bf16(win - wh)
                den = np.sqrt(np.sum(tt.astype(np.float64) ** 2) *
                              np.sum(win.astype(np.float64) ** 2, axis=1))
                for num, acc in ((win @ tt.astype(np.float64), exact),
                                 (wh @ th + wl @ th + wh @ tl, split)):
                    cc = np.where(den > 1e-6, num / den, 0.0)
                    acc += np.arctanh(cc - 10 * eps) * z
        out[t, ks] = (np.tanh(split / zsum) - np.tanh(exact / zsum)) * scale[t]
    return out


@pytest.mark.parametrize("step", [1, 3])
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_variable_tensor_core_short_channels(oracle_built, step, normalize):
    """Channels far shorter than the longest one (down to 4 taps, fewer taps
    than some phases reach): the tensor-core issuers stop each channel's K
    range at its own length, the prefix-sum windows use that length.

    With 4-40 taps many coefficients lie near +-1, where atanh's slope
    1 / (1 - cc^2) reaches ~100: the split-bf16 rounding of the products
    alone then moves outputs by up to ~1e-3 (FP64 emulation).  For 'short'
    the bar is the oracle shifted by that emulated split-bf16 change, within
    TOL_TC; 'full' (centred windows, no coefficient near 1 here) is held to
    TOL_TC against the oracle directly."""
    rng = np.random.default_rng(90 + step)
    tp, mo, w, d = random_search(95 + step, 4, 3, 3, 300, 12000, -50, 150,
                                 dc=2.0 if normalize == "full" else 0.0, zero_weights=3)
    nt = rng.integers(4, 40, mo.shape).astype(np.int32)
    nt[0, 0, 0] = 300
    nt[1] = rng.integers(200, 301, nt[1].shape)
    tp = np.ascontiguousarray(tp[..., :int(nt.max())])
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    got = fmf.matched_filter(tp, mo, w, d, step, n_samples_template=nt, check_zeros=False,
                             normalize=normalize, precision="split_bf16")
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, step, normalize)
    if normalize == "short":
        ref = ref + _split_bf16_shift(tp, nt, mo, w, d, step)
    _check(got, ref, float(np.sum(w)), TOL_TC)


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_variable_full_with_drift(oracle_built, precision):
    """'full' on data whose window means dominate their spread (a DC offset
    and a slow drift 50x the noise): the centred window energies
    S2 - S1^2 / n are formed from the running sums (d^2 exact fixed point, d
    float pairs) in double-float arithmetic and must keep float accuracy
    despite the cancellation."""
    rng = np.random.default_rng(44)
    tp, mo, w, d = random_search(45, 3, 3, 2, 160, 9000, -20, 120, zero_weights=1)
    i = np.arange(d.shape[-1])
    d = (d + 300.0 + 50.0 * np.sin(2 * np.pi * i / 5000.0)).astype(np.float32)
    nt = rng.integers(60, 161, mo.shape).astype(np.int32)
    tp = np.ascontiguousarray(tp[..., :int(nt.max())])
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    got = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                             normalize="full", precision=precision)
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, 1, "full")
    _check(got, ref, float(np.sum(w)), _tol(precision))


def test_variable_equal_lengths_match_fixed_length_coefficients(oracle_built):
    """With every length equal to L the per-channel coefficients are the
    precise ones: atanh/tanh of a single channel recovers its coefficient."""
    tp, mo, w, d = random_search(5, 1, 1, 1, 100, 5000, 0, 0)
    nt = np.full(mo.shape, 100, np.int32)
    got = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False)
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, 1)
    _check(got, ref, 1.0)


def test_fisher_atanh_accuracy():
    """The atanh of the tensor-core Fisher-z epilogue (series for |y| <= 1/4,
    logarithm reduction above) against FP64 atanh: within 4 ulp everywhere in
    (-1, 1), +-inf at +-1, NaN beyond."""
    torch = pytest.importorskip("torch")
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(7)
    y = np.concatenate([
        rng.uniform(-1, 1, 2_000_000), rng.uniform(-0.3, 0.3, 1_000_000),
        1 - np.logspace(-7.2, 0, 100_000), -(1 - np.logspace(-7.2, 0, 100_000)),
        np.logspace(-40, -0.5, 100_000), np.nextafter(np.float32(0.25), np.float32([0, 1])),
        np.float32([0.0, -0.0, 1e-45, 0.25, -0.25])]).astype(np.float32)
    y = y[np.abs(y) < 1]
    dy = torch.from_numpy(y).cuda()
    out = torch.empty_like(dy)
    _lib.check(lib.fmf_eval_atanh(dy.data_ptr(), out.data_ptr(), y.size, None), lib)
    got = out.cpu().numpy().astype(np.float64)
    exact = np.arctanh(y.astype(np.float64))
    ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    err = np.abs(got - exact) / ulp
    assert err.max() <= 4.0, "max %.2f ulp at y=%r" % (err.max(), y[np.argmax(err)])
    special = np.float32([1.0, -1.0, 1.0000001, -1.5, np.nan, np.inf])
    ds = torch.from_numpy(special).cuda()
    os_ = torch.empty_like(ds)
    _lib.check(lib.fmf_eval_atanh(ds.data_ptr(), os_.data_ptr(), special.size, None), lib)
    s = os_.cpu().numpy()
    assert s[0] == np.inf and s[1] == -np.inf and np.isnan(s[2:]).all()


def test_variable_launch_count_per_call():
    """fmf_last_launch_count reports the launches of the last call only
    (the counter restarts at every entry point)."""
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()
    tp, mo, w, d = random_search(12, 2, 2, 2, 80, 4000, 0, 50)
    nt = np.full(mo.shape, 80, np.int32)
    counts = []
    for precision in ("fp32", "fp32", "split_bf16", "split_bf16"):
        fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                           precision=precision)
        counts.append(lib.fmf_last_launch_count())
    assert counts[0] == counts[1] and counts[2] == counts[3], counts
    assert 0 < counts[0] <= 14 and 0 < counts[2] <= 14, counts


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_variable_host_result_in_chunks_equals_device_result(monkeypatch, precision):
    """A result above 64 MB goes to host memory in template chunks whose copies
    overlap the later chunks' kernels; it must equal, bit for bit, the same
    search with device arrays (one launch, no chunks)."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("FMF_TC_PARTS", "1")  # chunking only; channel parts change the sums
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(31)
    T, S, C, L, N = 20, 2, 1, 100, 1_050_000
    tp, mo, w, d = random_search(31, T, S, C, L, N, 0, 80)
    nt = rng.integers(20, L + 1, mo.shape).astype(np.int32)
    nt[0, 0, 0] = L
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    host = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                              precision=precision)
    assert host.nbytes > 64 << 20
    sst = np.sum(tp.astype(np.float32) ** 2, axis=-1).astype(np.float32)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (tp, sst, mo, d, w, nt)]
    out = torch.empty(host.shape, dtype=torch.float32, device="cuda")
    st = lib.fmf_matched_filter_variable_ex(
        dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), dev[3].data_ptr(), dev[4].data_ptr(),
        1, dev[5].data_ptr(), N, T, S, C, host.shape[1], out.data_ptr(), 0,
        _lib.FLAG_DEVICE_POINTERS | _lib.flag_precision(precision), None)
    _lib.check(st, lib)
    torch.cuda.synchronize()
    _lib.check(lib.fmf_device_errors(), lib)
    got = out.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(host))
    ok = ~np.isnan(host)
    assert np.array_equal(got[ok], host[ok])


@pytest.mark.parametrize("normalize", ["short", "full"])
def test_variable_channel_parts(oracle_built, monkeypatch, normalize):
    """A small per-channel-length search runs its tile items as channel parts:
    the parts add raw Fisher-z sums and the transform follows the addition.
    Forced k = 1, 3 and the automatic choice all meet the bar and agree."""
    rng = np.random.default_rng(81)
    tp, mo, w, d = random_search(82, 3, 3, 2, 140, 9000, -20, 120,
                                 dc=2.0 if normalize == "full" else 0.0, zero_weights=2)
    nt = rng.integers(40, 141, mo.shape).astype(np.int32)
    nt[0, 0, 0] = 140
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, 1, normalize)
    got = {}
    for k in ("1", "3", None):
        if k is None:
            monkeypatch.delenv("FMF_TC_PARTS", raising=False)
        else:
            monkeypatch.setenv("FMF_TC_PARTS", k)
        got[k] = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                                    normalize=normalize, precision="split_bf16")
        _check(got[k], ref, float(np.sum(w)), TOL_TC)
    assert np.abs(got["1"] - got["3"]).max() <= 1e-5 * float(np.sum(w))
