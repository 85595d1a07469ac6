"""precision='auto' (FMF_PREC_AUTO): the split-bf16 tensor-core form where
its error model allows 1e-5, the plain FP32 form elsewhere -- held to the
suite's 1e-5 bar on the searches where an explicit split-bf16 request needs a
wider one (needs a GB300)."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from oracle import fp64
from tests._cases import canonical, golden_names_fixed, golden_names_variable, load_golden, random_search
from tests.test_gpu_parity import TOL, assert_parity, oracle_of

pytestmark = pytest.mark.gpu


def test_short_single_channel_templates_run_in_fp32(oracle_built):
    """70,000 single-channel templates of 8 taps: a split-bf16 coefficient
    averages nothing there (1.45e-5 seen), so auto runs FP32."""
    rng = np.random.default_rng(1)
    T, L, N = 70000, 8, 64
    tp = rng.standard_normal((T, 1, 1, L)).astype(np.float32)
    d = rng.standard_normal((1, 1, N)).astype(np.float32)
    mo = rng.integers(0, 5, (T, 1, 1)).astype(np.int32)
    w = np.ones((T, 1, 1), np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, precision="auto")
    assert fmf.last_precision() == "fp32"
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 1, "short", True), TOL)


@pytest.mark.parametrize("normalize", ["short", "full"])
def test_many_channel_search_runs_split(oracle_built, normalize):
    tp, mo, w, d = random_search(21, 4, 6, 3, 300, 60000, 0, 150,
                                 dc=2.0 if normalize == "full" else 0.0, zero_weights=2)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize=normalize,
                             precision="auto")
    assert fmf.last_precision() == "split_bf16"
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 1, normalize, True), TOL)


def test_full_with_a_drift_runs_fp32():
    """Window means far from the channel centre (a DC of 300 and a drift of
    50x the noise): every split product is as large as the mean, so auto
    runs FP32; the result holds 1e-5 against FP64."""
    tp, mo, w, d = random_search(22, 3, 4, 3, 200, 40000, 0, 100)
    i = np.arange(d.shape[-1])
    d = (d + 300.0 + 50.0 * np.sin(2 * np.pi * i / 5000.0)).astype(np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize="full",
                             precision="auto")
    assert fmf.last_precision() == "fp32"
    ref = fp64.fp64_matched_filter(tp, mo, w, d, 1, "full", True)
    assert np.abs(got.astype(np.float64) - ref).max() <= TOL


def test_full_with_a_burst_runs_split():
    """A large transient moves a channel's mean but not its median, the
    centre 'full' subtracts: the quiet windows stay small, auto keeps the
    tensor cores, and the result holds 1e-5 against FP64."""
    rng = np.random.default_rng(23)
    tp, mo, w, d = random_search(23, 3, 4, 3, 300, 40000, 0, 100, amp=1e-2)
    d[0, :, 12000:13000] += rng.standard_normal((3, 1000)).astype(np.float32) * 1e3
    d = (d + 5.0).astype(np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize="full",
                             precision="auto")
    assert fmf.last_precision() == "split_bf16"
    ref = fp64.fp64_matched_filter(tp, mo, w, d, 1, "full", True)
    assert np.abs(got.astype(np.float64) - ref).max() <= TOL


@pytest.mark.parametrize("name", golden_names_fixed())
def test_golden_fixtures(name):
    inputs, opts, expected = load_golden(name)
    got = fmf.matched_filter(check_zeros=False, precision="auto", **inputs, **dict(
        normalize=opts["normalize"], network_sum=opts["network_sum"]))
    assert_parity(got, expected.reshape(got.shape), TOL)


def _variable_check(got, ref, w):
    err = np.abs(got.astype(np.float64) - ref).max()
    assert err <= TOL * max(1.0, float(np.sum(w))), err


@pytest.mark.parametrize("name", golden_names_variable())
def test_variable_golden_fixtures(name):
    inputs, opts, expected = load_golden(name)
    got = fmf.matched_filter(check_zeros=False, arch="variable_precise", precision="auto",
                             normalize=opts["normalize"], **inputs)
    _variable_check(got, expected.reshape(got.shape), inputs["weights"])


@pytest.mark.parametrize("normalize", ["short", "full"])
@pytest.mark.parametrize("lengths,expect", [((4, 40), "fp32"), ((400, 600), "split_bf16")])
def test_variable_lengths(oracle_built, normalize, lengths, expect):
    """Per-channel lengths: channels of 4-40 taps run in FP32, channels of
    400-600 taps on the tensor cores; both within 1e-5 (of the output
    scale) of the reference's algorithm."""
    rng = np.random.default_rng(24)
    L = lengths[1]
    tp, mo, w, d = random_search(25, 3, 6, 3, L, 50000, 0, 200,
                                 dc=2.0 if normalize == "full" else 0.0)
    nt = rng.integers(lengths[0], lengths[1] + 1, mo.shape).astype(np.int32)
    nt[0, 0, 0] = L
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    got = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                             normalize=normalize, precision="auto")
    assert fmf.last_precision() == expect
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, 1, normalize)
    _variable_check(got, ref, w)


def test_auto_is_rejected_by_batches():
    with pytest.raises(fmf.FMFError):
        fmf.Batch("auto")


def _random_case(seed):
    """A seeded search drawn over the shapes and value ranges callers meet:
    1-6 templates, 1-8 stations, 1-3 components, 4-700 taps (log-uniform),
    step 1-3, 'short' or 'full', channel amplitudes 1e-3..1e3, DC offsets up
    to 1e3 for 'full', weights normalised to sum 1 with some zero; planted
    copies at amplitudes from 0.05 to exact (scaled by a power of two, where
    the split products' rounding errors share a sign), on the channel's DC."""
    rng = np.random.default_rng(1000 + seed)
    T, S, C = int(rng.integers(1, 7)), int(rng.integers(1, 9)), int(rng.integers(1, 4))
    L = int(np.exp(rng.uniform(np.log(4), np.log(700))))
    step = int(rng.integers(1, 4))
    normalize = "full" if rng.random() < 0.5 else "short"
    N = L + int(rng.integers(2000, 40000))
    amp = 10.0 ** rng.uniform(-3, 3, (S, C, 1))
    dc = np.zeros((S, C, 1))
    if normalize == "full" and rng.random() < 0.5:
        dc = rng.uniform(-1e3, 1e3, (S, C, 1))
    d = rng.standard_normal((S, C, N)) * amp + dc
    tp = rng.standard_normal((T, S, C, L)) * np.hanning(L + 2)[1:-1]
    mo = rng.integers(0, 60, (T, S, C))
    w = rng.uniform(0, 1, (T, S, C))
    w[rng.random((T, S, C)) < 0.15] = 0.0
    w[:, 0, 0] += 0.1  # at least one live channel
    w /= w.sum(axis=(1, 2), keepdims=True)
    for t in range(T):
        k = int(rng.integers(0, max(1, (N - L - 60) // step)))
        scale = 2.0 ** int(rng.integers(-3, 4)) if rng.random() < 0.5 else rng.uniform(0.05, 1.0)
        for s in range(S):
            for c in range(C):
                a = k * step + mo[t, s, c]
                if a + L <= N:
                    if scale >= 0.125 and rng.random() < 0.5:  # an exact copy (on the DC)
                        d[s, c, a:a + L] = dc[s, c, 0] + scale * tp[t, s, c] * amp[s, c, 0]
                    else:
                        d[s, c, a:a + L] += scale * tp[t, s, c] * amp[s, c, 0]
    return (tp.astype(np.float32), mo.astype(np.int32), w.astype(np.float32), d.astype(np.float32),
            step, normalize)


@pytest.mark.parametrize("seed", range(24))
def test_auto_holds_the_bar_on_random_searches(seed):
    """precision='auto' within 1e-5 of FP64 on every output of 24 random
    searches (whichever form it picks)."""
    tp, mo, w, d, step, normalize = _random_case(seed)
    got = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False, normalize=normalize,
                             precision="auto")
    ref = fp64.fp64_matched_filter(tp, mo, w, d, step, normalize, True)
    err = np.abs(got.astype(np.float64) - ref).max()
    assert err <= TOL, "seed %d (%s): max %.3g with %s" % (seed, normalize, err, fmf.last_precision())


def test_full_level_shift_holds_the_bar():
    """A quiet stretch 100 noise-sigmas away from the channel's centre (a level
    shift): every product of a window there carries the offset, so split
    products would err by ~1e-4 and auto runs FP32, whose error grows as
    ~6e-8 x the offset in sigmas (4.6e-6 here); within 1e-5 of FP64."""
    rng = np.random.default_rng(26)
    L, N = 300, 40000
    tp = (rng.standard_normal((2, 1, 1, L)) * np.hanning(L + 2)[1:-1]).astype(np.float32)
    mo = np.zeros((2, 1, 1), np.int32)
    w = np.ones((2, 1, 1), np.float32)
    d = rng.standard_normal((1, 1, N)) * 1e-3 + 5.0
    d[..., 20000:24000] += 0.1
    d[0, 0, 21000:21000 + L] += 3e-3 * tp[0, 0, 0]
    d = d.astype(np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize="full",
                             precision="auto")
    assert fmf.last_precision() == "fp32"
    ref = fp64.fp64_matched_filter(tp, mo, w, d, 1, "full", True)
    assert np.abs(got.astype(np.float64) - ref).max() <= TOL
