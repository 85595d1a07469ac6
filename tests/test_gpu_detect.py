"""GPU detection (fmf_detect, fmf_matched_filter_detect) against the oracle
(needs a GB300).  Bar: median, MAD and threshold equal to numpy's float32
values exactly, the same peak lags and values, the same counts."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import FMFError
from oracle import detect as odet

pytestmark = pytest.mark.gpu


def same_float(a, b):
    return (np.isnan(a) and np.isnan(b)) or a == b


def assert_matches(det, cc, n_mad, sep, max_det, begin=None, end=None):
    ref = odet.detect(cc, n_mad, sep, begin, end)
    for t, (med, mad, thr, lags, vals) in enumerate(ref):
        assert same_float(det.median[t], med), (t, det.median[t], med)
        assert same_float(det.mad[t], mad), (t, det.mad[t], mad)
        assert same_float(det.threshold[t], thr), (t, det.threshold[t], thr)
        assert det.count[t] == lags.size, (t, det.count[t], lags.size)
        k = min(lags.size, max_det)
        assert np.array_equal(det.lags[t], lags[:k]), t
        assert np.array_equal(det.values[t], vals[:k]), t


def cc_rows(seed, T, n, quantise=False):
    rng = np.random.default_rng(seed)
    x = np.stack([np.convolve(rng.standard_normal(n), np.hanning(11), mode="same")
                  for _ in range(T)]) * 0.02
    for t in range(T):  # planted detections
        for p in rng.choice(n - 200, 5, replace=False) + 100:
            x[t, p - 20:p + 21] += 0.3 * np.hanning(41)
    if quantise:  # equal values: ties, flat tops
        x = np.round(x * 512) / 512
    return x.astype(np.float32)


@pytest.mark.parametrize("n", [200000, 200001])
@pytest.mark.parametrize("quantise", [False, True])
def test_detect_matches_oracle(n, quantise):
    cc = cc_rows(n + quantise, 4, n, quantise)
    det = fmf.detect(cc, n_mad=6.0, min_separation=25, max_detections=64)
    assert_matches(det, cc, 6.0, 25, 64)
    assert all(c >= 5 for c in det.count)  # the planted peaks


@pytest.mark.parametrize("sep", [1, 2, 300])
def test_detect_separation(sep):
    cc = cc_rows(11, 3, 50000, quantise=True)
    det = fmf.detect(cc, n_mad=2.0, min_separation=sep, max_detections=5000)
    assert_matches(det, cc, 2.0, sep, 5000)


def test_detect_windows_and_tiny_rows():
    cc = cc_rows(5, 6, 3000)
    begin = np.array([0, 100, 500, 7, 2999, 10], np.int32)
    end = np.array([3000, 2900, 500, 9, 3000, 13], np.int32)  # full, inner, empty, 2, 1, 3
    det = fmf.detect(cc, n_mad=1.0, min_separation=3, max_detections=100,
                     lag_begin=begin, lag_end=end)
    assert_matches(det, cc, 1.0, 3, 100, begin, end)
    assert np.isnan(det.median[2]) and det.count[2] == 0


def test_detect_truncates_to_max_detections():
    cc = cc_rows(9, 2, 40000)
    det = fmf.detect(cc, n_mad=0.5, min_separation=2, max_detections=7)
    assert_matches(det, cc, 0.5, 2, 7)
    assert all(c > 7 for c in det.count)
    assert all(len(l) == 7 for l in det.lags)


def test_detect_capacity_exceeded_is_an_error():
    n = 2 * fmf.detection.DETECT_CAPACITY + 200
    row = np.tile(np.array([0.0, 1.0], np.float32), n // 2)  # a local maximum every 2 samples
    cc = np.stack([row, cc_rows(3, 1, n)[0]])
    with pytest.raises(FMFError) as e:
        fmf.detect(cc, n_mad=-1.0, min_separation=1, max_detections=4)
    assert e.value.status == 6 and "template 0" in str(e.value)


def test_detect_device_arrays_match_host():
    torch = pytest.importorskip("torch")
    cc = cc_rows(21, 3, 120000, quantise=True)
    host = fmf.detect(cc, n_mad=5.0, min_separation=40, max_detections=32)
    dev = fmf.detect(torch.from_numpy(cc).cuda(), n_mad=5.0, min_separation=40, max_detections=32)
    torch.cuda.synchronize()
    assert np.array_equal(dev.count.cpu().numpy(), host.count)
    assert np.array_equal(dev.threshold.cpu().numpy(), host.threshold)
    for t in range(3):
        k = int(host.count[t])
        assert np.array_equal(dev.lag_table[t, :k].cpu().numpy(), host.lags[t])
        assert np.array_equal(dev.value_table[t, :k].cpu().numpy(), host.values[t])
    # capacity overflow on device arrays: count -1, no exception
    n = 2 * fmf.detection.DETECT_CAPACITY + 200
    row = torch.tensor([0.0, 1.0], device="cuda").repeat(n // 2).reshape(1, -1).contiguous()
    d2 = fmf.detect(row, n_mad=-1.0, min_separation=1, max_detections=4)
    torch.cuda.synchronize()
    assert int(d2.count[0]) == -1


def test_detect_many_rows_in_chunks():
    cc = cc_rows(8, 1500, 600)  # more rows than one round of scratch (1024)
    det = fmf.detect(cc, n_mad=3.0, min_separation=10, max_detections=8)
    assert_matches(det, cc, 3.0, 10, 8)


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("normalize,step", [("short", 1), ("full", 2)])
def test_search_and_detect_equals_two_steps(precision, normalize, step):
    from tests._cases import random_search
    tp, mo, w, d = random_search(31, 3, 4, 3, 120, 40000, -30, 200, dc=2.0 if normalize == "full" else 0.0)
    kw = dict(n_mad=5.0, min_separation=50, max_detections=40)
    fused = fmf.matched_filter_detect(tp, mo, w, d, step, normalize=normalize,
                                      precision=precision, **kw)
    cc = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False, normalize=normalize,
                            precision=precision)
    b, e = fmf.valid_lag_range(mo, step, tp.shape[-1], d.shape[-1], cc.shape[1])
    two = fmf.detect(cc, lag_begin=b, lag_end=e, **kw)
    assert np.array_equal(fused.count, two.count)
    assert np.array_equal(fused.threshold, two.threshold)
    assert np.array_equal(fused.median, two.median) and np.array_equal(fused.mad, two.mad)
    for t in range(tp.shape[0]):
        assert np.array_equal(fused.lags[t], two.lags[t])
        assert np.array_equal(fused.values[t], two.values[t])
    assert_matches(two, cc, 5.0, 50, 40, b, e)
    assert all(c >= 1 for c in fused.count)  # planted copies are found


def test_search_and_detect_in_template_chunks(monkeypatch):
    """The fused call processes templates in chunks when their correlation rows
    would not fit its device-memory budget; the result must not depend on it."""
    from tests._cases import random_search
    tp, mo, w, d = random_search(41, 7, 3, 2, 90, 20000, 0, 150)
    kw = dict(n_mad=5.0, min_separation=30, max_detections=16)
    whole = fmf.matched_filter_detect(tp, mo, w, d, 1, **kw)
    n_corr = d.shape[-1] - tp.shape[-1] + 1
    monkeypatch.setenv("FMF_SEARCH_DETECT_CHUNK_BYTES", str(3 * n_corr * 4))  # 3 templates
    chunked = fmf.matched_filter_detect(tp, mo, w, d, 1, **kw)
    assert np.array_equal(whole.count, chunked.count)
    assert np.array_equal(whole.threshold, chunked.threshold)
    for t in range(tp.shape[0]):
        assert np.array_equal(whole.lags[t], chunked.lags[t])
        assert np.array_equal(whole.values[t], chunked.values[t])


def _sampled_rows(n, seed):
    """Rows of n = 8 x 16,384 samples whose values at every 8th position (the
    positions the 16,384-value sample of each row reads) differ from the rest:
    row 0 shifted there (the sample's median window misses the median), row 1
    spread ten-fold there (the median window holds, the MAD window misses),
    row 2 plain (both hold)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((3, n))
    x[0, ::8] += 3.0
    x[1, ::8] *= 10.0
    for t in range(3):
        x[t, rng.choice(n - 200, 4, replace=False) + 100] += 12.0
    return x.astype(np.float32)


@pytest.mark.parametrize("n_mad", [4.0, 8.0])
def test_detect_when_the_sample_windows_miss(n_mad):
    """A median window that misses: median and MAD over the whole row, peaks
    by a pass of their own; a MAD window that misses: the MAD over the whole
    row."""
    cc = _sampled_rows(8 * 16384, 61)
    det = fmf.detect(cc, n_mad=n_mad, min_separation=400, max_detections=4096)
    assert_matches(det, cc, n_mad, 400, 4096)


def test_detect_negative_n_mad():
    """n_mad < 0: the threshold falls with the MAD, so the hot values of the
    one read are bounded with the MAD window's upper end."""
    cc = cc_rows(64, 3, 60000)
    det = fmf.detect(cc, n_mad=-0.5, min_separation=30, max_detections=4096)
    assert_matches(det, cc, -0.5, 30, 4096)


def test_detect_ties_and_constant_rows():
    """A row 40 % zeros (the median's candidates nearly all one key), a constant
    row (MAD 0), and a row of three values (every deviation near the MAD
    undecided until the median is known: the list of such values overflows)."""
    rng = np.random.default_rng(62)
    n = 300000
    x = rng.standard_normal((4, n)).astype(np.float32) * 0.1
    x[0, rng.random(n) < 0.4] = 0.0
    x[1] = 0.25
    x[2] = rng.choice(np.array([-1.0, 0.0, 1.0], np.float32), n) + \
        rng.standard_normal(n).astype(np.float32) * 1e-4
    x[3, rng.random(n) < 0.3] = 0.5
    for t in (0, 2, 3):
        x[t, rng.choice(n - 200, 3, replace=False) + 100] += 5.0
    det = fmf.detect(x, n_mad=30.0, min_separation=1000, max_detections=256)
    assert_matches(det, x, 30.0, 1000, 256)
