"""Pinning of the detection oracle (CPU, no GPU needed).

The detection step has no reference counterpart; its definition is numpy's
median and scipy's find_peaks, so the oracle (oracle/detect.py) is pinned
against those two libraries themselves.  Also: the valid-lag-range helper of
the product package against the oracle's restatement of the reference's
start/stop rule, and the argument checks of fmf_detect (no GPU touched).
"""
import ctypes as ct

import numpy as np
import pytest

from oracle import detect as odet

signal = pytest.importorskip("scipy.signal")


def rows(seed, n, kind):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n)
    if kind == "smooth":
        x = np.convolve(x, np.hanning(15), mode="same")
    elif kind == "quantised":  # many equal values: ties and flat tops
        x = np.round(np.convolve(x, np.hanning(9), mode="same") * 8) / 8
    elif kind == "spiky":
        x = 0.05 * x
        k = min(40, n)
        idx = rng.choice(n, k, replace=False)
        x[idx] += rng.uniform(0.3, 1.0, k)
    return x.astype(np.float32)


@pytest.mark.parametrize("n", [1, 2, 3, 10, 11, 4096, 4097, 100000])
@pytest.mark.parametrize("kind", ["smooth", "quantised", "spiky"])
def test_threshold_matches_numpy(n, kind):
    x = rows(n, n, kind)
    med, mad, thr = odet.robust_threshold(x, 6.5)
    ref_med = np.median(x)
    ref_mad = np.median(np.abs(x - ref_med))
    ref_thr = ref_med + np.float32(6.5) * ref_mad
    assert med.dtype == np.float32 and ref_med.dtype == np.float32
    assert med == ref_med and mad == ref_mad and thr == ref_thr
    assert ref_thr.dtype == np.float32


def test_threshold_of_empty_row_is_nan():
    med, mad, thr = odet.robust_threshold(np.zeros(0, np.float32), 3.0)
    assert np.isnan(med) and np.isnan(mad) and np.isnan(thr)


@pytest.mark.parametrize("distance", [1, 2, 7, 50, 400])
@pytest.mark.parametrize("kind", ["smooth", "spiky"])
def test_peaks_match_scipy(distance, kind):
    x = rows(100 + distance, 50000, kind)
    # rank transform: same peaks, every value distinct (scipy's tie order is then moot)
    x = np.argsort(np.argsort(x)).astype(np.float32) / np.float32(x.size)
    med, mad, thr = odet.robust_threshold(x, 1.0)  # ranks: threshold near the top quarter
    ref, _ = signal.find_peaks(x, height=thr, distance=distance)
    assert ref.size >= 10
    _, _, _, lags, vals = odet.detect_row(x, 1.0, distance)
    assert np.array_equal(lags, ref)
    assert np.array_equal(vals, x[ref])


def test_flat_tops_match_scipy():
    x = np.array([0, 1, 1, 1, 0, 2, 2, 0, 3, 3, 3, 3, 4, 1, 5, 5], np.float32)
    ref, _ = signal.find_peaks(x)
    assert np.array_equal(odet.local_maxima(x), ref)  # [2, 5, 12]; the last flat top is open
    assert list(ref) == [2, 5, 12]


def test_equal_heights_keep_the_later_lag():
    x = np.zeros(40, np.float32)
    x[10] = x[14] = 1.0  # equal peaks 4 apart
    _, _, _, lags, _ = odet.detect_row(x, 0.0, 5)
    assert list(lags) == [14]


def test_window_offsets_lags():
    x = rows(7, 3000, "spiky")
    _, _, _, lags, _ = odet.detect_row(x, 3.0, 10, 500, 2500)
    _, _, _, lags2, _ = odet.detect_row(x[500:2500], 3.0, 10)
    assert np.array_equal(lags, lags2 + 500)


def test_valid_lag_range_matches_reference_rule():
    from fast_matched_filter_gb300 import valid_lag_range
    from oracle.fp64 import valid_range
    rng = np.random.default_rng(3)
    for step in (1, 2, 3, 7):
        mo = rng.integers(-60, 200, (50, 4, 3))
        mo[0] = 5000  # nothing valid
        mo[1] = -5000  # nothing valid
        L, N = 40, 1000
        n_corr = int((N - L) / step + 1)
        b, e = valid_lag_range(mo, step, L, N, n_corr)
        for t in range(mo.shape[0]):
            k0, k1 = valid_range(mo[t].ravel(), step, L, N)
            if k1 <= k0:
                assert e[t] <= b[t] or e[t] == b[t]
            else:
                assert (b[t], e[t]) == (k0, min(k1, n_corr))


def test_detect_rejects_bad_arguments():
    from fast_matched_filter_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    cc = np.zeros((2, 100), np.float32)
    cnt = np.zeros(2, np.int32)
    lags = np.zeros((2, 4), np.int32)
    vals = np.zeros((2, 4), np.float32)
    outs = [None, None, None, cnt.ctypes.data, lags.ctypes.data, vals.ctypes.data]
    call = lambda T, n, ms, nmad=3.0, b=None, e=None, o=outs: lib.fmf_detect(  # noqa: E731
        cc.ctypes.data, T, n, b, e, nmad, ms, 4, *o, 0, None)
    assert call(0, 100, 1) == _lib.FMF_ERR_ARG
    assert call(2, 100, 0) == _lib.FMF_ERR_ARG
    assert call(2, 100, 1, nmad=float("nan")) == _lib.FMF_ERR_ARG
    assert call(2, 100, 1, o=[None, None, None, None, lags.ctypes.data, vals.ctypes.data]) == \
        _lib.FMF_ERR_ARG
    b = np.array([0, 50], np.int32)
    e = np.array([100, 101], np.int32)
    assert call(2, 100, 1, b=b.ctypes.data, e=e.ctypes.data) == _lib.FMF_ERR_ARG
    assert call(2, 100, 1, b=b.ctypes.data, e=None) == _lib.FMF_ERR_ARG
    st, msg = _lib.last_error(lib)
    assert st == _lib.FMF_ERR_ARG and "lag_begin" in msg
