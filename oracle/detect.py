"""Oracle of the detection step (TEST INFRASTRUCTURE ONLY).

A restatement, in numpy and small Python loops, of what
``fast_matched_filter_gb300.detect`` computes per row:

* median / MAD / threshold as numpy computes them on float32 data
  (numpy's ``median``: the middle value, or the float32 mean of the two
  middle values; MAD = median of the float32 ``|x - median|``; threshold =
  ``median + float32(n_mad) * mad`` in float32);
* peaks as ``scipy.signal.find_peaks(x, height=thr, distance=d)``
  (scipy/signal/_peak_finding.py ``find_peaks``; local maxima with flat tops
  from ``_peak_finding_utils._local_maxima_1d``; the distance filter of
  ``_peak_finding_utils._select_by_peak_distance``), with equal heights
  ordered by lag (the later lag is treated as the higher priority, which is
  what scipy does when its priority sort keeps equal keys in lag order).

Pinned against numpy.median and scipy.signal.find_peaks themselves in
tests/test_detect_oracle.py.
"""
import numpy as np


def robust_threshold(x, n_mad):
    """(median, mad, threshold) of a float32 row, as float32 scalars."""
    x = np.asarray(x, dtype=np.float32)
    n = x.size
    if n == 0:
        nan = np.float32(np.nan)
        return nan, nan, nan

    def median(v):
        s = np.sort(v)
        if n % 2:
            return s[n // 2]
        return np.float32(np.float32(s[n // 2 - 1] + s[n // 2]) * np.float32(0.5))

    med = median(x)
    mad = median(np.abs(x - med))
    thr = np.float32(med + np.float32(np.float32(n_mad) * mad))
    return med, mad, thr


def local_maxima(x):
    """Peak positions of scipy's local-maximum rule: x[i-1] < x[i], then a run
    of equal values, then a lower value; the peak is the run's middle (rounded
    down).  The first and last samples are never peaks."""
    x = np.asarray(x)
    n = x.size
    peaks = []
    i = 1
    i_max = n - 1
    while i < i_max:
        if x[i - 1] < x[i]:
            j = i + 1
            while j < i_max and x[j] == x[i]:
                j += 1
            if x[j] < x[i]:
                peaks.append((i + j - 1) // 2)
                i = j
        i += 1
    return np.asarray(peaks, dtype=np.int64)


def distance_filter(peaks, heights, distance):
    """Greedy from the highest peak (equal heights: later lag first): a kept
    peak removes the peaks closer than ``distance`` samples."""
    m = peaks.size
    keep = np.ones(m, dtype=bool)
    order = np.lexsort((peaks, heights))  # ascending height, then ascending lag
    for q in range(m - 1, -1, -1):
        j = order[q]
        if not keep[j]:
            continue
        k = j - 1
        while k >= 0 and peaks[j] - peaks[k] < distance:
            keep[k] = False
            k -= 1
        k = j + 1
        while k < m and peaks[k] - peaks[j] < distance:
            keep[k] = False
            k += 1
    return keep


def detect_row(x, n_mad, min_separation, begin=0, end=None):
    """Detections of one row over the window [begin, end): (median, mad,
    threshold, lags, values) with lags as absolute row indices."""
    x = np.asarray(x, dtype=np.float32)
    end = x.size if end is None else end
    w = x[begin:end]
    med, mad, thr = robust_threshold(w, n_mad)
    pk = local_maxima(w)
    if pk.size:
        pk = pk[w[pk] >= thr]
    keep = distance_filter(pk, w[pk], int(min_separation)) if pk.size else np.zeros(0, bool)
    pk = pk[keep]
    return med, mad, thr, (pk + begin).astype(np.int32), w[pk]


def detect(cc, n_mad, min_separation, lag_begin=None, lag_end=None):
    """All rows of cc (T, n_corr): lists of the detect_row results."""
    cc = np.asarray(cc, dtype=np.float32)
    out = []
    for t in range(cc.shape[0]):
        b = 0 if lag_begin is None else int(lag_begin[t])
        e = cc.shape[1] if lag_end is None else int(lag_end[t])
        out.append(detect_row(cc[t], n_mad, min_separation, b, e))
    return out
