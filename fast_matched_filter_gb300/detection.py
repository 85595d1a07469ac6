"""Detection on network-summed correlation rows, on the GPU.

The reference stops at ``cc_sums`` (fast_matched_filter.py:318-321); its
callers then threshold every template's row and pick the peaks.  This module
does that step in the library, so that only the detections come back to the
host (``fmf_detect`` / ``fmf_matched_filter_detect`` in include/fmf_gb300.h).

Semantics, per template row and lag window (the same as this numpy/scipy code
on a float32 row ``x = cc[t, begin:end]``)::

    med = np.median(x)
    mad = np.median(np.abs(x - med))
    thr = med + np.float32(n_mad) * mad
    peaks, _ = scipy.signal.find_peaks(x, height=thr, distance=min_separation)
    lags = begin + peaks

with one tie rule fixed: among peaks of equal height the later lag is kept
first.  Every row holds at most ``DETECT_CAPACITY`` local maxima at or above
its threshold; a row with more raises ``FMFError`` (raise ``n_mad``).
"""
import ctypes as ct

import numpy as np

from . import _lib, autotune
from .fast_matched_filter import _require_lib, prepare

DETECT_CAPACITY = _lib.DETECT_CAPACITY


class Detections:
    """Per-template robust statistics and peaks.

    median, mad, threshold : (T,) float32
    count : (T,) int32, peaks found per template (may exceed max_detections;
        -1 = more local maxima above the threshold than the capacity, only with
        device arrays)
    lags, values : lists of T arrays, the first min(count, max_detections)
        peaks of each template in lag order (lags are output indices of the row)
    """

    def __init__(self, median, mad, threshold, count, lag_table, value_table):
        self.median = median
        self.mad = mad
        self.threshold = threshold
        self.count = count
        self.lag_table = lag_table
        self.value_table = value_table
        n = np.minimum(np.maximum(count, 0), lag_table.shape[1] if lag_table.ndim == 2 else 0)
        self.lags = [lag_table[t, :n[t]] for t in range(len(count))]
        self.values = [value_table[t, :n[t]] for t in range(len(count))]

    def __len__(self):
        return len(self.count)


def valid_lag_range(moveouts, step, n_samples_template, n_samples_data, n_corr=None):
    """[begin, end) of the output indices each template's search can produce:
    the reference's per-template start and stop (matched_filter.c:53-76), the
    rest of the row being zeros.  moveouts (T, ...) -> two int32 arrays (T,)."""
    mo = np.asarray(moveouts).reshape(np.asarray(moveouts).shape[0], -1).astype(np.int64)
    step = int(step)
    L, N = int(n_samples_template), int(n_samples_data)
    if n_corr is None:
        n_corr = int((N - L) / step + 1)
    lo = np.minimum(mo.min(axis=1), 0)
    hi = np.maximum(mo.max(axis=1), 0)
    first = np.where(lo < 0, (-lo + step - 1) // step, 0)
    last = N - L - hi
    end = np.where(last >= 0, np.minimum(last // step + 1, n_corr), 0)
    begin = np.where(last >= 0, np.minimum(first, end), 0)
    return begin.astype(np.int32), end.astype(np.int32)


def _check_detect_args(n_mad, min_separation, max_detections):
    if not np.isfinite(n_mad):
        raise ValueError("n_mad must be finite")
    if int(min_separation) < 1:
        raise ValueError("min_separation must be at least 1")
    if int(max_detections) < 0:
        raise ValueError("max_detections must be >= 0")


def _host_outputs(T, max_detections):
    return dict(median=np.zeros(T, np.float32), mad=np.zeros(T, np.float32),
                threshold=np.zeros(T, np.float32), count=np.zeros(T, np.int32),
                lags=np.zeros((T, max(int(max_detections), 1)), np.int32),
                values=np.zeros((T, max(int(max_detections), 1)), np.float32))


def _addresses(out):
    return [out[k].ctypes.data for k in ("median", "mad", "threshold", "count", "lags", "values")]


def _finish(out, max_detections):
    m = int(max_detections)
    return Detections(out["median"], out["mad"], out["threshold"], out["count"],
                      out["lags"][:, :m], out["values"][:, :m])


def detect(cc, n_mad=8.0, min_separation=1, max_detections=256, lag_begin=None, lag_end=None,
           stream=None):
    """Robust threshold and peaks of every row of ``cc`` (T, n_corr) float32.

    ``cc`` a numpy array: synchronous, returns ``Detections``.  ``cc`` a torch
    CUDA tensor: every array stays on the device and the call is asynchronous
    on ``stream`` (default: torch's current stream); returns ``Detections``
    whose fields are torch tensors (call ``.cpu()`` after synchronising).
    lag_begin / lag_end (T,) restrict each row to a window (both or neither).
    """
    lib = _require_lib()
    _check_detect_args(n_mad, min_separation, max_detections)
    if (lag_begin is None) != (lag_end is None):
        raise ValueError("give both lag_begin and lag_end, or neither")
    if hasattr(cc, "is_cuda") and cc.is_cuda:
        return _detect_device(lib, cc, n_mad, min_separation, max_detections, lag_begin, lag_end,
                              stream)
    cc = np.asarray(cc)
    if cc.ndim == 1:
        cc = cc[None, :]
    if cc.ndim != 2:
        raise ValueError("cc must be (T, n_corr)")
    cc = np.ascontiguousarray(cc, dtype=np.float32)
    T, n_corr = cc.shape
    b = e = None
    if lag_begin is not None:
        b = np.ascontiguousarray(lag_begin, dtype=np.int32).reshape(T)
        e = np.ascontiguousarray(lag_end, dtype=np.int32).reshape(T)
    out = _host_outputs(T, max_detections)
    st = lib.fmf_detect(cc.ctypes.data, T, n_corr, None if b is None else b.ctypes.data,
                        None if e is None else e.ctypes.data, float(n_mad), int(min_separation),
                        int(max_detections), *_addresses(out), 0, None)
    _lib.check(st, lib)
    return _finish(out, max_detections)


def _detect_device(lib, cc, n_mad, min_separation, max_detections, lag_begin, lag_end, stream):
    import torch  # plumbing only: device memory and streams

    if cc.dim() == 1:
        cc = cc.unsqueeze(0)
    if cc.dtype != torch.float32 or not cc.is_contiguous() or cc.dim() != 2:
        raise ValueError("cc must be a contiguous (T, n_corr) float32 CUDA tensor")
    T, n_corr = cc.shape
    dev = cc.device
    m = max(int(max_detections), 1)
    out = dict(median=torch.empty(T, dtype=torch.float32, device=dev),
               mad=torch.empty(T, dtype=torch.float32, device=dev),
               threshold=torch.empty(T, dtype=torch.float32, device=dev),
               count=torch.empty(T, dtype=torch.int32, device=dev),
               lags=torch.empty((T, m), dtype=torch.int32, device=dev),
               values=torch.empty((T, m), dtype=torch.float32, device=dev))
    b = e = None
    if lag_begin is not None:
        b = torch.as_tensor(lag_begin, dtype=torch.int32, device=dev).contiguous()
        e = torch.as_tensor(lag_end, dtype=torch.int32, device=dev).contiguous()
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    handle = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    st = lib.fmf_detect(cc.data_ptr(), T, n_corr, None if b is None else b.data_ptr(),
                        None if e is None else e.data_ptr(), float(n_mad), int(min_separation),
                        int(max_detections),
                        *[out[k].data_ptr() for k in ("median", "mad", "threshold", "count", "lags",
                                                      "values")],
                        _lib.FLAG_DEVICE_POINTERS, handle)
    _lib.check(st, lib)
    det = Detections.__new__(Detections)
    det.median, det.mad, det.threshold, det.count = (out["median"], out["mad"], out["threshold"],
                                                     out["count"])
    det.lag_table = out["lags"][:, :int(max_detections)]
    det.value_table = out["values"][:, :int(max_detections)]
    det.lags = det.values = None  # ragged lists need the host: use the tables and count
    return det


def matched_filter_detect(templates, moveouts, weights, data, step, normalize="short",
                          n_mad=8.0, min_separation=1, max_detections=256, precision="fp32"):
    """Network-sum search and detection in one call: ``matched_filter``'s
    inputs (any of its formats), then ``detect`` on each template's valid lag
    range.  The (T, n_corr) correlation rows stay on the device; returns
    ``Detections`` (lags are output indices, i.e. sample = lag * step)."""
    assert normalize in ("short", "full"), "Only know short or full normalization methods"
    if precision not in _lib.PRECISIONS:
        raise ValueError("precision must be one of %s" % sorted(_lib.PRECISIONS))
    _check_detect_args(n_mad, min_separation, max_detections)
    lib = _require_lib()
    pp = prepare(templates, moveouts, weights, data, step, normalize, energies="device")
    if pp is None:
        print("Template and data dimensions are not compatible!")
        return None
    T, S, C = pp["T"], pp["S"], pp["C"]
    flags = 0 if precision == "fp32" else autotune.flags_for(pp["L"], pp["step"], S * C, normalize,
                                                              precision)
    out = _host_outputs(T, max_detections)
    st = lib.fmf_matched_filter_detect(
        pp["templates"].ctypes.data, None if pp["sst"] is None else pp["sst"].ctypes.data,
        pp["moveouts"].ctypes.data,
        pp["data"].ctypes.data, pp["weights"].ctypes.data, pp["step"], pp["L"], pp["N"], T, S, C,
        pp["n_corr"], pp["normalize"], _lib.PRECISIONS[precision], float(n_mad),
        int(min_separation), int(max_detections), *_addresses(out), flags, None)
    _lib.check(st, lib)
    return _finish(out, max_detections)
