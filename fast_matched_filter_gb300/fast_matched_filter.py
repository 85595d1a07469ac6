"""Python interface of the GB300 matched filter.

``matched_filter`` keeps the reference call
(fast_matched_filter/fast_matched_filter.py:66-362): same arguments, same
input formats (4-D templates, single template, "traces"), the same moveout /
weight broadcasting, n_corr, template energies, output layout and
``check_zeros`` report.  ``arch='gpu'`` runs this package's CUDA library; the
reference's CPU architectures are not part of this package, which reports
them as not loaded exactly as the reference wrapper does when its CPU
library is missing (fast_matched_filter.py:164-177).

One keyword is added: ``precision`` -- 'fp32' (plain FP32 CUDA-core form,
the default and the drop-in), 'split_bf16' (tensor cores, bf16 hi+lo with
three products), 'auto' (split_bf16 where its error model puts the search's
largest error at or below 1e-5, else fp32; ``last_precision()`` tells which)
or 'bf16' (single bf16 product).

``matched_filter_device`` runs the same computation on arrays already
resident on the GPU (torch CUDA tensors), asynchronously on a stream.
"""
import ctypes as ct

import numpy as np

from . import _lib, autotune

CPU_LOADED = False
# The library is loaded by the first call that needs it (or the first read of
# GPU_LOADED), not at import: importing the package for its generators or
# its shape handling maps no native code.
_LIB, _LIB_ERROR = None, "not loaded yet"


def __getattr__(name):
    """GPU_LOADED: whether libfmf_gb300.so loads (the reference's flag,
    fast_matched_filter.py:52-63), evaluated on first use."""
    if name == "GPU_LOADED":
        global _LIB, _LIB_ERROR
        if _LIB is None:
            _LIB, _LIB_ERROR = _lib.try_load()
        return _LIB is not None
    raise AttributeError("module %r has no attribute %r" % (__name__, name))


def _require_lib():
    """The loaded library, loaded on first use.  Raises RuntimeError when it
    cannot be loaded (no CPU fallback)."""
    global _LIB, _LIB_ERROR
    if _LIB is None:
        _LIB, _LIB_ERROR = _lib.try_load()
    if _LIB is None:
        raise RuntimeError(
            "fast_matched_filter_gb300: libfmf_gb300.so is not loadable (%s); "
            "build it with `python -m fast_matched_filter_gb300.build`" % _LIB_ERROR)
    return _LIB


def _broadcast(arr, T, S, C, what):
    """(T,S,C) broadcast rule of fast_matched_filter.py:235-251."""
    arr = np.asarray(arr)
    if arr.shape == (T, S, C):
        return arr
    ratio = (T * S * C) / arr.size
    if ratio == C:
        return np.repeat(arr, C).reshape(T, S, C)
    if ratio == 1.0:
        return arr.reshape(T, S, C)
    raise ValueError("%s of shape %s cannot be broadcast to (%d, %d, %d)"
                     % (what, arr.shape, T, S, C))


def _infer_dims(templates, data):
    """Input-format inference of fast_matched_filter.py:179-214.
    Returns (T, S, C) or None for incompatible dimensions."""
    if templates.ndim > data.ndim:
        T = int(templates.shape[0])
        assert templates.shape[1] == data.shape[0]
        S = int(templates.shape[1])
        if templates.ndim == 4:
            assert templates.shape[2] == data.shape[1]
            return T, S, int(templates.shape[2])
        if templates.ndim == 3:
            return T, S, 1
        return None
    if templates.ndim == data.ndim:
        assert templates.shape[0] == data.shape[0]
        S = int(templates.shape[0])
        if templates.ndim == 3:
            assert templates.shape[1] == data.shape[1]
            return 1, S, int(templates.shape[1])
        if templates.ndim == 2:
            return 1, S, 1
        return None
    return None


def _check_zeros_option(check_zeros):
    """Option check of fast_matched_filter.py:322-327."""
    if (check_zeros is not False) and (check_zeros != "first") and (check_zeros != "all"):
        print("check_zeros should be False, 'first', or 'all'. Set it to "
              "the default value: 'first'")
        check_zeros = "first"
    return check_zeros


def _zero_stop(moveouts_flat, n_corr, step, last_axis):
    """The reference's slice end int(n_corr - max moveout / step) applied to
    the last axis (length last_axis), as Python slicing resolves it."""
    stop = int(n_corr - moveouts_flat.max() / step)
    return len(range(last_axis)[:stop])


def _zero_report(cc, moveouts_flat, weights_flat, n_templates, n_corr, step,
                 network_sum, check_zeros, counts=None):
    """The check_zeros diagnostic of fast_matched_filter.py:322-361, including
    its slicing of the last axis in the per-channel layout.  ``counts``: the
    per-template zero counts already made on the device (else counted here)."""
    check_zeros = _check_zeros_option(check_zeros)
    if not check_zeros:
        return None
    if counts is not None:
        zeros = counts[0:1] if check_zeros == "first" else counts
    else:
        stop = int(n_corr - moveouts_flat.max() / step)
        if check_zeros == "first":
            if network_sum:
                zeros = np.sum(cc[0:1, :stop] == 0.0, axis=-1)
            else:
                zeros = np.sum(cc[0:1, :, :, :stop] == 0.0, axis=(1, 2, 3))
        else:
            zeros = np.sum(cc[..., :stop].reshape(n_templates, -1) == 0.0, axis=-1)
    threshold = 10
    if not network_sum:
        threshold *= np.sum(weights_flat[0, ...] > 0.0)
    for t in range(zeros.shape[0]):
        if zeros[t] > threshold:
            print("{} correlation computations were skipped on the {:d}-th "
                  "template. Can be caused by zeros in data, or too low "
                  "amplitudes (try to increase the gain).".format(zeros[t], t))
    return zeros


def prepare(templates, moveouts, weights, data, step, normalize="short", energies="host"):
    """Shape handling of the reference wrapper: returns the flat float32/int32
    buffers and sizes (fast_matched_filter.py:179-268), or None for
    incompatible dimensions.

    energies='device' leaves the template energies of float32 templates to
    the library (``sst`` None): it computes them on the GPU bit-identically
    to the numpy sum below.  Other dtypes are summed here, in their own dtype,
    as the reference does."""
    dims = _infer_dims(templates, data)
    if dims is None:
        return None
    T, S, C = dims
    L = templates.shape[-1]
    if templates.shape != (T, S, C, L):
        templates = templates.reshape(T, S, C, L)
    N = data.shape[-1]
    if data.shape != (S, C, N):
        data = data.reshape(S, C, N)
    assert np.asarray(moveouts).shape == np.asarray(weights).shape
    moveouts = _broadcast(moveouts, T, S, C, "moveouts")
    weights = _broadcast(weights, T, S, C, "weights")
    step = int(step)
    if step < 1:
        raise ValueError("step must be a positive integer, got %d" % step)
    if N < L:
        raise ValueError("data (%d samples) shorter than the templates (%d)" % (N, L))
    n_corr = int((N - L) / step + 1)
    if energies == "device" and templates.dtype == np.float32:
        sst = None
    else:
        sst = np.ascontiguousarray(np.sum(templates ** 2, axis=-1).flatten(), dtype=np.float32)
    # flat C-order buffers, as the reference's .flatten() makes them, but views
    # (no copy) of inputs that are already C-contiguous in the right dtype
    return dict(
        templates=np.ascontiguousarray(templates, dtype=np.float32).reshape(-1),
        sst=sst,
        moveouts=np.ascontiguousarray(moveouts, dtype=np.int32).reshape(-1),
        weights=np.ascontiguousarray(weights, dtype=np.float32).reshape(-1),
        data=np.ascontiguousarray(data, dtype=np.float32).reshape(-1),
        T=T, S=S, C=C, L=int(L), N=int(N), step=step, n_corr=n_corr,
        normalize=1 if normalize == "full" else 0)


def _ptr(a, typ):
    return None if a is None else a.ctypes.data_as(ct.POINTER(typ))


def _addr(a):
    return None if a is None else a.ctypes.data


def matched_filter(templates, moveouts, weights, data, step,
                   n_samples_template=None, arch="gpu", check_zeros="first",
                   normalize="short", network_sum=True, precision="fp32", out=None):
    """Correlation coefficients between ``templates`` and ``data``
    (reference: fast_matched_filter.py:66-362).

    templates : (T, S, C, L), (T, traces, L) or single-template (S, C, L) /
        (traces, L) float array.
    moveouts, weights : (T, S, C) or (T, S) arrays (broadcast over C).
    data : (S, C, N) or (traces, N).
    step : output decimation, in samples.
    arch : 'gpu' (this package); 'cpu', 'precise' and 'variable_precise' are
        the reference's CPU libraries and are reported as not loaded.
    normalize : 'short' or 'full' (window mean removed).
    network_sum : True -> (T, n_corr) weighted sums; False -> (T, n_corr, S, C).
    precision : 'fp32' | 'split_bf16' | 'auto' | 'bf16' (numerator arithmetic;
        'auto' picks split_bf16 or fp32 per call, see ``last_precision``).
    out : optional writable, C-contiguous float32 array of the output's shape;
        every element is written and ``out`` is returned.  Reusing one array
        (or a page-locked one) across calls saves allocating and faulting in
        a fresh output per call.
    """
    assert normalize in ("short", "full"), "Only know short or full normalization methods"
    if normalize == "full":
        assert arch != "cpu", "Full normalization not supported with cpu arch - try arch=precise"
    if n_samples_template is not None or arch.lower() == "variable_precise":
        if arch.lower() not in ("gpu", "variable_precise"):
            print("Compiled library for {} not loaded; exiting!".format(arch))
            return None
        return _matched_filter_variable(templates, moveouts, weights, data, step,
                                        n_samples_template, check_zeros, normalize,
                                        network_sum, precision, out)
    if arch.lower() != "gpu":
        print("Compiled library for {} not loaded; exiting!".format(arch))
        return None
    if precision not in _lib.PRECISIONS:
        raise ValueError("precision must be one of %s" % sorted(_lib.PRECISIONS))
    lib = _require_lib()
    pp = prepare(templates, moveouts, weights, data, step, normalize, energies="device")
    if pp is None:
        print("Template and data dimensions are not compatible!")
        return None
    T, S, C, n_corr = pp["T"], pp["S"], pp["C"], pp["n_corr"]
    cc = _output_array(out, (T, n_corr) if network_sum else (T, n_corr, S, C))
    args = (_ptr(pp["templates"], ct.c_float), _ptr(pp["sst"], ct.c_float),
            _ptr(pp["moveouts"], ct.c_int), _ptr(pp["data"], ct.c_float),
            _ptr(pp["weights"], ct.c_float), pp["step"], pp["L"], pp["N"], T, S, C,
            n_corr, _ptr(cc, ct.c_float), pp["normalize"], int(bool(network_sum)))
    check_zeros = _check_zeros_option(check_zeros)
    flags = 0 if precision == "fp32" else autotune.flags_for(pp["L"], pp["step"], S * C, normalize,
                                                              precision)
    ex = (pp["templates"].ctypes.data, _addr(pp["sst"]), pp["moveouts"].ctypes.data,
          pp["data"].ctypes.data, pp["weights"].ctypes.data, pp["step"], pp["L"], pp["N"],
          T, S, C, n_corr, cc.ctypes.data, pp["normalize"], int(bool(network_sum)),
          _lib.PRECISIONS[precision], flags, None)
    counts = None
    if check_zeros:  # counted on the device before the copy out
        counts = np.zeros(T, dtype=np.uint64)
        stop = _zero_stop(pp["moveouts"], n_corr, pp["step"], n_corr if network_sum else C)
        st = lib.fmf_matched_filter_check_zeros(*ex, stop, counts.ctypes.data)
    elif precision == "fp32":
        st = lib.fmf_matched_filter(*args)
    else:
        st = lib.fmf_matched_filter_ex(*ex)
    _lib.check(st, lib)
    cc = cc.reshape(T, n_corr) if network_sum else cc.reshape(T, n_corr, S, C)
    _zero_report(cc, pp["moveouts"], pp["weights"], T, n_corr, pp["step"],
                 network_sum, check_zeros, counts)
    return cc if out is None else out


def last_precision():
    """The numerator precision ('fp32', 'split_bf16' or 'bf16') of the last
    search this thread ran; with precision='auto', the one chosen."""
    return _lib.PRECISION_NAMES.get(_require_lib().fmf_last_precision())


def _output_array(out, shape):
    """The flat float32 output: a new array (the library writes every element,
    so it is not zeroed first, and maps its pages on several threads while the
    GPU computes), or a view of ``out`` after checking that the library may
    write it in place."""
    if out is None:
        return np.empty(int(np.prod(shape)), dtype=np.float32)
    if not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.flags.c_contiguous
            and out.flags.writeable and out.shape == tuple(shape)):
        raise ValueError("out must be a writable C-contiguous float32 array of shape %s"
                         % (tuple(shape),))
    return out.reshape(-1)


def _matched_filter_variable(templates, moveouts, weights, data, step, n_samples_template,
                             check_zeros, normalize, network_sum, precision="fp32", out=None):
    """Per-channel template lengths (the reference's arch 'variable_precise',
    fast_matched_filter.py:216-229, 307-313) on the GPU library; ``precision``
    selects the plain FP32 or the tensor-core numerators."""
    if precision not in _lib.PRECISIONS:
        raise ValueError("precision must be one of %s" % sorted(_lib.PRECISIONS))
    if n_samples_template is None:
        raise ValueError("arch='variable_precise' needs n_samples_template")
    if not network_sum:
        raise NotImplementedError("Variable precise without network sum is not yet implemented.")
    lib = _require_lib()
    n_samples_template = np.asarray(n_samples_template)
    assert n_samples_template.shape == np.asarray(moveouts).shape
    max_len = int(np.max(n_samples_template))
    dims = _infer_dims(templates, data)
    if dims is None:
        print("Template and data dimensions are not compatible!")
        return None
    T, S, C = dims
    templates = templates.reshape(T, S, C, max_len)
    pp = prepare(templates, moveouts, weights, data, step, normalize)
    n_corr = int((pp["N"] - max_len) / pp["step"] + 1)
    nt = np.ascontiguousarray(n_samples_template.flatten(), dtype=np.int32)
    cc = _output_array(out, (T, n_corr))
    st = lib.fmf_matched_filter_variable_ex(
        pp["templates"].ctypes.data, pp["sst"].ctypes.data, pp["moveouts"].ctypes.data,
        pp["data"].ctypes.data, pp["weights"].ctypes.data, pp["step"], nt.ctypes.data,
        pp["N"], T, S, C, n_corr, cc.ctypes.data, pp["normalize"], _lib.flag_precision(precision),
        None)
    _lib.check(st, lib)
    cc = cc.reshape(T, n_corr)
    _zero_report(cc, pp["moveouts"], pp["weights"], T, n_corr, pp["step"], True, check_zeros)
    return cc if out is None else out


def matched_filter_device(templates, sum_square_templates, moveouts, weights, data,
                          step, out, normalize="short", network_sum=True,
                          precision="fp32", stream=None):
    """Run on device-resident, canonical, C-contiguous torch CUDA tensors:
    templates (T,S,C,L) f32, sum_square_templates (T,S,C) f32 or None (then
    computed on the GPU as numpy.sum(templates**2, axis=-1) would), moveouts
    (T,S,C) int32, weights (T,S,C) f32, data (S,C,N) f32, out (T,n_corr) or
    (T,n_corr,S,C) f32.  Asynchronous on ``stream`` (a torch.cuda.Stream or
    raw handle; default: torch's current stream).  Returns the launch count."""
    import torch  # plumbing only: device memory and streams

    lib = _require_lib()
    T, S, C, L = templates.shape
    N = data.shape[-1]
    n_corr = out.shape[1]
    for name, t, dt in (("templates", templates, torch.float32),
                        ("sum_square_templates", sum_square_templates, torch.float32),
                        ("moveouts", moveouts, torch.int32), ("weights", weights, torch.float32),
                        ("data", data, torch.float32), ("out", out, torch.float32)):
        if t is None and name == "sum_square_templates":
            continue
        if not (t.is_cuda and t.dtype == dt and t.is_contiguous()):
            raise ValueError("%s must be a contiguous CUDA tensor of %s" % (name, dt))
    if stream is None:
        stream = torch.cuda.current_stream()
    handle = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    flags = _lib.FLAG_DEVICE_POINTERS | autotune.flags_for(L, step, S * C, normalize, precision)
    st = lib.fmf_matched_filter_ex(
        templates.data_ptr(),
        None if sum_square_templates is None else sum_square_templates.data_ptr(),
        moveouts.data_ptr(), data.data_ptr(), weights.data_ptr(), int(step), L, N, T, S, C, n_corr,
        out.data_ptr(), 1 if normalize == "full" else 0, int(bool(network_sum)),
        _lib.PRECISIONS[precision], flags, handle)
    _lib.check(st, lib)
    return lib.fmf_last_launch_count()


def test_matched_filter(n_templates=1, n_stations=1, n_components=1,
                        template_duration=10, data_duration=86400,
                        sampling_rate=100, step=1, arch="gpu",
                        check_zeros="first", normalize="short",
                        network_sum=True, precision="fp32"):
    """Synthetic self-test of the reference (fast_matched_filter.py:365-569):
    uniform-noise data (mean removed per channel), templates cut from the data
    at random times with random moveouts of 0-10 s, unit weights, so that the
    maximum coefficient of every template is 1.  Returns (templates,
    moveouts, data, step, cc_sums, run_time); with arch='variable_precise'
    every station of every template keeps a random length of 1/2 to 1 times
    the template duration (fast_matched_filter.py:512-531), and the returned
    tuple carries those lengths before run_time (as the reference's,
    fast_matched_filter.py:566-567)."""
    from time import time as clock

    starts = np.random.random_sample(n_templates) * (data_duration / 2)
    if step != 1:
        starts = np.round(starts / (step / sampling_rate)) * (step / sampling_rate)
    moveouts = np.zeros((n_templates, n_stations, n_components))
    for t in range(n_templates):
        for s in range(n_stations):
            moveouts[t, s, :] = np.random.random_sample(n_components) * 10.0
    moveouts = np.int32(np.round(moveouts * sampling_rate))
    n_data = data_duration * sampling_rate
    if float(int(n_data)) != float(n_data):
        print("The data duration times the sampling rate yields a non-integer number of samples !")
        return None
    n_data = int(n_data)
    data = np.random.random_sample((n_stations, n_components, n_data)).astype("float32")
    data -= data.mean(axis=-1, keepdims=True)
    n_tp = template_duration * sampling_rate
    if float(int(n_tp)) != float(n_tp):
        print("The template duration times the sampling rate yields a non-integer number of samples !")
        return None
    n_tp = int(n_tp)
    templates = np.zeros((n_templates, n_stations, n_components, n_tp), dtype=np.float32)
    for t in range(n_templates):
        first = starts[t] * sampling_rate
        for s in range(n_stations):
            for c in range(n_components):
                a = int(first + moveouts[t, s, c])
                templates[t, s, c, :] = data[s, c, a:a + n_tp]
    weights = np.ones((n_templates, n_stations, n_components), dtype=np.float32)
    lengths = None
    if arch == "variable_precise":
        lengths = np.zeros(moveouts.shape, dtype=np.int32)
        for t in range(n_templates):
            for s in range(n_stations):
                lengths[t, s, :] = np.int32(np.round(np.random.random_sample() * n_tp / 2
                                                     + n_tp / 2))
        templates = templates[:, :, :, :np.max(lengths)]
        for idx in np.ndindex(lengths.shape):
            templates[idx][lengths[idx]:] = 0.0
    t0 = clock()
    cc_sum = matched_filter(templates, moveouts, weights, data, step, arch=arch,
                            n_samples_template=lengths, check_zeros=check_zeros,
                            normalize=normalize, network_sum=network_sum, precision=precision)
    run_time = clock() - t0
    print("Matched filter ({}) for {} templates on {} stations/{} components over "
          "{} samples ({} step) ran in {:.3f}s".format(
              arch, n_templates, n_stations, n_components, n_data, step, run_time))
    if lengths is not None:
        return templates, moveouts, data, step, cc_sum, lengths, run_time
    return templates, moveouts, data, step, cc_sum, run_time


class Batch:
    """Many independent searches run as one CUDA graph (C ABI fmf_batch_*).

    ``add`` takes canonical, contiguous torch CUDA tensors (as
    ``matched_filter_device``) and keeps references to them; ``run`` launches
    every search asynchronously on ``stream`` -- preprocessing, then one
    persistent tensor-core launch over a shared tile queue (or the plain
    kernel per search for precision='fp32').  The graph is captured on the
    first ``run`` after the last ``add`` and replayed afterwards.
    """

    def __init__(self, precision="split_bf16", lag_blocks=0, template_group=0):
        self._lib = _require_lib()
        self._h = ct.c_void_p()
        _lib.check(self._lib.fmf_batch_create(ct.byref(self._h), _lib.PRECISIONS[precision]),
                   self._lib)
        self._keep = []
        if lag_blocks or template_group:
            _lib.check(self._lib.fmf_batch_set_tiles(self._h, lag_blocks, template_group), self._lib)

    def add(self, templates, sum_square_templates, moveouts, weights, data, step, out,
            normalize="short", network_sum=True):
        T, S, C, L = templates.shape
        N = data.shape[-1]
        st = self._lib.fmf_batch_add(
            self._h, templates.data_ptr(), sum_square_templates.data_ptr(), moveouts.data_ptr(),
            data.data_ptr(), weights.data_ptr(), int(step), L, N, T, S, C, out.shape[1],
            out.data_ptr(), 1 if normalize == "full" else 0, int(bool(network_sum)))
        _lib.check(st, self._lib)
        self._keep.append((templates, sum_square_templates, moveouts, weights, data, out))

    def run(self, stream=None):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream()
        handle = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        _lib.check(self._lib.fmf_batch_run(self._h, handle), self._lib)
        return self._lib.fmf_batch_launch_count(self._h)

    def close(self):
        if self._h:
            self._lib.fmf_batch_destroy(self._h)
            self._h = ct.c_void_p()
            self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
