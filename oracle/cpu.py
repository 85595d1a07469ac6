"""ctypes front-end of the CPU checker libraries (test infrastructure only).

``run_oracle`` calls ``fmo_matched_filter`` from ``oracle/fmf_oracle.c``.
``run_reference`` calls the reference's own CPU symbols
(``matched_filter``, ``matched_filter_precise``, ``*_no_sum``; prototypes in
fast_matched_filter/src/matched_filter_CPU.h:1-59) from ``oracle/_ref``,
which exists only where the reference sources were available at build time.

Both take canonical arrays -- templates (T,S,C,L), moveouts (T,S,C),
weights (T,S,C), data (S,C,N) -- and return (T,n_corr) or (T,n_corr,S,C)
float32, exactly like the reference wrapper's flattened call
(fast_matched_filter.py:253-321).
"""
import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libfmf_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "matched_filter_CPU.so")

_fp = ct.POINTER(ct.c_float)
_ip = ct.POINTER(ct.c_int)
_sz = ct.c_size_t
# argument list of the reference CPU entry points (fast_matched_filter.py:19-33)
_REF_ARGS = [_fp, _fp, _ip, _fp, _fp, _sz, _sz, _sz, _sz, _sz, _sz, _sz, _fp]

_oracle = None
_ref = None

# Where the reference checkout is read from (its CPU library source, its test
# data): $FMF_REFERENCE_ROOT, else the checkout this build recipe was written
# against.  Where neither exists, only the restatement is built and the tests
# that need the reference skip.
DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_root():
    return os.environ.get("FMF_REFERENCE_ROOT") or DEFAULT_REFERENCE_ROOT


def build(ref_src=None):
    """Compile the restatement (always) and the reference (when its source exists)."""
    subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)
    src = ref_src or os.path.join(reference_root(), "fast_matched_filter", "src",
                                  "matched_filter.c")
    if os.path.exists(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF_SRC=" + src],
                              stdout=subprocess.DEVNULL)


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = ct.CDLL(ORACLE_SO)
        lib.fmo_matched_filter.argtypes = _REF_ARGS + [ct.c_int] * 4
        lib.fmo_matched_filter.restype = ct.c_int
        lib.fmo_cumsum_sq.argtypes = [_fp, _sz, ct.POINTER(ct.c_double)]
        lib.fmo_cumsum_sq.restype = None
        lib.fmo_max_threads.restype = ct.c_int
        lib.fmo_matched_filter_variable.argtypes = [_fp, _fp, _ip, _fp, _fp, _sz, _ip, _sz, _sz, _sz,
                                                    _sz, _sz, _fp, ct.c_int, ct.c_int]
        lib.fmo_matched_filter_variable.restype = ct.c_int
        _oracle = lib
    return _oracle


def reference_available():
    return os.path.exists(REF_SO)


def reference_lib():
    global _ref
    if _ref is None:
        lib = ct.CDLL(REF_SO)
        for name in ("matched_filter", "matched_filter_no_sum"):
            getattr(lib, name).argtypes = _REF_ARGS
            getattr(lib, name).restype = None
        for name in ("matched_filter_precise", "matched_filter_precise_no_sum"):
            getattr(lib, name).argtypes = _REF_ARGS + [ct.c_int]
            getattr(lib, name).restype = None
        lib.matched_filter_variable_precise.argtypes = _REF_ARGS[:6] + [_ip] + _REF_ARGS[7:] + [ct.c_int]
        lib.matched_filter_variable_precise.restype = None
        lib.neumaier_cumsum_squared.argtypes = [_fp, _sz, ct.POINTER(ct.c_double)]
        lib.neumaier_cumsum_squared.restype = None
        _ref = lib
    return _ref


def flatten_inputs(templates, moveouts, weights, data, step):
    """Canonical arrays -> the flat buffers and sizes of the C call.

    Template energies are computed as the reference wrapper does
    (fast_matched_filter.py:256-261): summed in the templates' dtype, then
    cast to float32."""
    T, S, C, L = templates.shape
    N = data.shape[-1]
    n_corr = int((N - L) / step + 1)
    sst = np.ascontiguousarray(np.sum(templates ** 2, axis=-1).ravel(), dtype=np.float32)
    tp = np.ascontiguousarray(templates.ravel(), dtype=np.float32)
    mo = np.ascontiguousarray(np.asarray(moveouts).reshape(T, S, C).ravel(), dtype=np.int32)
    w = np.ascontiguousarray(np.asarray(weights).reshape(T, S, C).ravel(), dtype=np.float32)
    d = np.ascontiguousarray(data.reshape(S, C, N).ravel(), dtype=np.float32)
    return tp, sst, mo, d, w, dict(T=T, S=S, C=C, L=L, N=N, n_corr=n_corr, step=int(step))


def _ptr(a, typ):
    return a.ctypes.data_as(ct.POINTER(typ))


def _out(dims, network_sum):
    n = dims["T"] * dims["n_corr"] * (1 if network_sum else dims["S"] * dims["C"])
    return np.zeros(n, dtype=np.float32)


def _shape(cc, dims, network_sum):
    if network_sum:
        return cc.reshape(dims["T"], dims["n_corr"])
    return cc.reshape(dims["T"], dims["n_corr"], dims["S"], dims["C"])


def run_oracle(templates, moveouts, weights, data, step, arch="cpu",
               normalize="short", network_sum=True, n_threads=0):
    """Oracle restatement.  arch 'cpu' (prefix-sum energy, short only) or
    'precise' (direct sums, short or full)."""
    tp, sst, mo, d, w, dims = flatten_inputs(templates, moveouts, weights, data, step)
    cc = _out(dims, network_sum)
    rc = oracle_lib().fmo_matched_filter(
        _ptr(tp, ct.c_float), _ptr(sst, ct.c_float), _ptr(mo, ct.c_int),
        _ptr(d, ct.c_float), _ptr(w, ct.c_float), dims["step"], dims["L"],
        dims["N"], dims["T"], dims["S"], dims["C"], dims["n_corr"],
        _ptr(cc, ct.c_float), 0 if arch == "cpu" else 1,
        1 if normalize == "full" else 0, int(bool(network_sum)), int(n_threads))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return _shape(cc, dims, network_sum)


def run_reference(templates, moveouts, weights, data, step, arch="cpu",
                  normalize="short", network_sum=True):
    """The reference CPU library itself (oracle/_ref), same calling convention
    as the reference wrapper (fast_matched_filter.py:276-316)."""
    lib = reference_lib()
    tp, sst, mo, d, w, dims = flatten_inputs(templates, moveouts, weights, data, step)
    cc = _out(dims, network_sum)
    args = (_ptr(tp, ct.c_float), _ptr(sst, ct.c_float), _ptr(mo, ct.c_int),
            _ptr(d, ct.c_float), _ptr(w, ct.c_float), dims["step"], dims["L"],
            dims["N"], dims["T"], dims["S"], dims["C"], dims["n_corr"],
            _ptr(cc, ct.c_float))
    if arch == "cpu":
        assert normalize == "short"
        (lib.matched_filter if network_sum else lib.matched_filter_no_sum)(*args)
    else:
        fn = lib.matched_filter_precise if network_sum else lib.matched_filter_precise_no_sum
        fn(*args, 1 if normalize == "full" else 0)
    return _shape(cc, dims, network_sum)


def _variable_args(templates, n_samples_template, moveouts, weights, data, step):
    """Flat buffers of the variable-length call, as the reference wrapper
    builds them (fast_matched_filter.py:216-268): templates (T,S,C,max_len)
    zero-padded, energies over the padded length, n_samples_template int32."""
    tp, sst, mo, d, w, dims = flatten_inputs(templates, moveouts, weights, data, step)
    nt = np.ascontiguousarray(np.asarray(n_samples_template).reshape(-1), dtype=np.int32)
    dims["n_corr"] = int((dims["N"] - int(nt.max())) / step + 1)
    return tp, sst, mo, d, w, nt, dims


def run_oracle_variable(templates, n_samples_template, moveouts, weights, data, step,
                        normalize="short", n_threads=0):
    """Oracle restatement of the per-channel-length Fisher-z search."""
    tp, sst, mo, d, w, nt, dims = _variable_args(templates, n_samples_template, moveouts,
                                                 weights, data, step)
    cc = np.zeros(dims["T"] * dims["n_corr"], dtype=np.float32)
    rc = oracle_lib().fmo_matched_filter_variable(
        _ptr(tp, ct.c_float), _ptr(sst, ct.c_float), _ptr(mo, ct.c_int), _ptr(d, ct.c_float),
        _ptr(w, ct.c_float), dims["step"], _ptr(nt, ct.c_int), dims["N"], dims["T"], dims["S"],
        dims["C"], dims["n_corr"], _ptr(cc, ct.c_float), 1 if normalize == "full" else 0,
        int(n_threads))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return cc.reshape(dims["T"], dims["n_corr"])


def run_reference_variable(templates, n_samples_template, moveouts, weights, data, step,
                           normalize="short"):
    """The reference's matched_filter_variable_precise (oracle/_ref)."""
    tp, sst, mo, d, w, nt, dims = _variable_args(templates, n_samples_template, moveouts,
                                                 weights, data, step)
    cc = np.zeros(dims["T"] * dims["n_corr"], dtype=np.float32)
    reference_lib().matched_filter_variable_precise(
        _ptr(tp, ct.c_float), _ptr(sst, ct.c_float), _ptr(mo, ct.c_int), _ptr(d, ct.c_float),
        _ptr(w, ct.c_float), dims["step"], _ptr(nt, ct.c_int), dims["N"], dims["T"], dims["S"],
        dims["C"], dims["n_corr"], _ptr(cc, ct.c_float), 1 if normalize == "full" else 0)
    return cc.reshape(dims["T"], dims["n_corr"])


def cumsum_sq(x, use_reference=False):
    """Compensated prefix sums of x**2 with a leading zero (length n+1)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros(x.size + 1, dtype=np.float64)
    if use_reference:
        # the reference writes entries 1..n (MF.c:672-675)
        reference_lib().neumaier_cumsum_squared(
            _ptr(x, ct.c_float), x.size, out[1:].ctypes.data_as(ct.POINTER(ct.c_double)))
    else:
        oracle_lib().fmo_cumsum_sq(_ptr(x, ct.c_float), x.size,
                                   out.ctypes.data_as(ct.POINTER(ct.c_double)))
    return out


def max_threads():
    return int(oracle_lib().fmo_max_threads())
