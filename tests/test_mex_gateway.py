"""The MATLAB MEX gateway (fast_matched_filter_gb300/matlab/fmf_gb300_mex.c),
compiled against a test double of the MATLAB C API (tests/mex_mock/) since no
MATLAB is installed: argument checks on the CPU, and on a GB300 the search
through the gateway against the Python front-end.

The gateway takes the reference MEX gateway's twelve arguments
(src/matched_filter_mex.c) plus normalize and precision."""
import ctypes as ct
import os
import shutil
import subprocess

import numpy as np
import pytest

from fast_matched_filter_gb300 import _lib
from tests._cases import random_search

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
MX_DOUBLE, MX_SINGLE, MX_INT32 = 6, 7, 12


@pytest.fixture(scope="module")
def mex(tmp_path_factory):
    if not shutil.which("gcc") or not os.path.exists(_lib.LIB_PATH):
        pytest.skip("needs gcc and the built library")
    out = str(tmp_path_factory.mktemp("mex") / "libfmf_mex_mock.so")
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.check_call(
        ["gcc", "-O2", "-std=c99", "-shared", "-fPIC", "-Wall", "-Werror",
         "-I" + os.path.join(HERE, "mex_mock"), "-I" + os.path.join(REPO, "include"),
         os.path.join(REPO, "fast_matched_filter_gb300", "matlab", "fmf_gb300_mex.c"),
         os.path.join(HERE, "mex_mock", "mock_mx.c"),
         "-L" + libdir, "-lfmf_gb300", "-Wl,-rpath," + libdir, "-o", out])
    lib = ct.CDLL(out)
    lib.mock_array.restype = ct.c_void_p
    lib.mock_array.argtypes = [ct.c_int, ct.c_size_t, ct.c_void_p]
    lib.mock_free.argtypes = [ct.c_void_p]
    lib.mock_call.restype = ct.c_int
    lib.mock_call.argtypes = [ct.c_int, ct.c_int, ct.POINTER(ct.c_void_p), ct.c_void_p, ct.c_size_t,
                              ct.POINTER(ct.c_size_t), ct.c_char_p, ct.c_size_t]
    return lib


def _matlab_args(tp, mo, w, d, step, extra=()):
    """The gateway's arguments as MATLAB would pass them: column-major
    [time x comp x station x template] is the row-major (T, S, C, L) buffer."""
    T, S, C, L = tp.shape
    N = d.shape[-1]
    n_corr = (N - L) // step + 1
    arrays = [(MX_SINGLE, np.ascontiguousarray(tp, np.float32).reshape(-1)),
              (MX_SINGLE, np.sum(tp.astype(np.float32) ** 2, axis=-1).astype(np.float32).reshape(-1)),
              (MX_INT32, np.ascontiguousarray(mo, np.int32).reshape(-1)),
              (MX_SINGLE, np.ascontiguousarray(d, np.float32).reshape(-1)),
              (MX_SINGLE, np.ascontiguousarray(w, np.float32).reshape(-1))]
    scalars = [step, L, N, T, S, C, n_corr] + list(extra)
    arrays += [(MX_DOUBLE, np.array([float(v)])) for v in scalars]
    return arrays, n_corr * T


def _call(mex, arrays, n_out, nlhs=1):
    keep = [a for _, a in arrays]
    handles = [mex.mock_array(cls, a.size, a.ctypes.data) for cls, a in arrays]
    prhs = (ct.c_void_p * len(handles))(*handles)
    out = np.zeros(max(n_out, 1), np.float32)
    n = ct.c_size_t(0)
    msg = ct.create_string_buffer(1024)
    rc = mex.mock_call(nlhs, len(handles), prhs, out.ctypes.data, out.size, ct.byref(n), msg, 1024)
    for h in handles:
        mex.mock_free(h)
    del keep
    return rc, out[:n.value], msg.value.decode()


def _small():
    return random_search(7, 2, 3, 2, 64, 3000, 0, 40)


def test_argument_count_is_checked(mex):
    tp, mo, w, d = _small()
    arrays, n_out = _matlab_args(tp, mo, w, d, 1)
    rc, _, msg = _call(mex, arrays[:11], n_out)
    assert rc == 1 and "12 to 14 inputs" in msg


def test_array_class_is_checked(mex):
    tp, mo, w, d = _small()
    arrays, n_out = _matlab_args(tp, mo, w, d, 1)
    arrays[2] = (MX_DOUBLE, arrays[2][1].astype(np.float64))  # moveouts as double
    rc, _, msg = _call(mex, arrays, n_out)
    assert rc == 1 and "argument 3 must be a real int32 array" in msg


def test_array_size_is_checked(mex):
    tp, mo, w, d = _small()
    arrays, n_out = _matlab_args(tp, mo, w, d, 1)
    arrays[3] = (MX_SINGLE, arrays[3][1][:-5].copy())  # data 5 samples short
    rc, _, msg = _call(mex, arrays, n_out)
    assert rc == 1 and "argument 4 has" in msg


def test_scalar_arguments_are_checked(mex):
    tp, mo, w, d = _small()
    arrays, n_out = _matlab_args(tp, mo, w, d, 1)
    arrays[5] = (MX_DOUBLE, np.array([1.5]))  # step
    rc, _, msg = _call(mex, arrays, n_out)
    assert rc == 1 and "argument 6 must be a non-negative integer" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("normalize,precision,step", [(0, 0, 1), (1, 0, 2), (0, 3, 1)])
def test_gateway_equals_the_python_front_end(mex, normalize, precision, step):
    import fast_matched_filter_gb300 as fmf
    tp, mo, w, d = random_search(8, 3, 3, 2, 200, 20000, 0, 120,
                                 dc=2.0 if normalize else 0.0)
    arrays, n_out = _matlab_args(tp, mo, w, d, step, extra=(normalize, precision))
    rc, got, msg = _call(mex, arrays, n_out)
    assert rc == 0, msg
    name = {0: "fp32", 3: "auto"}[precision]
    ref = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False,
                             normalize="full" if normalize else "short", precision=name)
    got = got.reshape(ref.shape)  # MATLAB: reshape(cc_sum, [], n_templates) is [lags x templates]
    if precision == 0:
        assert np.array_equal(got, ref)
    else:
        assert np.abs(got - ref).max() <= 1e-5
