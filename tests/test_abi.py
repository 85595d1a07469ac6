"""C-ABI checks that need no GPU: the library loads, exports every symbol
include/fmf_gb300.h declares, and rejects bad arguments with a status code
and a message (the reference exits the process instead,
matched_filter.cu:30-39, 236-242, 286-299)."""
import ctypes as ct
import os
import re

import numpy as np
import pytest

from fast_matched_filter_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "fmf_gb300.h")


def declared_functions():
    """Names of the functions the header exports (declarations marked FMF_API)."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = "\n".join(l for l in src.splitlines() if not l.lstrip().startswith("#"))
    return sorted(set(re.findall(r"FMF_API[^;(]*?\b([A-Za-z_]\w*)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from fast_matched_filter_gb300 import build
    build.build()
    return _lib.load()


def test_header_declares_the_reference_entry_point():
    names = declared_functions()
    assert "matched_filter" in names and "fmf_matched_filter" in names
    assert set(_lib.EXPORTS) <= set(names)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version(lib):
    assert lib.fmf_version().decode().startswith("fmf_gb300")


def _args(T=2, S=2, C=3, L=16, N=200, step=1):
    n_corr = (N - L) // step + 1
    tp = np.ones((T, S, C, L), np.float32)
    sst = np.full((T, S, C), float(L), np.float32)
    mo = np.zeros((T, S, C), np.int32)
    w = np.ones((T, S, C), np.float32)
    d = np.ones((S, C, N), np.float32)
    cc = np.zeros(T * n_corr, np.float32)
    keep = (tp, sst, mo, d, w, cc)
    f = lambda a, t: a.ctypes.data_as(ct.POINTER(t))  # noqa: E731
    args = [f(tp, ct.c_float), f(sst, ct.c_float), f(mo, ct.c_int), f(d, ct.c_float),
            f(w, ct.c_float), step, L, N, T, S, C, n_corr, f(cc, ct.c_float), 0, 1]
    return args, keep


@pytest.mark.parametrize("field,value", [(5, 0), (6, 0), (8, 0), (9, 0), (10, 0), (11, 0),
                                         (6, 500), (11, 10 ** 6), (13, 2)])
def test_bad_arguments_return_status(lib, field, value):
    args, keep = _args()
    args[field] = value
    st = lib.fmf_matched_filter(*args)
    assert st == _lib.FMF_ERR_ARG
    code, msg = _lib.last_error(lib)
    assert code == st and msg


def test_null_pointer_rejected(lib):
    args, keep = _args()
    args[3] = None
    assert lib.fmf_matched_filter(*args) == _lib.FMF_ERR_ARG


def test_misaligned_device_array_rejected(lib):
    """Device arrays are read in place: one off its element alignment is an
    argument error, reported before any device work."""
    args, keep = _args()
    ex = [a if not hasattr(a, "contents") else ct.cast(a, ct.c_void_p).value for a in args]
    ex[3] += 2  # data, 2 bytes off
    st = lib.fmf_matched_filter_ex(*ex, 0, _lib.FLAG_DEVICE_POINTERS, None)
    assert st == _lib.FMF_ERR_ARG
    assert "aligned" in _lib.last_error(lib)[1]


def test_unknown_precision_rejected(lib):
    args, keep = _args()
    ex = [a if not hasattr(a, "contents") else ct.cast(a, ct.c_void_p).value for a in args]
    st = lib.fmf_matched_filter_ex(*ex, 7, 0, None)
    assert st == _lib.FMF_ERR_ARG


def test_precision_flag_matches_header():
    src = open(HEADER).read()
    m = re.search(r"#define FMF_FLAG_PRECISION\(p\) \(\(\(p\) & (\d+)\) << (\d+)\)", src)
    assert m, "FMF_FLAG_PRECISION not found"
    mask, shift = int(m.group(1)), int(m.group(2))
    for name, code in _lib.PRECISIONS.items():
        assert _lib.flag_precision(name) == (code & mask) << shift


def test_variable_precision_field_takes_auto(lib):
    """FMF_FLAG_PRECISION is two bits and each value is a precision; AUTO (3)
    passes the argument checks (here, without a GPU, the call then fails at
    its first CUDA call, never on the precision)."""
    args, keep = _args()
    ex = [a if not hasattr(a, "contents") else ct.cast(a, ct.c_void_p).value for a in args]
    nt = np.full((2, 2, 3), 16, np.int32)
    # (templates, sst, moveouts, data, weights, step, n_samples_template, N, T, S, C, n_corr, cc,
    #  normalize, flags, stream)
    st = lib.fmf_matched_filter_variable_ex(ex[0], ex[1], ex[2], ex[3], ex[4], 1, nt.ctypes.data,
                                            200, 2, 2, 3, 185, ex[12], 0,
                                            _lib.flag_precision("auto"), None)
    assert st != _lib.FMF_ERR_ARG
    assert "precision" not in _lib.last_error(lib)[1]
    assert _lib.PRECISIONS["auto"] == 3 and _lib.flag_precision("auto") == 3 << 24


def test_python_layer_raises_on_status(lib):
    with pytest.raises(_lib.FMFError) as e:
        _lib.check(_lib.FMF_ERR_ARG, lib)
    assert "BAD_ARG" in str(e.value)


def _noalloc(lib):
    f = lib.fmf_matched_filter_noalloc
    f.argtypes = [ct.c_void_p] * 5 + [ct.c_size_t] * 7 + [ct.c_void_p, ct.c_int, ct.c_int,
                                                          ct.c_void_p]
    f.restype = ct.c_int
    return f


def test_noalloc_rejects_misaligned_array_before_device_work(lib):
    """The allocation-free entry point checks element alignment of every array
    before it touches the device, like the device-pointer path of
    fmf_matched_filter_ex."""
    args, keep = _args()
    ex = [a if not hasattr(a, "contents") else ct.cast(a, ct.c_void_p).value for a in args]
    for k in (0, 1, 2, 3, 4, 12):
        bad = list(ex)
        bad[k] += 2
        st = _noalloc(lib)(*bad[:13], 0, 1, None)
        assert st == _lib.FMF_ERR_ARG, k
        assert "aligned" in _lib.last_error(lib)[1]


@pytest.mark.parametrize("T,S,C,L,N", [
    (1, 20, 3, 50, 200000),                 # 48 MB of window energies
    (2 ** 31 - 1, 1, 1, 8, 2 ** 30 - 1),    # products that would wrap unguarded
    (1 << 20, 1 << 11, 1, 1 << 10, 1 << 29),
])
def test_noalloc_rejects_searches_beyond_its_scratch(lib, T, S, C, L, N):
    args, keep = _args()
    ex = [a if not hasattr(a, "contents") else ct.cast(a, ct.c_void_p).value for a in args]
    ex[5:12] = [1, L, N, T, S, C, N - L + 1]
    st = _noalloc(lib)(*ex[:13], 1, 1, None)
    assert st == _lib.FMF_ERR_ARG
    assert "scratch" in _lib.last_error(lib)[1]
