"""Allocation-free entry point fmf_matched_filter_noalloc (needs a GB300).

Some callers cannot allocate device memory while they run: a real-time
detection loop that reserved its memory at start-up and must keep
cudaMalloc/cudaFree (which can synchronise the device) out of its processing
path, or a host application that owns the GPU's memory budget.  For them the
library offers an entry point whose working arrays live in one file-scope
device array.  This file checks, through the C ABI, that it gives the regular
entry point's results within the suite's tolerance on two calls in a row
(sharing that array), that it leaves free device memory unchanged, and that
it rejects a search larger than the array.  The file name makes pytest
collect it last.
"""
import ctypes as ct

import numpy as np
import pytest

from fast_matched_filter_gb300 import _lib
from tests._cases import random_search

TOL = 1e-5
pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _bind():
    lib = ct.CDLL(_lib.LIB_PATH)
    lib.fmf_matched_filter_noalloc.argtypes = [ct.c_void_p] * 5 + [ct.c_size_t] * 7 + [
        ct.c_void_p, ct.c_int, ct.c_int, ct.c_void_p]
    lib.fmf_matched_filter_noalloc.restype = ct.c_int
    lib.fmf_matched_filter_ex.argtypes = _lib.ARGTYPES_EX
    lib.fmf_matched_filter_ex.restype = ct.c_int
    lib.fmf_last_error.argtypes = [ct.c_char_p, ct.c_size_t]
    lib.fmf_last_error.restype = ct.c_int
    return lib


def _search(seed, T, S, C, L, N, step, normalize, network_sum):
    tp, mo, w, d = random_search(seed, T, S, C, L, N, -25, 150,
                                 dc=3.0 if normalize == "full" else 0.0, zero_weights=1)
    dev = torch.device("cuda")
    n_corr = (N - L) // step + 1
    shape = (T, n_corr) if network_sum else (T, n_corr, S, C)
    g = dict(tp=torch.from_numpy(tp).to(dev),
             sst=torch.from_numpy(np.sum(tp ** 2, axis=-1).astype(np.float32)).to(dev),
             mo=torch.from_numpy(mo).to(dev), d=torch.from_numpy(d).to(dev),
             w=torch.from_numpy(w).to(dev))
    args = (g["tp"].data_ptr(), g["sst"].data_ptr(), g["mo"].data_ptr(), g["d"].data_ptr(),
            g["w"].data_ptr(), step, L, N, T, S, C, n_corr)
    flags = (1 if normalize == "full" else 0, int(network_sum))
    return g, args, flags, shape


def _regular(lib, args, flags, shape):
    out = torch.full(shape, 7.0, dtype=torch.float32, device="cuda")
    st = lib.fmf_matched_filter_ex(*args, out.data_ptr(), *flags, _lib.PREC_FP32,
                                   _lib.FLAG_DEVICE_POINTERS, torch.cuda.current_stream().cuda_stream)
    assert st == 0, _lib.last_error(lib)
    return out


def _noalloc(lib, args, flags, shape):
    out = torch.full(shape, 7.0, dtype=torch.float32, device="cuda")
    st = lib.fmf_matched_filter_noalloc(*args, out.data_ptr(), *flags,
                                        torch.cuda.current_stream().cuda_stream)
    assert st == 0, _lib.last_error(lib)
    return out


def test_two_calls_in_a_row_match_the_regular_entry_point():
    lib = _bind()
    a = _search(1, 3, 4, 3, 120, 30000, 1, "short", True)
    b = _search(2, 2, 3, 2, 200, 20000, 2, "full", False)
    ref_a = _regular(lib, *a[1:]).cpu().numpy()
    ref_b = _regular(lib, *b[1:]).cpu().numpy()
    torch.cuda.synchronize()
    _noalloc(lib, *a[1:])  # first call on this device: looks up the scratch address
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    got_a = _noalloc(lib, *a[1:])
    got_b = _noalloc(lib, *b[1:])  # second call in a row reuses the same scratch
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    for got, ref in ((got_a.cpu().numpy(), ref_a), (got_b.cpu().numpy(), ref_b)):
        assert got.shape == ref.shape
        assert np.array_equal(got == 0.0, ref == 0.0)
        assert np.abs(got.astype(np.float64) - ref).max() <= TOL
    assert free1 == free0
    assert lib.fmf_device_errors() == 0


def test_search_larger_than_the_scratch_array_is_rejected():
    lib = _bind()
    # 4 * S*C*N = 4 * 60 * 200000 bytes of window energies > 32 MiB
    g, args, flags, shape = _search(3, 1, 20, 3, 50, 200000, 1, "short", True)
    out = torch.zeros(shape, dtype=torch.float32, device="cuda")
    st = lib.fmf_matched_filter_noalloc(*args, out.data_ptr(), *flags,
                                        torch.cuda.current_stream().cuda_stream)
    assert st == _lib.FMF_ERR_ARG
    code, msg = _lib.last_error(lib)
    assert code == st and "scratch" in msg
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0
