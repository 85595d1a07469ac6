"""Allocation-free entry point fmf_matched_filter_noalloc (needs a GB300).

Some callers cannot allocate device memory while they run: a real-time
detection loop that reserved its memory at start-up and must keep
cudaMalloc/cudaFree (which can synchronise the device) out of its processing
path, or a host application that owns the GPU's memory budget.  For them the
library offers an entry point whose working arrays live in one file-scope
device array.  This file checks, through the C ABI, that it gives the regular
entry point's results within the suite's tolerance on two calls in a row
(sharing that array) in every normalisation and output layout, with and
without caller-supplied template energies, across the 65,535-template launch
split and at a size that fills the array to its end; that it leaves free
device memory unchanged; and that it rejects a search larger than the array
and a misaligned device array.  The file name makes pytest
collect it last.
"""
import ctypes as ct

import numpy as np
import pytest

from fast_matched_filter_gb300 import _lib
from tests._cases import random_search

TOL = 1e-5
CAP = 32 * 1024 * 1024  # FMF_NOALLOC_SCRATCH_BYTES
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
    lib.fmf_last_launch_count.restype = ct.c_int
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


def _compare(got, ref):
    got = got.cpu().numpy()
    assert got.shape == ref.shape
    assert np.array_equal(got == 0.0, ref == 0.0)
    assert np.abs(got.astype(np.float64) - ref).max() <= TOL


def _scratch_bytes(T, SC, L, N, full, energies):
    """The entry point's documented scratch need (each part rounded to 256 B)."""
    al = lambda b: (b + 255) & ~255  # noqa: E731
    b = al(8 * T) + al(4 * SC * N * (2 if full else 1))
    if energies:
        b += al(4 * T * SC)
    if full:
        b += al(4 * SC * N) + al(4 * SC) + al(4 * T * SC * L) + al(4 * T * SC)
    return b


def _free_memory():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("normalize", ["short", "full"])
@pytest.mark.parametrize("network_sum", [True, False])
def test_two_calls_in_a_row_match_the_regular_entry_point(normalize, network_sum):
    lib = _bind()
    a = _search(1, 3, 4, 3, 120, 30000, 1, normalize, network_sum)
    b = _search(2, 2, 3, 2, 200, 20000, 2, normalize, network_sum)
    ref_a = _regular(lib, *a[1:]).cpu().numpy()
    ref_b = _regular(lib, *b[1:]).cpu().numpy()
    launches = lib.fmf_last_launch_count()
    _noalloc(lib, *a[1:])  # the first call on this device looks up the scratch address
    free0 = _free_memory()
    got_a = _noalloc(lib, *a[1:])
    got_b = _noalloc(lib, *b[1:])  # the second call in a row reuses the same scratch
    assert lib.fmf_last_launch_count() == launches  # every kernel it queues is counted
    free1 = _free_memory()
    _compare(got_a, ref_a)
    _compare(got_b, ref_b)
    assert free1 == free0
    assert lib.fmf_device_errors() == 0


def test_energies_computed_when_not_passed():
    """sum_square_templates = NULL: the energies are computed into the scratch
    array, as fmf_matched_filter computes them."""
    lib = _bind()
    g, args, flags, shape = _search(4, 4, 3, 3, 150, 25000, 1, "full", True)
    ref = _regular(lib, args, flags, shape).cpu().numpy()
    no_sst = (args[0], None) + args[2:]
    for _ in range(2):
        _compare(_noalloc(lib, no_sst, flags, shape), ref)


def test_more_templates_than_one_launch_takes():
    """70,000 templates: the plain kernel runs in launches of 65,535
    templates, each at its offset into the inputs and the output."""
    lib = _bind()
    g, args, flags, shape = _search(5, 70000, 1, 1, 8, 400, 1, "short", True)
    ref = _regular(lib, args, flags, shape).cpu().numpy()
    for _ in range(2):
        _compare(_noalloc(lib, args, flags, shape), ref)


@pytest.mark.parametrize("normalize,S,C,N,L", [("short", 4, 2, 1048000, 300),
                                               ("full", 4, 2, 349000, 200)])
def test_search_that_fills_the_scratch_array(normalize, S, C, N, L):
    """Sized so the carve ends within 64 KiB of the array's end."""
    lib = _bind()
    T = 2
    need = _scratch_bytes(T, S * C, L, N, normalize == "full", False)
    assert CAP - 65536 < need <= CAP
    g, args, flags, shape = _search(6, T, S, C, L, N, 1, normalize, True)
    ref = _regular(lib, args, flags, shape).cpu().numpy()
    for _ in range(2):
        _compare(_noalloc(lib, args, flags, shape), ref)


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


def test_misaligned_device_array_is_rejected():
    """A device array 2 bytes off its element alignment is an argument error,
    returned before anything is queued."""
    lib = _bind()
    g, args, flags, shape = _search(7, 2, 2, 3, 64, 5000, 1, "short", True)
    out = torch.zeros(shape, dtype=torch.float32, device="cuda")
    bad = args[:3] + (args[3] + 2,) + args[4:]
    st = lib.fmf_matched_filter_noalloc(*bad, out.data_ptr(), *flags,
                                        torch.cuda.current_stream().cuda_stream)
    assert st == _lib.FMF_ERR_ARG
    assert "aligned" in _lib.last_error(lib)[1]
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0
