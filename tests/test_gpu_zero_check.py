"""check_zeros counted on the device (fmf_matched_filter_check_zeros) equals
the reference wrapper's numpy count on the returned output (needs a GB300)."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import _lib
from fast_matched_filter_gb300.fast_matched_filter import _zero_report, prepare
from tests._cases import random_search

pytestmark = pytest.mark.gpu


def gapped_search(seed, mo_hi=150):
    tp, mo, w, d = random_search(seed, 4, 3, 2, 80, 6000, 0, mo_hi)
    d[0, :, 1000:1600] = 0.0  # a gap: zero windows on every channel of station 0
    d[1, :, 1000:1700] = 0.0
    d[2, :, 900:1650] = 0.0
    return tp, mo, w, d


@pytest.mark.parametrize("network_sum", [True, False])
@pytest.mark.parametrize("check_zeros", ["first", "all"])
@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_device_counts_print_what_numpy_counts(capsys, network_sum, check_zeros, precision):
    tp, mo, w, d = gapped_search(1)
    cc = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=check_zeros, network_sum=network_sum,
                            precision=precision)
    printed = capsys.readouterr().out
    pp = prepare(tp, mo, w, d, 1)
    T = tp.shape[0]
    zeros = _zero_report(cc, pp["moveouts"], pp["weights"], T, pp["n_corr"], 1, network_sum,
                         check_zeros)
    assert capsys.readouterr().out == printed
    assert "correlation computations were skipped" in printed
    assert zeros is not None and zeros.max() > 10


@pytest.mark.parametrize("network_sum", [True, False])
def test_device_counts_equal_numpy_counts(network_sum):
    tp, mo, w, d = gapped_search(2)
    lib = _lib.load()
    T, S, C, L = tp.shape
    N = d.shape[-1]
    n_corr = N - L + 1
    cc = np.zeros(T * n_corr * (1 if network_sum else S * C), np.float32)
    last = n_corr if network_sum else C
    for stop in (0, 1, 2, last // 2, last - 1, last, last + 5):
        counts = np.zeros(T, np.uint64)
        st = lib.fmf_matched_filter_check_zeros(
            tp.ctypes.data, None, mo.ctypes.data, d.ctypes.data, w.ctypes.data, 1, L, N, T, S, C,
            n_corr, cc.ctypes.data, 0, int(network_sum), 0, 0, None, stop, counts.ctypes.data)
        _lib.check(st, lib)
        out = cc.reshape((T, n_corr) if network_sum else (T, n_corr, S, C))
        ref = np.sum(out[..., :stop].reshape(T, -1) == 0.0, axis=-1)
        assert np.array_equal(counts, ref.astype(np.uint64)), stop


def test_device_counts_on_device_arrays():
    torch = pytest.importorskip("torch")
    tp, mo, w, d = gapped_search(3)
    T, S, C, L = tp.shape
    N = d.shape[-1]
    n_corr = N - L + 1
    g = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda()
         for k, v in (("tp", tp), ("mo", mo), ("w", w), ("d", d))}
    out = torch.empty((T, n_corr), dtype=torch.float32, device="cuda")
    counts = torch.empty(T, dtype=torch.int64, device="cuda")
    lib = _lib.load()
    st = lib.fmf_matched_filter_check_zeros(
        g["tp"].data_ptr(), None, g["mo"].data_ptr(), g["d"].data_ptr(), g["w"].data_ptr(), 1, L,
        N, T, S, C, n_corr, out.data_ptr(), 0, 1, 1, _lib.FLAG_DEVICE_POINTERS,
        torch.cuda.current_stream().cuda_stream, 3000, counts.data_ptr())
    _lib.check(st, lib)
    torch.cuda.synchronize()
    ref = (out[:, :3000] == 0).sum(dim=1)
    assert torch.equal(counts, ref)
