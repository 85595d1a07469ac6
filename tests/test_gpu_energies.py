"""Template energies on the GPU (fmf_template_energies, and the search
entry points called without sum_square_templates) -- bit-identical to the
reference wrapper's numpy.sum(templates**2, axis=-1) (needs a GB300)."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import _lib
from tests._cases import random_search

pytestmark = pytest.mark.gpu


def energies(t):
    lib = _lib.load()
    t = np.ascontiguousarray(t, dtype=np.float32)
    out = np.zeros(t.shape[:-1], np.float32)
    _lib.check(lib.fmf_template_energies(t.ctypes.data, out.size, t.shape[-1], out.ctypes.data, 0,
                                         None), lib)
    return out


@pytest.mark.parametrize("L", [1, 2, 7, 8, 9, 15, 16, 17, 127, 128, 129, 200, 256, 257, 600, 1201,
                               4000])
def test_energies_bit_identical_to_numpy(L):
    rng = np.random.default_rng(L)
    t = (rng.standard_normal((7, 5, L)) * np.exp(rng.uniform(-6, 6, (7, 5, 1)))).astype(np.float32)
    assert np.array_equal(energies(t), np.sum(t ** 2, axis=-1))


def test_energies_device_pointers():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    t = rng.standard_normal((40, 3, 777)).astype(np.float32)
    dt = torch.from_numpy(t).cuda()
    out = torch.empty((40, 3), dtype=torch.float32, device="cuda")
    lib = _lib.load()
    _lib.check(lib.fmf_template_energies(dt.data_ptr(), 120, 777, out.data_ptr(),
                                         _lib.FLAG_DEVICE_POINTERS,
                                         torch.cuda.current_stream().cuda_stream), lib)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), np.sum(t ** 2, axis=-1))


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("normalize,network_sum", [("short", True), ("full", True),
                                                   ("short", False)])
def test_search_without_energies_is_unchanged(precision, normalize, network_sum):
    """The front-end leaves float32 energies to the library; the result must
    equal the call with numpy's energies bit for bit."""
    tp, mo, w, d = random_search(17, 3, 3, 2, 333, 9000, -10, 120,
                                 dc=1.0 if normalize == "full" else 0.0)
    lib = _lib.load()
    T, S, C, L = tp.shape
    N = d.shape[-1]
    n_corr = N - L + 1
    nout = T * n_corr * (1 if network_sum else S * C)
    res = []
    for sst in (np.ascontiguousarray(np.sum(tp ** 2, axis=-1), np.float32), None):
        cc = np.zeros(nout, np.float32)
        st = lib.fmf_matched_filter_ex(tp.ctypes.data, None if sst is None else sst.ctypes.data,
                                       mo.ctypes.data, d.ctypes.data, w.ctypes.data, 1, L, N, T,
                                       S, C, n_corr, cc.ctypes.data,
                                       1 if normalize == "full" else 0, int(network_sum),
                                       _lib.PRECISIONS[precision], 0, None)
        _lib.check(st, lib)
        res.append(cc)
    assert np.array_equal(res[0], res[1])
    # and the front-end (device energies) equals the explicit call
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize=normalize,
                             network_sum=network_sum, precision=precision)
    assert np.array_equal(got.ravel(), res[0])
