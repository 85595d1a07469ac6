"""GPU parity of the tensor-core forms (tcgen05 split-BF16 and single BF16).

Split-BF16 must meet the same bar as the plain form: max |cc - oracle|
<= 1e-5 and the same zero pattern.  The single-BF16 form is checked only
for the size of its loss (it exists to show that loss).
"""
import os

import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import synthetic
from tests._cases import random_search
from tests.test_gpu_parity import TOL, assert_parity, oracle_of

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["32", "64", "auto"])
def tile_lags(request, monkeypatch):
    """Lag blocks per tile (128 outputs each); 'auto' lets the library choose."""
    if request.param == "auto":
        monkeypatch.delenv("FMF_TC_NB", raising=False)
    else:
        monkeypatch.setenv("FMF_TC_NB", request.param)
    return request.param


@pytest.mark.parametrize("step", [1, 2, 3])
@pytest.mark.parametrize("L", [16, 70, 200])
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_split_bf16_network_sum(oracle_built, tile_lags, step, L, normalize):
    tp, mo, w, d = random_search(500 + 10 * step + L, 2, 2, 2, L, 20000 + 7 * L, -40, 300,
                                 dc=4.0 if normalize == "full" else 0.0, zero_weights=1)
    got = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False, normalize=normalize,
                             precision="split_bf16")
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, step, normalize, True))


@pytest.mark.parametrize("normalize", ["short", "full"])
def test_split_bf16_per_channel(oracle_built, tile_lags, normalize):
    tp, mo, w, d = random_search(8, 2, 3, 2, 90, 9000, -5, 200, dc=2.0, zero_weights=2)
    got = fmf.matched_filter(tp, mo, w, d, 2, check_zeros=False, normalize=normalize,
                             network_sum=False, precision="split_bf16")
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 2, normalize, False))


@pytest.mark.parametrize("parts", ["1", "2", "5", "auto"])
@pytest.mark.parametrize("S,C,step,normalize,zero", [(2, 1, 1, "short", 0), (3, 1, 2, "full", 1),
                                                      (4, 3, 1, "short", 3), (1, 3, 3, "full", 0)])
def test_split_bf16_channel_parts(oracle_built, monkeypatch, parts, S, C, step, normalize, zero):
    """A lone search with fewer (tile, template) items than SMs runs each item
    as k channel parts whose network sums are added in part order afterwards;
    FMF_TC_PARTS forces k (at most the channel count).  Every k meets the parity
    bar and agrees with the undivided form."""
    tp, mo, w, d = random_search(70 + S * C + step, 3, S, C, 150, 30000, -20, 150,
                                 dc=3.0 if normalize == "full" else 0.0, zero_weights=zero)
    if zero == 3:  # one template with its whole first half of channels silent
        w[1].reshape(-1)[: S * C // 2] = 0.0
    if parts == "auto":
        monkeypatch.delenv("FMF_TC_PARTS", raising=False)
    else:
        monkeypatch.setenv("FMF_TC_PARTS", parts)
    got = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False, normalize=normalize,
                             precision="split_bf16")
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, step, normalize, True))
    monkeypatch.setenv("FMF_TC_PARTS", "1")
    other = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False, normalize=normalize,
                               precision="split_bf16")
    assert np.array_equal(got == 0, other == 0)
    assert np.abs(got - other).max() <= 1e-6


def test_split_bf16_config0(oracle_built):
    cfg = synthetic.config0()
    args = (cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"], cfg["step"])
    got = fmf.matched_filter(*args, check_zeros=False, precision="split_bf16")
    assert_parity(got, oracle_of(oracle_built, *args, "short", True))


def test_split_bf16_long_template(oracle_built):
    tp, mo, w, d = random_search(12, 2, 2, 1, 1200, 40000, 0, 1000)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, precision="split_bf16")
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 1, "short", True))


def test_split_bf16_matches_plain_on_long_trace():
    cfg = synthetic.config4(n_templates=2, n_samples=400000)
    args = (cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"], 1)
    a = fmf.matched_filter(*args, check_zeros=False, precision="fp32")
    b = fmf.matched_filter(*args, check_zeros=False, precision="split_bf16")
    assert np.array_equal(a == 0, b == 0)
    assert np.abs(a - b).max() <= TOL


def test_precision_stress_vs_fp64():
    """DC 1e3, amplitudes 1e-3..1e3, full normalisation, step 2: split-BF16
    within TOL of FP64; single BF16 visibly worse."""
    from oracle import fp64
    cfg = synthetic.config2(n_templates=2, n_samples=80000)
    tp, mo, w, d = cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"]
    ref = fp64.fp64_matched_filter(tp, mo, w, d, 2, "full", True)
    split = fmf.matched_filter(tp, mo, w, d, 2, check_zeros=False, normalize="full",
                               precision="split_bf16")
    single = fmf.matched_filter(tp, mo, w, d, 2, check_zeros=False, normalize="full",
                                precision="bf16")
    e_split = np.abs(split - ref).max()
    e_single = np.abs(single - ref).max()
    assert e_split <= TOL, e_split
    assert e_single > e_split and e_single < 5e-2


def test_no_device_errors_after_tc_runs():
    from fast_matched_filter_gb300 import _lib
    assert _lib.load().fmf_device_errors() == 0


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
def test_host_result_in_chunks_equals_device_result(monkeypatch, precision):
    """A result above 64 MB goes to host memory in template chunks: every chunk's
    kernels are queued first, then the copies (which block the host for numpy
    arrays).  The result must equal, bit for bit, the same search on device
    arrays in one launch."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("FMF_TC_PARTS", "1")  # chunking only; channel parts change the sums
    tp, mo, w, d = random_search(77, 20, 2, 1, 120, 1_050_000, 0, 60)
    host = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, precision=precision)
    assert host.nbytes > 64 << 20
    g = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in
         (tp, np.sum(tp ** 2, axis=-1).astype(np.float32), mo, w, d)]
    out = torch.empty(host.shape, dtype=torch.float32, device="cuda")
    fmf.matched_filter_device(*g, 1, out, precision=precision)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)


def test_concurrent_calls_from_host_threads():
    """The C ABI is reentrant: calls from several host threads at once (ctypes
    drops the GIL; error state and launch bookkeeping are thread-local, the
    device error word is allocated under a lock) give the results of the same
    calls made one after another."""
    import threading
    cases = [random_search(900 + i, 3, 2, 2, 90 + 10 * i, 30000, 0, 100) for i in range(4)]
    precs = ["fp32", "split_bf16", "split_bf16", "fp32"]
    serial = [fmf.matched_filter(*c, 1, check_zeros=False, precision=p) for c, p in zip(cases, precs)]
    results = [None] * len(cases)
    errors = []

    def work(i):
        try:
            for _ in range(3):
                results[i] = fmf.matched_filter(*cases[i], 1, check_zeros=False, precision=precs[i])
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(cases))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for a, b in zip(serial, results):
        assert np.array_equal(a, b)
