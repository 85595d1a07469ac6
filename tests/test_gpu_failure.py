"""Failure detection on the GPU without a fault (needs a GB300).

Every wait inside the library's kernels is bounded; when one gives up, the
kernel raises a device error word, stops, and the host reports
FMF_ERR_TIMEOUT.  A self-test kernel waits on a barrier that nothing ever
arrives on (limit 100 ms); the status must be FMF_ERR_TIMEOUT and the device
must stay usable for a normal search afterwards.
"""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300 import _lib
from tests._cases import random_search

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives():
    lib = _lib.load()
    assert lib.fmf_selftest_wait_timeout(100) == _lib.FMF_ERR_TIMEOUT
    st, msg = _lib.last_error(lib)
    assert st == _lib.FMF_ERR_TIMEOUT and "gave up" in msg
    assert lib.fmf_device_errors() == 0  # the word was read and cleared
    tp, mo, w, d = random_search(4, 2, 2, 2, 60, 4000)
    a = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, precision="split_bf16")
    b = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False)
    assert np.abs(a - b).max() <= 1e-5


def test_selftest_rejects_bad_limits():
    lib = _lib.load()
    assert lib.fmf_selftest_wait_timeout(0) == _lib.FMF_ERR_ARG
    assert lib.fmf_selftest_wait_timeout(100000) == _lib.FMF_ERR_ARG


def test_fp32_fma_rate_measurement():
    """fmf_measure_fp32_fma, the plain kernel's roofline denominator: a rate
    between half and 1.05 times the nominal 152 SMs x 128 lanes x 2.07 GHz."""
    import ctypes as ct
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()
    v = ct.c_double()
    assert lib.fmf_measure_fp32_fma(ct.byref(v)) == 0
    nominal = 152 * 128 * 2 * 2.07e9 / 1e12
    assert 0.5 * nominal < v.value < 1.05 * nominal, v.value
