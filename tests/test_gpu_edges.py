"""Edge cases of sizes and moveouts, both numerator forms (needs a GB300)."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from tests._cases import random_search
from tests.test_gpu_parity import assert_parity, oracle_of

pytestmark = pytest.mark.gpu
PRECISIONS = ["fp32", "split_bf16"]

# Worst-case error of one split-BF16 product relative to |t*d|: each operand
# is hi + lo with a residual of at most 2**-16 of its value (two 8-bit
# significands, round-to-nearest), and the dropped lo*lo term is at most
# 2**-16 as well.  A single unweighted channel of 8 taps averages nothing, so
# its cc can carry that bound; searches with many channels or long templates
# stay far below 1e-5 (the parity suite's bar).
SPLIT_SINGLE_CHANNEL_TOL = 3 * 2.0 ** -16


@pytest.mark.parametrize("precision", PRECISIONS)
def test_more_templates_than_a_grid_dimension(oracle_built, precision):
    # 70,000 templates > 65,535: template slicing / 1-D grids / tile queue
    rng = np.random.default_rng(1)
    T, L, N = 70000, 8, 64
    tp = rng.standard_normal((T, 1, 1, L)).astype(np.float32)
    d = rng.standard_normal((1, 1, N)).astype(np.float32)
    mo = rng.integers(0, 5, (T, 1, 1)).astype(np.int32)
    w = np.ones((T, 1, 1), np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, precision=precision)
    tol = SPLIT_SINGLE_CHANNEL_TOL if precision == "split_bf16" else 1e-5
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 1, "short", True), tol)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_moveouts_outside_the_trace(oracle_built, precision):
    tp, mo, w, d = random_search(2, 4, 2, 2, 50, 3000, 0, 100)
    mo[1, 0, 0] = 10 ** 6   # beyond the trace: no valid output
    mo[2, 1, 1] = -10 ** 6  # far before the trace: no valid output
    mo[3, :, :] -= 40       # negative but reachable
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, precision=precision)
    assert np.all(got[1] == 0.0) and np.all(got[2] == 0.0)
    for t in (0, 3):
        ref = oracle_of(oracle_built, tp[t:t + 1], mo[t:t + 1], w[t:t + 1], d, 1, "short", True)
        assert_parity(got[t:t + 1], ref)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_step_larger_than_template(oracle_built, precision, normalize):
    tp, mo, w, d = random_search(3, 2, 2, 1, 20, 6000, 0, 30, dc=1.0)
    got = fmf.matched_filter(tp, mo, w, d, 50, check_zeros=False, normalize=normalize,
                             precision=precision)
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 50, normalize, True))


@pytest.mark.parametrize("precision", PRECISIONS)
def test_single_channel_single_template(oracle_built, precision):
    tp, mo, w, d = random_search(4, 1, 1, 1, 300, 100000, 0, 0)
    got = fmf.matched_filter(tp[0, 0], mo[0, 0], w[0, 0], d[0], 1, check_zeros=False,
                             precision=precision)
    assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 1, "short", True))
    assert got.shape == (1, 100000 - 300 + 1)


def test_template_longer_than_data_rejected():
    with pytest.raises(ValueError):
        fmf.matched_filter(np.ones((1, 1, 1, 100), np.float32), np.zeros((1, 1, 1), np.int32),
                           np.ones((1, 1, 1), np.float32), np.ones((1, 1, 50), np.float32), 1)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("mode", ["sum", "no_sum", "variable"])
def test_out_is_written_in_full_and_returned(precision, mode):
    # a caller-owned output full of NaN: every element is overwritten (the
    # zeros outside the valid lags included) and the same array comes back
    rng = np.random.default_rng(7)
    T, S, C, L, N = 3, 4, 3, 50, 2000
    tp = rng.standard_normal((T, S, C, L)).astype(np.float32)
    d = rng.standard_normal((S, C, N)).astype(np.float32)
    mo = rng.integers(0, 40, (T, S, C)).astype(np.int32)
    w = rng.random((T, S, C)).astype(np.float32)
    kw = {"precision": precision, "check_zeros": False}
    if mode == "no_sum":
        kw["network_sum"] = False
    if mode == "variable":
        n = rng.integers(20, L + 1, (T, S, C))
        n[0, 0, 0] = L  # the template array's length is the longest
        kw["n_samples_template"] = n
    fresh = fmf.matched_filter(tp, mo, w, d, 1, **kw)
    out = np.full(fresh.shape, np.nan, np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, out=out, **kw)
    assert got is out
    np.testing.assert_array_equal(out, fresh)
