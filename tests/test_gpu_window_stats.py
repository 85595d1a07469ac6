"""Window statistics of every template length class against the oracle
(needs a GB300).

The statistics kernel sums each window from in-window 32-sample chunks: the
windows shorter than a chunk take a direct path, the others a suffix of the
first chunk, whole chunks and the start of the last one, 16 windows per
thread, 4,096 windows per block.  These searches cover lengths on both sides
of every boundary (1, 31, 32, 33, 63, 64, 97), traces that end inside a block
and inside a chunk, and both normalisations, in both numerator forms."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from tests._cases import random_search
from tests.test_gpu_parity import TOL, assert_parity, oracle_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("normalize", ["short", "full"])
@pytest.mark.parametrize("L", [1, 31, 32, 33, 63, 64, 97])
def test_window_lengths_around_the_chunk(oracle_built, L, normalize, precision):
    if precision == "split_bf16" and L < 16:
        pytest.skip("a split-bf16 coefficient of a few taps is outside its 1e-5 bound")
    N = 9000 + L  # three blocks of windows, the last one ragged; a ragged last chunk
    tp, mo, w, d = random_search(300 + L, 2, 2, 2, L, N, 0, 40,
                                 dc=4.0 if normalize == "full" else 0.0)
    for step in (1, 3):
        got = fmf.matched_filter(tp, mo, w, d, step, check_zeros=False, normalize=normalize,
                                 precision=precision)
        ref = oracle_of(oracle_built, tp, mo, w, d, step, normalize, True)
        tol = TOL if precision == "fp32" or L >= 32 else 3 * 2.0 ** -16
        assert_parity(got, ref, tol)


@pytest.mark.parametrize("N", [4096, 4097, 4127, 8192 + 600, 600])
def test_trace_lengths_around_the_block(oracle_built, N):
    """Traces ending exactly at, just past and inside a block of windows, and a
    trace no longer than one template (one output)."""
    tp, mo, w, d = random_search(400 + N % 97, 2, 3, 1, 600, N, 0, 0, plant=False)
    for normalize in ("short", "full"):
        got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize=normalize)
        assert_parity(got, oracle_of(oracle_built, tp, mo, w, d, 1, normalize, True), TOL)
