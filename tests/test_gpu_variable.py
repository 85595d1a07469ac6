"""GPU parity of per-channel template lengths (the reference's arch
'variable_precise', matched_filter.c:321-412) against the oracle and the
golden fixtures made by the reference itself (needs a GB300).

Outputs are scaled by the reference's template-cumulative weight sum, so the
bar is TOL relative to that scale."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from tests._cases import canonical, golden_names_variable, load_golden, random_search
from tests.test_gpu_parity import TOL

pytestmark = pytest.mark.gpu


def _check(got, ref, scale):
    assert got.shape == ref.shape
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    err = np.abs(got[ok].astype(np.float64) - ref[ok]).max()
    assert err <= TOL * max(1.0, scale), "max |diff| %.3g" % err


@pytest.mark.parametrize("name", golden_names_variable())
def test_variable_golden(name):
    inputs, opts, expected = load_golden(name)
    got = fmf.matched_filter(check_zeros=False, arch="variable_precise",
                             normalize=opts["normalize"], **inputs)
    _check(got, expected.reshape(got.shape), float(np.sum(inputs["weights"])))


@pytest.mark.parametrize("step", [1, 2, 3])
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_variable_random_vs_oracle(oracle_built, step, normalize):
    rng = np.random.default_rng(60 + step)
    tp, mo, w, d = random_search(70 + step, 3, 3, 2, 160, 8000, -30, 200,
                                 dc=3.0 if normalize == "full" else 0.0, zero_weights=2)
    nt = rng.integers(60, 161, mo.shape).astype(np.int32)
    tp = np.ascontiguousarray(tp[..., :int(nt.max())])
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    got = fmf.matched_filter(tp, mo, w, d, step, n_samples_template=nt, arch="gpu",
                             check_zeros=False, normalize=normalize)
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, step, normalize)
    _check(got, ref, float(np.sum(w)))


def test_variable_equal_lengths_match_fixed_length_coefficients(oracle_built):
    """With every length equal to L the per-channel coefficients are the
    precise ones: atanh/tanh of a single channel recovers its coefficient."""
    tp, mo, w, d = random_search(5, 1, 1, 1, 100, 5000, 0, 0)
    nt = np.full(mo.shape, 100, np.int32)
    got = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False)
    ref = oracle_built.run_oracle_variable(tp, nt, mo, w, d, 1)
    _check(got, ref, 1.0)
