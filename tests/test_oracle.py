"""Pinning of the oracle (CPU, no GPU needed).

The C restatement (oracle/fmf_oracle.c) must reproduce the reference CPU
library bit for bit: against the committed golden fixtures (made by the
reference's own wrapper and library), against the reference library itself
when it was compiled here (oracle/_ref), and on the reference's own test
data when that checkout is present.  The FP64 oracle must agree with both
to FP32 rounding.
"""
import os

import numpy as np
import pytest

from oracle import cpu
from tests._cases import (canonical, golden_names, golden_names_fixed, golden_names_variable,
                          load_golden, random_search)

REF_DATA = os.path.join(cpu.reference_root(), "fast_matched_filter", "tests", "data")


@pytest.mark.parametrize("name", golden_names_fixed())
def test_oracle_matches_golden_bit_exact(oracle_built, name):
    inputs, opts, expected = load_golden(name)
    tp, mo, w, d = canonical(inputs)
    got = oracle_built.run_oracle(tp, mo, w, d, inputs["step"], **opts)
    assert got.shape == expected.reshape(got.shape).shape
    assert np.array_equal(got, expected.reshape(got.shape)), \
        "max diff %g" % np.abs(got - expected.reshape(got.shape)).max()


@pytest.mark.parametrize("name", golden_names_fixed())
def test_fp64_oracle_close_to_golden(name):
    from oracle import fp64
    inputs, opts, expected = load_golden(name)
    tp, mo, w, d = canonical(inputs)
    thr = "sqrt" if opts["arch"] == "precise" else "product"
    got = fp64.fp64_matched_filter(tp, mo, w, d, inputs["step"], opts["normalize"],
                                   opts["network_sum"], threshold=thr)
    assert np.abs(got - expected.reshape(got.shape)).max() < 2e-6


def variable_inputs(inputs):
    """Canonical arrays of a variable-length fixture (the templates' last axis
    is the longest template)."""
    tp, mo, w, d = canonical(inputs)
    return tp, np.asarray(inputs["n_samples_template"]).reshape(mo.shape), mo, w, d


@pytest.mark.parametrize("name", golden_names_variable())
def test_oracle_variable_matches_golden_bit_exact(oracle_built, name):
    inputs, opts, expected = load_golden(name)
    tp, nt, mo, w, d = variable_inputs(inputs)
    got = oracle_built.run_oracle_variable(tp, nt, mo, w, d, inputs["step"], opts["normalize"])
    assert np.array_equal(got, expected.reshape(got.shape))


@pytest.mark.parametrize("name", golden_names_variable())
def test_fp64_variable_close_to_golden(name):
    """The FP64 per-channel-length evaluation against the reference library's
    own outputs, relative to each row's output scale."""
    from oracle import fp64
    inputs, opts, expected = load_golden(name)
    tp, nt, mo, w, d = variable_inputs(inputs)
    got = fp64.fp64_matched_filter_variable(tp, nt, mo, w, d, inputs["step"], opts["normalize"])
    exp = expected.reshape(got.shape).astype(np.float64)
    scale = np.cumsum(w.reshape(w.shape[0], -1).sum(axis=1))[:, None]
    assert np.array_equal(np.isnan(got), np.isnan(exp))
    ok = ~np.isnan(exp)
    assert (np.abs(got - exp) / scale)[ok].max() < 2e-6


def test_golden_fixtures_cover_the_reference_options():
    names = golden_names()
    assert len(names) >= 10
    seen = set()
    for n in names:
        _, o, cc = load_golden(n)
        seen.add((o["arch"], o["normalize"], o["network_sum"]))
    assert ("cpu", "short", True) in seen and ("cpu", "short", False) in seen
    assert ("precise", "full", True) in seen and ("precise", "full", False) in seen
    assert ("variable_precise", "short", True) in seen
    assert ("variable_precise", "full", True) in seen


needs_ref = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))), "oracle", "_ref", "matched_filter_CPU.so")),
    reason="reference CPU library not compiled here (no reference checkout)")


@needs_ref
@pytest.mark.parametrize("step", [1, 2, 5])
@pytest.mark.parametrize("arch,normalize", [("cpu", "short"), ("precise", "short"),
                                            ("precise", "full")])
@pytest.mark.parametrize("network_sum", [True, False])
def test_oracle_matches_reference_library(oracle_built, step, arch, normalize, network_sum):
    tp, mo, w, d = random_search(11 + step, 3, 3, 3, 57, 1500, -25, 80, dc=3.0,
                                 zero_weights=2)
    a = oracle_built.run_oracle(tp, mo, w, d, step, arch, normalize, network_sum)
    b = oracle_built.run_reference(tp, mo, w, d, step, arch, normalize, network_sum)
    assert np.array_equal(a, b)


@needs_ref
@pytest.mark.parametrize("step,normalize", [(1, "short"), (2, "full"), (3, "short"), (1, "full")])
def test_oracle_variable_matches_reference_library(oracle_built, step, normalize):
    rng = np.random.default_rng(40 + step)
    tp, mo, w, d = random_search(50 + step, 3, 3, 2, 110, 3000, -20, 90,
                                 dc=2.0 if normalize == "full" else 0.0, zero_weights=1)
    nt = rng.integers(40, 111, mo.shape).astype(np.int32)
    tp = np.ascontiguousarray(tp[..., :int(nt.max())])
    for idx in np.ndindex(nt.shape):
        tp[idx][nt[idx]:] = 0.0
    a = oracle_built.run_oracle_variable(tp, nt, mo, w, d, step, normalize)
    b = oracle_built.run_reference_variable(tp, nt, mo, w, d, step, normalize)
    assert np.array_equal(a, b)


@needs_ref
def test_cumsum_matches_reference(oracle_built):
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(20000) * np.exp(rng.uniform(-8, 8, 20000))).astype(np.float32)
    assert np.array_equal(oracle_built.cumsum_sq(x), oracle_built.cumsum_sq(x, True))


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DATA, "noisy_data.npy")),
                    reason="reference test data not present")
def test_oracle_on_reference_noisy_dataset(oracle_built):
    """The reference test's 'noisy' dataset (test_python.py:27-33, weights
    1/S as in test_python.py:38-40): the known maximum and zero tail."""
    d = np.load(os.path.join(REF_DATA, "noisy_data.npy"))
    tp = np.load(os.path.join(REF_DATA, "noisy_template.npy"))
    pads = np.load(os.path.join(REF_DATA, "noisy_pads.npy"))
    T, S = tp.shape[0], d.shape[0]
    w = np.ones((T, S)) / S
    inputs = dict(templates=tp, moveouts=pads, weights=w, data=d, step=1)
    ctp, cmo, cw, cd = canonical(inputs)
    cc = oracle_built.run_oracle(ctp, cmo, cw, cd, 1)
    assert abs(float(cc.max()) - 0.079792) < 5e-7
    assert int(np.argmax(cc[0])) == 83437
    assert np.all(cc[0, -int(cmo.max()):] == 0.0)
    assert cc[0, -int(cmo.max()) - 1] != 0.0
    if oracle_built.reference_available():
        ref = oracle_built.run_reference(ctp, cmo, cw, cd, 1)
        assert np.array_equal(cc, ref)


def test_fp64_valid_range_matches_reference_rules():
    from oracle.fp64 import valid_range
    mo = np.array([-7, 3, 12])
    # start = ceil(7/3)*3 = 9 -> index 3; last sample 100-20-12 = 68 -> index 22
    assert valid_range(mo, 3, 20, 100) == (3, 23)
    assert valid_range(np.array([0, 90]), 1, 20, 100) == (0, 0)
    assert valid_range(np.array([0, 80]), 1, 20, 100) == (0, 1)
