"""Window statistics next to a large transient (needs a GB300).

The reference keeps its running sums of d^2 in compensated FP64 because
"large amplitudes are recorded (e.g. large and proximal earthquakes)"
(matched_filter.c:29-31, 680-705), and its per-channel-length arch sums every
window directly (matched_filter.c:569-606).  A window's energy taken as a
difference of running sums loses the digits of everything summed before it:
after a 1,000-sample burst at amplitude 1e3, a window of 1e-2 noise holds
~1e-10 of the running sum.  These tests put such a burst before quiet
windows that hold a copy of the template (cc close to 1, where an error in the
energy shows in full) and compare every output with FP64 sums of each window:

* fixed template lengths: the burst and the copies inside one block of
  windows of the statistics kernel, 'short' and 'full', per-channel outputs;
* per-channel template lengths: the burst early in a 1.08M-sample trace and
  copies up to a million samples later (the running sums span the trace).
"""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from oracle import fp64
from tests.test_gpu_parity import TOL

pytestmark = pytest.mark.gpu

BURST_AMP, NOISE = 1e3, 1e-2


def _templates(rng, T, S, C, L):
    return (rng.standard_normal((T, S, C, L)) * np.hanning(L + 2)[1:-1]).astype(np.float32)


def _transient(rng, S, C, N, burst_at, burst_len=1000, dc=0.0):
    d = rng.standard_normal((S, C, N)) * NOISE
    d[0, :, burst_at:burst_at + burst_len] += rng.standard_normal((C, burst_len)) * BURST_AMP
    return d + dc


def _plant(d, tp, t, at, amp):
    """A copy of template t (every channel, no moveout) at sample `at`."""
    L = tp.shape[-1]
    d[:, :, at:at + L] += amp * tp[t].astype(np.float64)


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_burst_then_quiet_windows_in_one_block(normalize, precision):
    """One station, two components, 40,000 samples: the burst at 12,400-13,400
    and copies at 13,600 (template 0) and 15,000 (template 1), all inside the
    statistics kernel's block of windows [12,288, 16,384); per-channel outputs
    over the whole trace against FP64 window sums."""
    rng = np.random.default_rng(31)
    T, S, C, L, N = 2, 1, 2, 300, 40000
    tp = _templates(rng, T, S, C, L)
    d = _transient(rng, S, C, N, 12400, dc=5.0 if normalize == "full" else 0.0)
    _plant(d, tp, 0, 13600, 3 * NOISE)
    _plant(d, tp, 1, 15000, 3 * NOISE)
    d = d.astype(np.float32)
    mo = np.zeros((T, S, C), np.int32)
    w = np.full((T, S, C), 0.5, np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, check_zeros=False, normalize=normalize,
                             network_sum=False, precision=precision)
    ref = fp64.fp64_matched_filter(tp, mo, w, d, 1, normalize, False)
    assert ref[0, 13600].min() > 0.8 and ref[1, 15000].min() > 0.8
    err = np.abs(got.astype(np.float64) - ref)
    assert err.max() <= TOL, "max %.3g at %s" % (err.max(), np.unravel_index(err.argmax(), err.shape))
    assert np.array_equal(got == 0, ref == 0)


def _variable_fp64(tp, nt, w, d, normalize):
    mo = np.zeros(w.shape, np.int32)
    return fp64.fp64_matched_filter_variable(tp, nt, mo, w, d, 1, normalize)


@pytest.mark.parametrize("precision", ["fp32", "split_bf16"])
@pytest.mark.parametrize("normalize", ["short", "full"])
def test_burst_early_in_a_day_per_channel_lengths(normalize, precision):
    """Per-channel lengths (300 and 240 taps) on one channel of 1.08M
    samples: burst at 5,000, copies at 100,000 (template 0), 600,000 and
    1,070,000 (template 1)."""
    rng = np.random.default_rng(32)
    T, L, N = 2, 300, 1080000
    tp = _templates(rng, T, 1, 1, L)
    nt = np.array([300, 240], np.int32).reshape(T, 1, 1)
    tp[1, 0, 0, 240:] = 0.0
    tp[1, 0, 0, :240] *= np.hanning(242)[1:-1] / np.hanning(L + 2)[1:241]
    d = _transient(rng, 1, 1, N, 5000, dc=5.0 if normalize == "full" else 0.0)
    _plant(d, tp, 0, 100000, 3 * NOISE)
    _plant(d, tp, 1, 600000, 3 * NOISE)
    _plant(d, tp, 1, 1070000, 3 * NOISE)
    d = d.astype(np.float32)
    mo = np.zeros((T, 1, 1), np.int32)
    w = np.ones((T, 1, 1), np.float32)
    got = fmf.matched_filter(tp, mo, w, d, 1, n_samples_template=nt, check_zeros=False,
                             normalize=normalize, precision=precision)
    ref = _variable_fp64(tp, nt, w, d, normalize)
    assert ref[0, 100000] > 0.8 and ref[1, 600000] > 0.8 * 2
    # relative to each row's output scale (the running sum of the weights)
    err = np.abs(got.astype(np.float64) - ref) / np.cumsum(w.reshape(T, -1).sum(axis=1))[:, None]
    assert err.max() <= TOL, "max %.3g at %s" % (err.max(), np.unravel_index(err.argmax(), err.shape))
