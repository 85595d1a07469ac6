"""Oracle of the template energies (TEST INFRASTRUCTURE ONLY).

The reference wrapper computes sum_square_templates = numpy.sum(templates**2,
axis=-1) (fast_matched_filter.py:256-261).  For float32 templates numpy sums
each contiguous row with its pairwise summation
(numpy/_core/src/umath/loops_utils.h.src, ``pairwise_sum``); this module
restates that order in plain Python so the GPU kernel that reproduces it
(template_energy_kernel) has a readable reference.  Pinned against numpy.sum
in tests/test_energies_oracle.py.
"""
import numpy as np

F = np.float32


def _leaf(a):
    n = a.size
    if n < 8:
        r = F(-0.0)
        for v in a:
            r = F(r + v)
        return r
    r = [F(v) for v in a[:8]]
    i = 8
    while i < n - (n % 8):
        for k in range(8):
            r[k] = F(r[k] + a[i + k])
        i += 8
    res = F(F(F(r[0] + r[1]) + F(r[2] + r[3])) + F(F(r[4] + r[5]) + F(r[6] + r[7])))
    while i < n:
        res = F(res + a[i])
        i += 1
    return res


def pairwise_sum(a):
    """numpy's float32 pairwise sum of a 1-D float32 array."""
    a = np.asarray(a, dtype=np.float32)
    n = a.size
    if n <= 128:
        return _leaf(a)
    n2 = n // 2
    n2 -= n2 % 8
    return F(pairwise_sum(a[:n2]) + pairwise_sum(a[n2:]))


def template_energies(templates):
    """(..., L) float32 templates -> (...) float32 energies, numpy's order."""
    t = np.asarray(templates, dtype=np.float32)
    sq = (t * t).astype(np.float32)
    flat = sq.reshape(-1, sq.shape[-1])
    return np.array([pairwise_sum(r) for r in flat], dtype=np.float32).reshape(t.shape[:-1])
