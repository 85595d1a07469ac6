"""The float32 rounding facts the one-read detection rests on (CPU, no GPU).

The counting pass decides each value's MAD class before the median is exact:
with the median known to lie in [m_lo, m_hi] (floats), a value x is counted
below the MAD window when |x - m| < a_lo for *every* float m in that range,
and dropped when |x - m| > a_hi for every such m.  The kernels test only the
two ends (fmf_detect.cu: below_all, near_some), which is exact if float32
|x - m| (round to nearest, as __fsub_rn) first falls, then rises, in m.  The
hot values are those >= thr_lo = m_lo + n_mad * a_lo, which bounds
thr = med + n_mad * mad from below if float32 rounding keeps that expression
monotone in med and in mad.  numpy's float32 arithmetic is IEEE round to
nearest, as the kernels' __fsub_rn / __fadd_rn / __fmul_rn."""
import numpy as np

f32 = np.float32


def dev(x, m):
    return np.abs(f32(x) - f32(m))


def _floats(rng, n, scale):
    """Floats of mixed magnitudes and signs around 0 and around an offset."""
    base = rng.standard_normal(n).astype(np.float32) * f32(scale)
    off = rng.choice(np.array([0.0, 1e-3, 0.37, 5.0, -2.0], np.float32), n)
    return (base + off).astype(np.float32)


def test_deviation_falls_then_rises_in_m():
    """For floats m1 <= m2 <= m3: |x - m2| <= max(|x - m1|, |x - m3|) and
    >= min of the two when x is outside [m1, m3] -- so the largest and the
    smallest deviation over [m_lo, m_hi] are at its ends (or 0 inside)."""
    rng = np.random.default_rng(71)
    for scale in (1e-6, 1e-3, 1.0, 1e3):
        x = _floats(rng, 200000, scale)
        m = np.sort(_floats(rng, 3 * 200000, scale).reshape(-1, 3), axis=1)
        d1, d2, d3 = dev(x, m[:, 0]), dev(x, m[:, 1]), dev(x, m[:, 2])
        assert np.all(d2 <= np.maximum(d1, d3))
        outside = (x < m[:, 0]) | (x > m[:, 2])
        assert np.all(d2[outside] >= np.minimum(d1, d3)[outside])


def test_deviation_is_monotone_in_x_on_each_side():
    """|x - m| falls as x rises towards m and rises after it: each MAD class
    is an interval of x, so bisection over the float keys finds its ends."""
    rng = np.random.default_rng(72)
    m = f32(0.37)
    x = np.sort(_floats(rng, 400000, 1.0))
    d = dev(x, m)
    left, right = x <= m, x >= m
    assert np.all(np.diff(d[left]) <= 0)
    assert np.all(np.diff(d[right]) >= 0)


def test_threshold_is_monotone_in_median_and_mad():
    """thr = med + n_mad * mad (multiply, then add; no fused multiply-add)
    never falls when med or mad rises (n_mad >= 0), and never rises with mad
    for n_mad < 0: thr_lo from the windows' lower ends bounds thr."""
    rng = np.random.default_rng(73)
    for n_mad in (f32(8.0), f32(3.5), f32(0.0), f32(-0.5)):
        med = np.sort(_floats(rng, 2 * 100000, 0.01).reshape(-1, 2), axis=1)
        mad = np.sort(np.abs(_floats(rng, 2 * 100000, 0.01)).reshape(-1, 2), axis=1)
        thr = lambda a, b: (a + (n_mad * b).astype(np.float32)).astype(np.float32)  # noqa: E731
        assert np.all(thr(med[:, 0], mad[:, 0]) <= thr(med[:, 1], mad[:, 0]))
        if n_mad >= 0:
            assert np.all(thr(med[:, 0], mad[:, 0]) <= thr(med[:, 0], mad[:, 1]))
        else:
            assert np.all(thr(med[:, 0], mad[:, 1]) <= thr(med[:, 0], mad[:, 0]))


def test_midpoints_stay_inside_their_ends():
    """numpy's median of an even count, (a + b) * 0.5 in float32, and the
    window middle 0.5 * m_lo + 0.5 * m_hi both lie in [a, b]: a median whose
    two middle values are in the window is in [m_lo, m_hi]."""
    rng = np.random.default_rng(74)
    for scale in (1e-30, 1e-3, 1.0, 1e30):
        ab = np.sort(_floats(rng, 2 * 200000, scale).reshape(-1, 2), axis=1)
        a, b = ab[:, 0], ab[:, 1]
        med = ((a + b).astype(np.float32) * f32(0.5)).astype(np.float32)
        mid = (f32(0.5) * a + f32(0.5) * b).astype(np.float32)
        assert np.all((a <= med) & (med <= b))
        assert np.all((a <= mid) & (mid <= b))


def test_signed_zero_compares_as_one_value():
    """The counting pass compares floats (where -0 == +0) and keys its
    candidates as x + 0, which is +0 for x = -0: the two views agree."""
    z = np.array([-0.0, 0.0], np.float32)
    assert z[0] == z[1]
    assert np.signbit((z + f32(0.0))[0]) == np.False_
    assert dev(z[0], f32(0.0)) == dev(z[1], f32(0.0)) == 0
