"""Seeded synthetic matched-filter searches (inputs only).

The reference ships one synthetic generator, ``test_matched_filter``
(fast_matched_filter.py:365-569).  These generators produce the searches the
benchmarks and parity tests use -- shapes, sizes and value distributions as
described below -- from ``numpy.random.default_rng(seed)``, so every run of a
given workload sees the same arrays.  No recorded dataset is involved.

Every generator returns a dict with canonical arrays: templates (T,S,C,L)
float32, moveouts (T,S,C) int32, weights (T,S,C) float32, data (S,C,N)
float32, plus step, normalize, network_sum and a name.
"""
import numpy as np


def _hann_noise(rng, shape, band=None):
    """Hann-tapered N(0,1) noise; ``band`` (odd int) low-passes it with a
    boxcar of that many taps before tapering (band-limited noise)."""
    x = rng.standard_normal(shape).astype(np.float32)
    if band:
        k = np.ones(band, dtype=np.float32) / band
        x = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), -1, x)
        x /= x.std(axis=-1, keepdims=True) + 1e-12
    return (x * np.hanning(shape[-1]).astype(np.float32)).astype(np.float32)


def _plant(rng, data, templates, moveouts, copies, amp, step=1):
    """Add ``copies`` scaled copies of every template at seeded output indices,
    each channel shifted by that template's moveout."""
    T, S, C, L = templates.shape
    N = data.shape[-1]
    for t in range(T):
        hi = N - L - int(moveouts[t].max()) - 1
        if hi <= 0:
            continue
        for k in rng.integers(0, hi // step, size=copies):
            i = int(k) * step
            for s in range(S):
                for c in range(C):
                    a = i + int(moveouts[t, s, c])
                    data[s, c, a:a + L] += amp * templates[t, s, c]


def _gaps(rng, data, stations, duty, seg=(500, 20000)):
    """Zero random segments on the given stations until ``duty`` of their
    samples are zero."""
    N = data.shape[-1]
    for s in stations:
        zeroed = 0
        while zeroed < duty * N:
            n = int(rng.integers(seg[0], seg[1]))
            a = int(rng.integers(0, N - n))
            data[s, :, a:a + n] = 0.0
            zeroed += n


def config0(seed=100):
    """Small plain search: data (12, 3, 60000) N(0,1); 20 Hann-tapered N(0,1)
    templates of 400 samples, 5 planted copies each at amplitude 0.5,
    moveouts U{0..200}, weights 1/36, step 1, short, network sum."""
    rng = np.random.default_rng(seed)
    S, C, N, T, L = 12, 3, 60000, 20, 400
    data = rng.standard_normal((S, C, N)).astype(np.float32)
    templates = _hann_noise(rng, (T, S, C, L))
    moveouts = rng.integers(0, 201, (T, S, C)).astype(np.int32)
    _plant(rng, data, templates, moveouts, 5, 0.5)
    weights = np.full((T, S, C), 1.0 / 36.0, dtype=np.float32)
    return dict(name="config0_S12C3N60000_T20L400", templates=templates, moveouts=moveouts,
                weights=weights, data=data, step=1, normalize="short", network_sum=True)


def config1(seed=101, n_templates=100, n_samples=1080000):
    """One long window: data (20, 3, 1,080,000), channel sigma log-U[1e-2,1e2],
    5% zeroed gap segments on 4 stations; 100 Hann-tapered band-limited noise
    templates of 800 samples; moveouts U{0..1000}; weights U(0,1) normalised
    to sum 1 per template; step 1, short."""
    rng = np.random.default_rng(seed)
    S, C, N, T, L = 20, 3, n_samples, n_templates, 800
    sigma = 10.0 ** rng.uniform(-2, 2, (S, C, 1))
    data = (rng.standard_normal((S, C, N), dtype=np.float32) * sigma).astype(np.float32)
    templates = _hann_noise(rng, (T, S, C, L), band=5)
    moveouts = rng.integers(0, 1001, (T, S, C)).astype(np.int32)
    _plant(rng, data, templates * sigma[None].astype(np.float32), moveouts, 1, 0.5)
    _gaps(rng, data, rng.choice(S, 4, replace=False), 0.05)
    weights = rng.uniform(0, 1, (T, S, C)).astype(np.float32)
    weights /= weights.sum(axis=(1, 2), keepdims=True)
    return dict(name="config1_S20C3N%d_T%dL800" % (N, T), templates=templates,
                moveouts=moveouts, weights=weights.astype(np.float32), data=data, step=1,
                normalize="short", network_sum=True)


def config2(seed=102, n_templates=200, n_samples=2160000):
    """Precision stress: data (16, 3, 2,160,000) with a DC offset of 1e3 per
    channel and noise amplitude log-U[1e-3, 1e3]; 200 Hann-tapered templates
    of 600 samples at their channel's amplitude; full normalisation, step 2,
    moveouts U{0..500}; uniform weights."""
    rng = np.random.default_rng(seed)
    S, C, N, T, L = 16, 3, n_samples, n_templates, 600
    amp = 10.0 ** rng.uniform(-3, 3, (S, C, 1))
    noise = rng.standard_normal((S, C, N), dtype=np.float32) * amp
    templates = (_hann_noise(rng, (T, S, C, L)) * amp[None]).astype(np.float32)
    moveouts = rng.integers(0, 501, (T, S, C)).astype(np.int32)
    _plant(rng, noise, templates, moveouts, 1, 0.5, step=2)
    data = (noise + 1000.0).astype(np.float32)
    weights = np.full((T, S, C), 1.0 / (S * C), dtype=np.float32)
    return dict(name="config2_S16C3N%d_T%dL600_full_step2" % (N, T), templates=templates,
                moveouts=moveouts, weights=weights, data=data, step=2, normalize="full",
                network_sum=True)


def config3_shapes(seed=103, n_problems=64, max_templates=500, max_samples=4320000):
    """Sizes of the batched uneven searches: per problem T in [10, max_templates],
    S in [4, 40], C in {1, 3}, L in [200, 1200], N in [1e5, max_samples]
    (log-uniform), step in {1, 2}, half 'short' and half 'full'."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(n_problems):
        out.append(dict(
            T=int(np.exp(rng.uniform(np.log(10), np.log(max_templates)))),
            S=int(rng.integers(4, 41)), C=int(rng.choice([1, 3])),
            L=int(rng.integers(200, 1201)),
            N=int(np.exp(rng.uniform(np.log(1e5), np.log(max_samples)))),
            step=int(rng.choice([1, 2])), normalize="short" if p % 2 == 0 else "full",
            seed=int(rng.integers(0, 2 ** 31))))
    return out


def config3_problem(shape):
    """Inputs of one batched problem: N(0,1) data, Hann-tapered templates,
    one planted copy per template, moveouts U{0..300}, uniform weights."""
    rng = np.random.default_rng(shape["seed"])
    T, S, C, L, N = shape["T"], shape["S"], shape["C"], shape["L"], shape["N"]
    data = rng.standard_normal((S, C, N), dtype=np.float32)
    templates = _hann_noise(rng, (T, S, C, L))
    moveouts = rng.integers(0, 301, (T, S, C)).astype(np.int32)
    _plant(rng, data, templates, moveouts, 1, 0.5, step=shape["step"])
    weights = np.full((T, S, C), 1.0 / (S * C), dtype=np.float32)
    return dict(name="config3_problem", templates=templates, moveouts=moveouts, weights=weights,
                data=data, step=shape["step"], normalize=shape["normalize"], network_sum=True)


def config4(seed=104, n_templates=500, n_samples=4320000):
    """Full-day search: data (20, 3, 4,320,000) N(0,1) with sparse zeroed gaps;
    500 Hann-tapered N(0,1) templates of 600 samples, moveouts U{0..1500},
    uniform weights, step 1, short, network sum."""
    rng = np.random.default_rng(seed)
    S, C, N, T, L = 20, 3, n_samples, n_templates, 600
    data = rng.standard_normal((S, C, N), dtype=np.float32)
    _gaps(rng, data, rng.choice(S, 2, replace=False), 0.002, seg=(200, 2000))
    templates = _hann_noise(rng, (T, S, C, L))
    moveouts = rng.integers(0, 1501, (T, S, C)).astype(np.int32)
    weights = np.full((T, S, C), 1.0 / (S * C), dtype=np.float32)
    return dict(name="config4_S20C3N%d_T%dL600" % (N, T), templates=templates,
                moveouts=moveouts, weights=weights, data=data, step=1, normalize="short",
                network_sum=True)


def variable(seed=105, n_templates=100, n_samples=1080000, normalize="short"):
    """Per-channel template lengths (the reference's 'variable_precise'):
    data (20, 3, 1,080,000) N(0,1); 100 Hann-tapered templates whose channels
    keep U{400..800} samples (zero-padded to 800); moveouts U{0..1000}; uniform
    weights; step 1; network sum (Fisher z).  normalize='full' adds a DC
    offset U(-100, 100) per channel, which the window means remove."""
    rng = np.random.default_rng(seed)
    S, C, N, T, L = 20, 3, n_samples, n_templates, 800
    data = rng.standard_normal((S, C, N), dtype=np.float32)
    nt = rng.integers(400, L + 1, (T, S, C)).astype(np.int32)
    nt[0, 0, 0] = L  # the longest channel sets the template axis and n_corr
    templates = np.zeros((T, S, C, L), dtype=np.float32)
    for idx in np.ndindex(nt.shape):
        n = int(nt[idx])
        templates[idx][:n] = (rng.standard_normal(n) * np.hanning(n)).astype(np.float32)
    moveouts = rng.integers(0, 1001, (T, S, C)).astype(np.int32)
    _plant(rng, data, templates, moveouts, 1, 0.5)
    weights = np.full((T, S, C), 1.0 / (S * C), dtype=np.float32)
    if normalize == "full":
        data += rng.uniform(-100.0, 100.0, (S, C, 1)).astype(np.float32)
    return dict(name="variable_S20C3N%d_T%dL400-800%s" % (N, T, "_full" if normalize == "full" else ""),
                templates=templates, moveouts=moveouts, weights=weights, data=data, step=1,
                normalize=normalize, network_sum=True, n_samples_template=nt)


def variable_macs(n_samples_template, n_samples, step):
    """Multiply-accumulates of a per-channel-length search: n_corr times the
    sum of every template's channel lengths."""
    nt = np.asarray(n_samples_template)
    n_corr = (n_samples - int(nt.max())) // step + 1
    return int(n_corr) * int(nt.astype(np.int64).sum())


def macs(templates_shape, n_samples, step):
    """Algorithmic multiply-accumulates of one search: T * n_corr * S * C * L."""
    T, S, C, L = templates_shape
    n_corr = (n_samples - L) // step + 1
    return T * n_corr * S * C * L
