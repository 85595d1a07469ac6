"""Shared helpers of the test suite: golden fixtures and seeded searches."""
import glob
import os

import numpy as np

from fast_matched_filter_gb300.fast_matched_filter import prepare

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    inputs = {k: z[k] for k in ("templates", "moveouts", "weights", "data")}
    inputs["step"] = int(z["step"])
    if "n_samples_template" in z.files:
        inputs["n_samples_template"] = z["n_samples_template"]
    opts = dict(arch=str(z["arch"]), normalize=str(z["normalize"]),
                network_sum=bool(z["network_sum"]))
    return inputs, opts, z["cc"]


def golden_names_fixed():
    """Fixtures of the fixed-length archs ('cpu', 'precise')."""
    return [n for n in golden_names() if not n.startswith("variable")]


def golden_names_variable():
    """Fixtures of the per-channel-length arch ('variable_precise')."""
    return [n for n in golden_names() if n.startswith("variable")]


def canonical(inputs):
    """Wrapper-format inputs -> canonical (T,S,C,L), (T,S,C), (T,S,C), (S,C,N)."""
    pp = prepare(inputs["templates"], inputs["moveouts"], inputs["weights"],
                 inputs["data"], inputs["step"])
    T, S, C, L, N = pp["T"], pp["S"], pp["C"], pp["L"], pp["N"]
    return (pp["templates"].reshape(T, S, C, L), pp["moveouts"].reshape(T, S, C),
            pp["weights"].reshape(T, S, C), pp["data"].reshape(S, C, N))


def random_search(seed, T, S, C, L, N, mo_lo=0, mo_hi=100, dc=0.0, amp=1.0,
                  zero_weights=0, plant=True):
    rng = np.random.default_rng(seed)
    tp = (rng.standard_normal((T, S, C, L)) * np.hanning(L + 2)[1:-1]).astype(np.float32)
    d = (rng.standard_normal((S, C, N)) * amp + dc).astype(np.float32)
    mo = rng.integers(mo_lo, mo_hi + 1, (T, S, C)).astype(np.int32)
    w = rng.uniform(0.0, 1.0, (T, S, C)).astype(np.float32)
    w /= w.sum(axis=(1, 2), keepdims=True)
    for z in range(zero_weights):
        w[rng.integers(T), rng.integers(S), rng.integers(C)] = 0.0
    if plant:
        for t in range(T):
            i0 = int(rng.integers(0, max(1, N - L - mo_hi)))
            for s in range(S):
                for c in range(C):
                    a = i0 + mo[t, s, c]
                    if 0 <= a and a + L <= N:
                        d[s, c, a:a + L] += 0.7 * amp * tp[t, s, c]
    return tp, mo, w, d
