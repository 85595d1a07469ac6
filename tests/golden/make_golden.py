"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own Python wrapper (fast_matched_filter.py) from the
read-only reference checkout, with its CPU library compiled from the
reference source by ``oracle/Makefile`` (``make -C oracle ref``) into
``oracle/_ref``.  Each fixture stores the inputs exactly as passed to the
wrapper, the call options and the wrapper's output.

    python tests/golden/make_golden.py [/path/to/reference/checkout]

Needs the reference checkout; the fixtures it writes are committed so that
tests elsewhere need neither.
"""
import ctypes as ct
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import cpu  # noqa: E402


def load_reference_wrapper(ref_root):
    """Import the reference wrapper by path and bind it to oracle/_ref."""
    path = os.path.join(ref_root, "fast_matched_filter", "fast_matched_filter.py")
    spec = importlib.util.spec_from_file_location("fmf_reference_wrapper", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)  # prints "not compiled": its lib/ dir is empty
    lib = ct.cdll.LoadLibrary(cpu.REF_SO)
    lib.matched_filter.argtypes = mod.argtypes
    lib.matched_filter_precise.argtypes = mod.argtypes + [ct.c_int]
    lib.matched_filter_no_sum.argtypes = mod.argtypes
    lib.matched_filter_precise_no_sum.argtypes = mod.argtypes + [ct.c_int]
    lib.matched_filter_variable_precise.argtypes = (mod.argtypes[0:6] + [ct.POINTER(ct.c_int)]
                                                    + mod.argtypes[7:] + [ct.c_int])
    mod._libCPU = lib
    mod.CPU_LOADED = True
    return mod


def cases():
    """(name, wrapper inputs, options).  Small seeded searches covering the
    formats, moveout signs, steps, normalisations, zero weights and gaps."""
    out = []

    def base(seed, T, S, C, L, N, mo_lo, mo_hi, dc=0.0, amp=1.0):
        rng = np.random.default_rng(seed)
        tp = (rng.standard_normal((T, S, C, L)) * np.hanning(L)).astype(np.float32)
        d = (rng.standard_normal((S, C, N)) * amp + dc).astype(np.float32)
        mo = rng.integers(mo_lo, mo_hi + 1, (T, S, C)).astype(np.int32)
        w = rng.uniform(0.1, 1.0, (T, S, C)).astype(np.float32)
        # plant one copy of template 0 so that some coefficients are large
        i0 = N // 3
        for s in range(S):
            for c in range(C):
                a = i0 + mo[0, s, c]
                if 0 <= a and a + L <= N:
                    d[s, c, a:a + L] += 0.8 * amp * tp[0, s, c]
        return tp, mo, w, d

    tp, mo, w, d = base(1, 3, 4, 3, 96, 3000, 0, 150)
    out.append(("cpu_short_sum", dict(templates=tp, moveouts=mo, weights=w, data=d, step=1),
                dict(arch="cpu", normalize="short", network_sum=True)))
    out.append(("precise_short_sum", dict(templates=tp, moveouts=mo, weights=w, data=d, step=1),
                dict(arch="precise", normalize="short", network_sum=True)))

    tp, mo, w, d = base(8, 2, 3, 2, 64, 1200, -10, 60)
    w[1, 1, 0] = 0.0
    out.append(("cpu_short_nosum", dict(templates=tp, moveouts=mo, weights=w, data=d, step=1),
                dict(arch="cpu", normalize="short", network_sum=False)))

    tp, mo, w, d = base(2, 2, 3, 3, 80, 2500, -40, 90)
    w[1, 0, 2] = 0.0
    w[0, 2, :] = 0.0
    out.append(("cpu_short_negmo_step3", dict(templates=tp, moveouts=mo, weights=w, data=d, step=3),
                dict(arch="cpu", normalize="short", network_sum=True)))

    tp, mo, w, d = base(3, 2, 3, 3, 120, 3200, 0, 100, dc=50.0, amp=2.0)
    out.append(("precise_full_sum_step2", dict(templates=tp, moveouts=mo, weights=w, data=d, step=2),
                dict(arch="precise", normalize="full", network_sum=True)))
    tp, mo, w, d = base(9, 2, 2, 3, 100, 1400, 0, 80, dc=-30.0, amp=3.0)
    out.append(("precise_full_nosum", dict(templates=tp, moveouts=mo, weights=w, data=d, step=2),
                dict(arch="precise", normalize="full", network_sum=False)))

    tp, mo, w, d = base(4, 2, 4, 1, 64, 2400, 0, 60)
    d[1, 0, 700:1100] = 0.0  # a gap longer than the template: zero coefficients
    d[2, 0, 1500:1530] = 0.0
    out.append(("cpu_short_gaps", dict(templates=tp, moveouts=mo, weights=w, data=d, step=1),
                dict(arch="cpu", normalize="short", network_sum=True)))

    # traces format: templates (T, traces, L), data (traces, N), moveouts (T, traces)
    tp, mo, w, d = base(5, 2, 6, 1, 72, 2000, 0, 40)
    out.append(("cpu_traces_format",
                dict(templates=tp.reshape(2, 6, 72), moveouts=mo.reshape(2, 6),
                     weights=w.reshape(2, 6), data=d.reshape(6, 2000), step=1),
                dict(arch="cpu", normalize="short", network_sum=True)))

    # single-template format: templates (S, C, L), moveouts/weights (S, C)
    tp, mo, w, d = base(6, 1, 3, 3, 90, 2200, 0, 70)
    out.append(("cpu_single_template",
                dict(templates=tp[0], moveouts=mo[0], weights=w[0], data=d, step=1),
                dict(arch="cpu", normalize="short", network_sum=True)))

    # moveouts/weights given per station (T, S), broadcast over components
    tp, mo, w, d = base(7, 2, 4, 3, 64, 2000, 0, 50)
    out.append(("cpu_station_moveouts",
                dict(templates=tp, moveouts=mo[:, :, 0].copy(), weights=w[:, :, 0].copy(),
                     data=d, step=2),
                dict(arch="cpu", normalize="short", network_sum=True)))
    # per-channel template lengths (arch='variable_precise'), short and full
    for name, seed, step, norm in (("variable_short", 10, 1, "short"),
                                   ("variable_full_step2", 11, 2, "full")):
        tp, mo, w, d = base(seed, 2, 3, 2, 90, 2600, -15, 80, dc=1.5 if norm == "full" else 0.0)
        rng = np.random.default_rng(seed + 100)
        nt = rng.integers(45, 91, (2, 3, 2)).astype(np.int32)
        tp = np.ascontiguousarray(tp[..., :int(nt.max())])  # last axis = longest template
        for t in range(2):
            for s_ in range(3):
                for c in range(2):
                    tp[t, s_, c, nt[t, s_, c]:] = 0.0
        out.append((name, dict(templates=tp, moveouts=mo, weights=w, data=d, step=step,
                               n_samples_template=nt),
                    dict(arch="variable_precise", normalize=norm, network_sum=True)))
    return out


def reference_data_cases(ref_root):
    """The reference test suite's 'noisy' dataset (tests/data/noisy_*.npy, used by
    test_python.py:27-40 with weights 1/S), cropped to 10,000 samples around the
    dataset's largest coefficient (lag 83,437), so that the fixture stays small."""
    ddir = os.path.join(ref_root, "fast_matched_filter", "tests", "data")
    data = np.load(os.path.join(ddir, "noisy_data.npy"))
    tp = np.load(os.path.join(ddir, "noisy_template.npy"))
    pads = np.load(os.path.join(ddir, "noisy_pads.npy"))
    T, S = tp.shape[0], data.shape[0]
    crop = np.ascontiguousarray(data[..., 80000:90000])
    inputs = dict(templates=tp, moveouts=pads, weights=np.ones((T, S), np.float32) / S,
                  data=crop, step=1)
    return [("reference_noisy_crop", inputs,
             dict(arch="cpu", normalize="short", network_sum=True))]


def main(ref_root=None):
    ref_root = ref_root or cpu.reference_root()
    cpu.build(os.path.join(ref_root, "fast_matched_filter", "src", "matched_filter.c"))
    ref = load_reference_wrapper(ref_root)
    for name, inputs, opts in cases() + reference_data_cases(ref_root):
        cc = ref.matched_filter(check_zeros=False, **inputs, **opts)
        arrays = {k: np.asarray(v) for k, v in inputs.items()}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), cc=cc,
                            arch=opts["arch"], normalize=opts["normalize"],
                            network_sum=opts["network_sum"], **arrays)
        print("%-26s cc %s max %.6f" % (name, cc.shape, float(np.abs(cc).max())))


if __name__ == "__main__":
    main(*sys.argv[1:])
