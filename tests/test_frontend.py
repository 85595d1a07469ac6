"""Host-side behaviour of the Python interface (no GPU needed): input
formats, broadcasting, n_corr and the check_zeros report follow the
reference wrapper (fast_matched_filter.py:152-362)."""
import numpy as np
import pytest

import fast_matched_filter_gb300 as fmf
from fast_matched_filter_gb300.fast_matched_filter import _zero_report, prepare
from tests._cases import canonical, load_golden


def test_reference_names_exported():
    for name in ("matched_filter", "test_matched_filter", "CPU_LOADED", "GPU_LOADED"):
        assert hasattr(fmf, name)
    assert fmf.CPU_LOADED is False


def test_import_maps_no_native_code():
    """Importing the package and its generators loads no library; the first
    read of GPU_LOADED (or the first call) does."""
    import subprocess
    import sys
    code = ("import fast_matched_filter_gb300 as f, fast_matched_filter_gb300.synthetic\n"
            "maps = lambda: open('/proc/self/maps').read()\n"
            "assert 'libfmf_gb300' not in maps()\n"
            "loaded = f.GPU_LOADED\n"
            "assert loaded == ('libfmf_gb300' in maps())\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       cwd=__import__("os").path.dirname(__import__("os").path.dirname(
                           __import__("os").path.abspath(__file__))))
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("arch", ["cpu", "precise"])
def test_cpu_architectures_reported_not_loaded(arch, capsys):
    tp = np.zeros((1, 1, 1, 8), np.float32)
    out = fmf.matched_filter(tp, np.zeros((1, 1, 1)), np.ones((1, 1, 1)),
                             np.zeros((1, 1, 100), np.float32), 1, arch=arch)
    assert out is None
    assert "not loaded" in capsys.readouterr().out


def test_full_with_cpu_arch_asserts():
    with pytest.raises(AssertionError):
        fmf.matched_filter(np.zeros((1, 1, 1, 8)), np.zeros((1, 1, 1)), np.ones((1, 1, 1)),
                           np.zeros((1, 1, 100)), 1, arch="cpu", normalize="full")


def test_unknown_normalize_asserts():
    with pytest.raises(AssertionError):
        fmf.matched_filter(np.zeros((1, 1, 1, 8)), np.zeros((1, 1, 1)), np.ones((1, 1, 1)),
                           np.zeros((1, 1, 100)), 1, normalize="half")


def test_incompatible_dimensions(capsys):
    assert prepare(np.zeros((2, 8)), np.zeros(2), np.ones(2), np.zeros((2, 3, 4, 100)), 1) is None


def test_formats_canonicalise_alike():
    rng = np.random.default_rng(0)
    tp = rng.standard_normal((2, 4, 3, 20)).astype(np.float32)
    d = rng.standard_normal((4, 3, 300)).astype(np.float32)
    mo = rng.integers(0, 9, (2, 4, 3)).astype(np.int32)
    w = rng.random((2, 4, 3)).astype(np.float32)
    a = prepare(tp, mo, w, d, 1)
    b = prepare(tp.reshape(2, 12, 20), mo.reshape(2, 12), w.reshape(2, 12), d.reshape(12, 300), 1)
    for k in ("templates", "moveouts", "weights", "data", "sst"):
        assert np.array_equal(a[k], b[k]), k
    assert (a["T"], a["S"], a["C"]) == (2, 4, 3) and (b["T"], b["S"], b["C"]) == (2, 12, 1)
    single = prepare(tp[0], mo[0], w[0], d, 1)
    assert single["T"] == 1 and np.array_equal(single["templates"], a["templates"][:4 * 3 * 20])


def test_station_moveouts_broadcast_over_components():
    inputs, _, _ = load_golden("cpu_station_moveouts")
    tp, mo, w, d = canonical(inputs)
    assert np.array_equal(mo, np.repeat(inputs["moveouts"], 3).reshape(mo.shape))
    assert np.array_equal(w, np.repeat(inputs["weights"], 3).reshape(w.shape).astype(np.float32))


def test_n_corr_rule():
    pp = prepare(np.zeros((1, 1, 1, 10)), np.zeros((1, 1, 1)), np.ones((1, 1, 1)),
                 np.zeros((1, 1, 107)), 4)
    assert pp["n_corr"] == int((107 - 10) / 4 + 1) == 25


def test_bad_broadcast_raises():
    with pytest.raises(ValueError):
        prepare(np.zeros((2, 3, 2, 10)), np.zeros((5,)), np.ones((5,)), np.zeros((3, 2, 100)), 1)


def test_zero_report_messages(capsys):
    cc = np.ones((2, 100), np.float32)
    cc[0, :30] = 0.0
    cc[1, :5] = 0.0
    mo = np.array([0, 10, 20], np.int32)
    w = np.ones(3, np.float32)
    z = _zero_report(cc, mo, w, 2, 100, 1, True, "all")
    assert list(z) == [30, 5]
    out = capsys.readouterr().out
    assert "30 correlation computations were skipped on the 0-th" in out
    assert "1-th" not in out
    z = _zero_report(cc, mo, w, 2, 100, 1, True, "first")
    assert list(z) == [30]
    _zero_report(cc, mo, w, 2, 100, 1, True, "bogus")
    assert "check_zeros should be False" in capsys.readouterr().out
    assert _zero_report(cc, mo, w, 2, 100, 1, True, False) is None


def test_zero_report_per_channel_layout_slices_last_axis():
    # the reference slices the component axis in the per-channel layout
    # (fast_matched_filter.py:339-342); the report keeps that behaviour
    cc = np.zeros((1, 50, 2, 3), np.float32)
    mo = np.array([0, 0, 0, 0, 0, 48], np.int32)  # stop = 50 - 48 = 2 components kept
    z = _zero_report(cc, mo, np.ones(6, np.float32), 1, 50, 1, False, "first")
    assert list(z) == [50 * 2 * 2]


def test_variable_lengths_without_network_sum_not_implemented():
    # as the reference wrapper (fast_matched_filter.py:310-313)
    with pytest.raises(NotImplementedError):
        fmf.matched_filter(np.zeros((1, 1, 1, 8), np.float32), np.zeros((1, 1, 1)),
                           np.ones((1, 1, 1)), np.zeros((1, 1, 100), np.float32), 1,
                           n_samples_template=np.full((1, 1, 1), 8), arch="variable_precise",
                           network_sum=False)


@pytest.mark.parametrize("bad", ["dtype", "shape", "order", "readonly"])
@pytest.mark.parametrize("variable", [False, True])
def test_out_must_match_the_output(bad, variable):
    T, S, C, L, N = 2, 2, 3, 8, 100
    tp = np.zeros((T, S, C, L), np.float32)
    mo = np.zeros((T, S, C), np.int32)
    w = np.ones((T, S, C), np.float32)
    d = np.zeros((S, C, N), np.float32)
    n_corr = N - L + 1
    out = {"dtype": np.zeros((T, n_corr), np.float64),
           "shape": np.zeros((T, n_corr + 1), np.float32),
           "order": np.zeros((n_corr, T), np.float32).T,
           "readonly": np.zeros((T, n_corr), np.float32)}[bad]
    if bad == "readonly":
        out.flags.writeable = False
    kw = {"n_samples_template": np.full((T, S, C), L)} if variable else {}
    with pytest.raises(ValueError, match="out must be"):
        fmf.matched_filter(tp, mo, w, d, 1, out=out, **kw)
