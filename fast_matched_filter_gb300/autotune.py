"""Tile-shape autotuner of the tensor-core forms.

Two shape parameters of ``tc_persistent`` (csrc/fmf_tc.cu) change its speed but
not its results: the lag blocks per tile (NB = 32, 64 or 128; 128 outputs each)
and the number of templates whose items are interleaved in the tile queue
(data rows and window statistics they share stay in L2 while the group sweeps
the tiles).  ``tune`` times candidate shapes on a sample of a real search
(its first templates, all channels, the whole trace) through the C ABI and
caches the fastest per search class -- template length, step, channels,
normalisation, precision -- in a JSON file (``$FMF_AUTOTUNE_CACHE``, default
``~/.cache/fmf_gb300/tiles.json``).  ``matched_filter`` and
``matched_filter_device`` use a cached shape when one exists.
"""
import json
import os
import time

from . import _lib

CANDIDATES = ((128, 16), (128, 8), (128, 32), (64, 16), (64, 32), (32, 16))


def cache_path():
    return os.environ.get("FMF_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "fmf_gb300", "tiles.json")


def search_class(L, step, n_channels, normalize, precision):
    return "L%d/step%d/ch%d/%s/%s" % (int(L), int(step), int(n_channels), normalize, precision)


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(table):
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(L, step, n_channels, normalize, precision):
    """Cached (lag_blocks, template_group) of a search class, or None."""
    e = _load().get(search_class(L, step, n_channels, normalize, precision))
    return (int(e["lag_blocks"]), int(e["template_group"])) if e else None


def flags_for(L, step, n_channels, normalize, precision):
    """fmf_matched_filter_ex flag bits of the cached shape (0: library default)."""
    if precision == "fp32":
        return 0
    if precision == "auto":  # the tile shape of the tensor-core form it may choose
        precision = "split_bf16"
    shape = lookup(L, step, n_channels, normalize, precision)
    if shape is None:
        return 0
    return _lib.flag_tile(shape[0]) | _lib.flag_template_group(shape[1])


def tune(templates, sum_square_templates, moveouts, weights, data, step, out,
         normalize="short", network_sum=True, precision="split_bf16",
         sample_templates=32, candidates=CANDIDATES, reps=2, save=True):
    """Time candidate shapes on the first ``sample_templates`` templates of a
    search given as device tensors (the arguments of ``matched_filter_device``);
    cache and return the fastest as a dict."""
    import torch

    lib = _lib.load()
    T, S, C, L = templates.shape
    N = data.shape[-1]
    ts = min(T, sample_templates)
    tp, sst = templates[:ts].contiguous(), sum_square_templates[:ts].contiguous()
    mo, w, o = moveouts[:ts].contiguous(), weights[:ts].contiguous(), out[:ts].contiguous()
    stream = torch.cuda.current_stream()
    results = []
    for nb, tg in candidates:
        flags = _lib.FLAG_DEVICE_POINTERS | _lib.flag_tile(nb) | _lib.flag_template_group(tg)

        def call():
            return lib.fmf_matched_filter_ex(
                tp.data_ptr(), sst.data_ptr(), mo.data_ptr(), data.data_ptr(), w.data_ptr(),
                int(step), L, N, ts, S, C, o.shape[1], o.data_ptr(),
                1 if normalize == "full" else 0, int(bool(network_sum)),
                _lib.PRECISIONS[precision], flags, stream.cuda_stream)

        if call() != _lib.FMF_OK:  # shape does not fit this template length
            continue
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            _lib.check(call(), lib)
        torch.cuda.synchronize()
        results.append(((time.perf_counter() - t0) / reps, nb, tg))
    if not results:
        raise RuntimeError("no tensor-core tile shape fits this search")
    ms, nb, tg = min(results)
    entry = {"lag_blocks": nb, "template_group": tg, "ms_sample": 1e3 * ms,
             "sample_templates": ts,
             "tried": [{"lag_blocks": b, "template_group": g, "ms": 1e3 * t} for t, b, g in results]}
    if save:
        table = _load()
        table[search_class(L, step, S * C, normalize, precision)] = entry
        _save(table)
    return entry
