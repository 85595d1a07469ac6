"""FP64 numpy evaluation of the matched-filter formulas (test infrastructure).

Same semantics as the reference CPU library (fast_matched_filter/src/
matched_filter.c), evaluated in float64 with direct window sums:

* lag range per template (matched_filter.c:53-76): output index k is valid
  when start <= k*step <= N-L-max_mo, with start = ceil(-min_mo/step)*step;
  all other outputs are 0;
* short  (matched_filter.c:611-627): cc = sum(t*d) / sqrt(sst * sum(d^2));
* full   (matched_filter.c:629-657): m = mean(window),
  cc = sum(t*(d-m)) / sqrt(sst * sum((d-m)^2)), sst = raw sum(t^2);
* threshold 1e-6 on the product sst*ssd ("product", the GPU library's test,
  matched_filter.cu:132-140, and the cpu arch's, matched_filter.c:624) or on
  its square root ("sqrt", the precise arch's, matched_filter.c:650-652);
* channels with weight 0 are skipped; network sum = sum(w*cc).

Used to state the error of each GPU form against exact-ish arithmetic.
"""
import numpy as np
from numpy.lib.stride_tricks import sliding_window_view

THRESHOLD = 1e-6


def valid_range(mo_t, step, L, N):
    """[k0, k1) of valid output indices for one template's moveouts."""
    lo = min(0, int(mo_t.min()))
    hi = max(0, int(mo_t.max()))
    start = int(np.ceil(-lo / float(step))) * step if lo < 0 else 0
    last = N - L - hi
    if last < 0 or start > last:
        return 0, 0
    return start // step, last // step + 1


def fp64_matched_filter(templates, moveouts, weights, data, step,
                        normalize="short", network_sum=True,
                        threshold="product", k_range=None, t_index=None,
                        chunk=16384):
    """templates (T,S,C,L), moveouts/weights (T,S,C), data (S,C,N).

    k_range=(k0,k1) restricts the evaluated output indices (others are not
    returned); t_index selects templates.  Returns float64 of shape
    (T', K) or (T', K, S, C)."""
    templates = np.asarray(templates, dtype=np.float32)
    T, S, C, L = templates.shape
    N = data.shape[-1]
    nch = S * C
    n_corr = int((N - L) / step + 1)
    k0, k1 = (0, n_corr) if k_range is None else k_range
    tix = range(T) if t_index is None else list(t_index)
    tp = templates.reshape(T, nch, L).astype(np.float64)
    mo = np.asarray(moveouts).reshape(T, nch).astype(np.int64)
    w = np.asarray(weights, dtype=np.float32).reshape(T, nch).astype(np.float64)
    d = np.asarray(data, dtype=np.float32).reshape(nch, N).astype(np.float64)
    K = k1 - k0
    out = np.zeros((len(tix), K) if network_sum else (len(tix), K, nch))
    for oi, t in enumerate(tix):
        a, b = valid_range(mo[t], step, L, N)
        a, b = max(a, k0), min(b, k1)
        if a >= b:
            continue
        sst = np.sum(tp[t] ** 2, axis=-1)
        for c0 in range(a, b, chunk):
            c1 = min(b, c0 + chunk)
            ks = np.arange(c0, c1)
            acc = np.zeros(c1 - c0)
            for ch in range(nch):
                if w[t, ch] == 0.0:
                    continue
                first = c0 * step + mo[t, ch]
                last = (c1 - 1) * step + mo[t, ch]
                win = sliding_window_view(d[ch, first:last + L], L)[::step]
                assert win.shape[0] == ks.size
                if normalize == "full":
                    m = win.mean(axis=1)
                    cen = win - m[:, None]
                    num = cen @ tp[t, ch]
                    ssd = np.sum(cen * cen, axis=1)
                else:
                    num = win @ tp[t, ch]
                    ssd = np.sum(win * win, axis=1)
                den = sst[ch] * ssd
                keep = (den > THRESHOLD) if threshold == "product" else (np.sqrt(den) > THRESHOLD)
                cc = np.where(keep, num / np.sqrt(np.where(keep, den, 1.0)), 0.0)
                if network_sum:
                    acc += w[t, ch] * cc
                else:
                    out[oi, c0 - k0:c1 - k0, ch] = cc
            if network_sum:
                out[oi, c0 - k0:c1 - k0] = acc
    if not network_sum:
        out = out.reshape(len(tix), K, S, C)
    return out


def fp64_matched_filter_variable(templates, n_samples_template, moveouts, weights, data, step,
                                 normalize="short", k_range=None, chunk=16384):
    """FP64 evaluation of the per-channel-length search (the reference's
    arch='variable_precise', matched_filter.c:321-412, 569-606): channel ch of
    template t uses its first n[t, ch] taps; per output the Fisher-z network
    sum sum_ch atanh(cc_ch - 10 eps) * z_ch with z_ch = sqrt(n - 3) * w_ch,
    then (tanh(sum / sum_ch z_ch) + n_used * 10 eps) * scale[t], where scale[t]
    is the running sum of the weights of templates 0..t (never reset in the
    reference, matched_filter.c:329,365).  Valid outputs: start <= k*step <
    N - L - max_mo - step (matched_filter.c:381-382), L the longest channel;
    the transform also maps the zeros outside that range.  cc uses the
    'precise' threshold sqrt(sst * ssd) > 1e-6 (matched_filter.c:650-652);
    sst is the raw sum of the channel's own taps squared.  Returns float64
    (T, K) for the outputs of k_range (default all n_corr)."""
    eps = float(np.finfo(np.float32).eps)
    templates = np.asarray(templates, dtype=np.float32)
    T, S, C, L = templates.shape
    N = data.shape[-1]
    nch = S * C
    n_corr = int((N - L) / step + 1)
    k0, k1 = (0, n_corr) if k_range is None else k_range
    tp = templates.reshape(T, nch, L).astype(np.float64)
    nt = np.asarray(n_samples_template).reshape(T, nch).astype(np.int64)
    mo = np.asarray(moveouts).reshape(T, nch).astype(np.int64)
    w = np.asarray(weights, dtype=np.float32).reshape(T, nch).astype(np.float64)
    d = np.asarray(data, dtype=np.float32).reshape(nch, N).astype(np.float64)
    out = np.zeros((T, k1 - k0))
    scale = np.cumsum(w.sum(axis=1))
    for t in range(T):
        z = np.sqrt(nt[t] - 3.0) * w[t]
        used = int(np.count_nonzero(w[t]))
        lo, hi = min(0, int(mo[t].min())), max(0, int(mo[t].max()))
        start = int(np.ceil(abs(lo) / float(step))) * step
        stop = N - L - hi - step
        a = max(k0, -(-start // step))
        b = min(k1, -(-stop // step) if stop > start else a)
        acc = np.zeros(k1 - k0)
        for c0 in range(a, b, chunk):
            c1 = min(b, c0 + chunk)
            part = np.zeros(c1 - c0)
            for ch in range(nch):
                if w[t, ch] == 0.0:
                    continue
                n = int(nt[t, ch])
                x = tp[t, ch, :n]
                first = c0 * step + mo[t, ch]
                last = (c1 - 1) * step + mo[t, ch]
                win = sliding_window_view(d[ch, first:last + n], n)[::step]
                if normalize == "full":
                    win = win - win.mean(axis=1)[:, None]
                num = win @ x
                den = np.sqrt(np.sum(x * x) * np.sum(win * win, axis=1))
                cc = np.where(den > THRESHOLD, num / np.where(den > THRESHOLD, den, 1.0), 0.0)
                part += np.arctanh(cc - 10 * eps) * z[ch]
            acc[c0 - k0:c1 - k0] = part
        out[t] = (np.tanh(acc / z.sum()) + used * eps * 10) * scale[t]
    return out
