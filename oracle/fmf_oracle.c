/*
 * fmf_oracle.c -- CPU restatement of the reference matched-filter algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is linked by the
 * parity tests, by the smoke check and by the benchmark's CPU-baseline leg.
 * Nothing in the product (fast_matched_filter_gb300) loads it.
 *
 * It restates, in plain C99 + OpenMP, the arithmetic of the reference CPU
 * library fast_matched_filter/src/matched_filter.c (abbreviated MF.c below):
 *
 *   - "cpu" arch   : per-channel FP64 compensated prefix sums of d^2
 *                    (MF.c:660-705), FP32 numerator, denominator
 *                    sst * (float)(window energy), threshold on the product
 *                    (MF.c:611-627), weighted FP32 network sum
 *                    (MF.c:416-455), lag range per template (MF.c:53-92).
 *   - "precise"    : FP32 window mean (normalize=1) and FP32 sum of squares
 *                    recomputed for every lag (MF.c:629-657), threshold on
 *                    sqrt(sst * ssd) (MF.c:650-652), network sum
 *                    (MF.c:457-494).
 *   - no-sum       : per-channel coefficients written at [t][lag][channel]
 *                    (MF.c:170-319, MF.c:496-567).
 *
 * Floating-point order follows the reference exactly: sequential FP32
 * accumulation in tap order, channels in station-major / component-minor
 * order.  The reference is built with gcc -O3 -march=native (Makefile:38);
 * on an FMA-capable x86-64 host that build computes the tap products of its
 * per-channel sums in vector registers (each product rounded, then added in
 * tap order) and finishes the last L mod 4 taps with scalar fused
 * multiply-adds; its network-sum update (cc_sum += cc * w, MF.c:450) is
 * fused.  This file is compiled with -ffp-contract=off and writes exactly
 * those fusions as fmaf(), so it reproduces that build bit for bit on
 * x86-64 and on aarch64 without host-specific flags.
 *
 * Lags outside a template's valid range are left untouched (callers pass a
 * zeroed buffer, as the reference wrapper does: fast_matched_filter.py:269-274).
 */
#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define FMO_THRESHOLD 0.000001f /* MF.c:17 */

/* Compensated running sum of squares with a leading zero entry:
 * out[0] = 0, out[k] = sum_{j<k} x[j]^2 (k = 1..n).  Restates
 * neumaier_cumsum_squared (MF.c:680-705) and the leading-zero layout of
 * cumsum_square_data (MF.c:660-677).  The branch test compares magnitudes
 * after conversion to float, as the reference's fabsf() call does. */
void fmo_cumsum_sq(const float *x, size_t n, double *out)
{
    out[0] = 0.0;
    if (n == 0)
        return;
    double run = (double)x[0] * (double)x[0];
    double comp = 0.0;
    out[1] = run;
    for (size_t k = 1; k < n; k++) {
        double sq = (double)x[k] * (double)x[k];
        double nxt = run + sq;
        if (fabsf((float)run) >= fabsf((float)sq))
            comp += (run - nxt) + sq;
        else
            comp += (sq - nxt) + run;
        run = nxt;
        out[k + 1] = nxt + comp;
    }
}

/* Short normalisation with prefix-sum energy (MF.c:611-627).  e0/e1 are the
 * prefix entries bracketing the window. */
static float corr_prefix(const float *tpl, float sst, const float *d,
                         double e0, double e1, size_t L)
{
    const size_t Lv = L - (L & 3);
    float num = 0.0f;
    for (size_t j = 0; j < Lv; j++)
        num += tpl[j] * d[j];
    for (size_t j = Lv; j < L; j++)
        num = fmaf(tpl[j], d[j], num);
    float den = sst * (float)(e1 - e0);
    if (den > FMO_THRESHOLD)
        return (float)((double)num / sqrt((double)den));
    return 0.0f;
}

/* Direct recomputation with optional window-mean removal (MF.c:629-657). */
static float corr_direct(const float *tpl, float sst, const float *d,
                         size_t L, int normalize)
{
    float mean = 0.0f;
    if (normalize > 0) {
        for (size_t j = 0; j < L; j++)
            mean += d[j];
        mean /= (float)L;
    }
    const size_t Lv = L - (L & 3);
    float num = 0.0f, ssd = 0.0f;
    for (size_t j = 0; j < Lv; j++) {
        float v = d[j] - mean;
        num += tpl[j] * v;
        ssd += v * v;
    }
    for (size_t j = Lv; j < L; j++) {
        float v = d[j] - mean;
        num = fmaf(tpl[j], v, num);
        ssd = fmaf(v, v, ssd);
    }
    float den = (float)sqrt((double)(sst * ssd));
    if (den > FMO_THRESHOLD)
        return num / den;
    return 0.0f;
}

/* Valid lag range of one template (MF.c:53-76): samples i = start, start+step,
 * ... < stop.  Returns 0 when the template has no valid lag (the reference
 * would wrap an unsigned subtraction there). */
static int lag_range(const int *mo, size_t nch, size_t step, size_t L,
                     size_t N, size_t *start, size_t *stop)
{
    int lo = 0, hi = 0;
    for (size_t ch = 0; ch < nch; ch++) {
        if (mo[ch] < lo)
            lo = mo[ch];
        if (mo[ch] > hi)
            hi = mo[ch];
    }
    *start = lo < 0 ? (size_t)ceilf(-lo / (float)step) * step : 0;
    if ((long long)N - (long long)L - (long long)hi < 0)
        return 0;
    *stop = 1 + (N - L - (size_t)hi);
    return *start < *stop;
}

/* One call of the reference library.
 *   arch 0 = "cpu"     (prefix-sum energy; normalize must be 0)
 *   arch 1 = "precise" (direct sums; normalize 0 = short, 1 = full)
 *   network_sum 1 -> cc is (T, n_corr); 0 -> cc is (T, n_corr, S*C)
 *   n_threads <= 0 -> OpenMP default.
 * Returns 0 on success, -1 on bad arguments or allocation failure. */
int fmo_matched_filter(const float *templates, const float *sst,
                       const int *moveouts, const float *data,
                       const float *weights, size_t step, size_t L,
                       size_t N, size_t T, size_t S, size_t C,
                       size_t n_corr, float *cc, int arch, int normalize,
                       int network_sum, int n_threads)
{
    const size_t nch = S * C;
    if (step == 0 || L == 0 || nch == 0 || (arch == 0 && normalize != 0))
        return -1;
#ifdef _OPENMP
    if (n_threads > 0)
        omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    double *csum = NULL;
    if (arch == 0) {
        csum = (double *)malloc(nch * (N + 1) * sizeof(double));
        if (!csum)
            return -1;
#pragma omp parallel for
        for (long long ch = 0; ch < (long long)nch; ch++)
            fmo_cumsum_sq(data + (size_t)ch * N, N, csum + (size_t)ch * (N + 1));
    }
    for (size_t t = 0; t < T; t++) {
        const int *mo = moveouts + t * nch;
        const float *w = weights + t * nch;
        const float *ss = sst + t * nch;
        const float *tp = templates + t * nch * L;
        size_t start, stop;
        if (!lag_range(mo, nch, step, L, N, &start, &stop))
            continue;
        long long n_lags = (long long)((stop - start + step - 1) / step);
#pragma omp parallel for
        for (long long k = 0; k < n_lags; k++) {
            size_t i = start + (size_t)k * step;
            size_t out = i / step;
            float acc = 0.0f;
            for (size_t ch = 0; ch < nch; ch++) {
                if (w[ch] == 0.0f)
                    continue;
                size_t off = i + (size_t)((long long)mo[ch]);
                const float *d = data + ch * N + off;
                float v;
                if (arch == 0) {
                    const double *cs = csum + ch * (N + 1) + off;
                    v = corr_prefix(tp + ch * L, ss[ch], d, cs[0], cs[L], L);
                } else {
                    v = corr_direct(tp + ch * L, ss[ch], d, L, normalize);
                }
                if (network_sum)
                    acc = fmaf(v, w[ch], acc);
                else
                    cc[(t * n_corr + out) * nch + ch] = v;
            }
            if (network_sum)
                cc[t * n_corr + out] = acc;
        }
    }
    free(csum);
    return 0;
}

/* Per-channel template lengths with a Fisher-z network sum: restates
 * matched_filter_variable_precise (MF.c:321-412) and
 * network_corr_variable_precise (MF.c:569-606).  Templates are stored with
 * stride max(n_tpl); channel ch of template t uses its first n_tpl[t][ch]
 * taps and the 'precise' correlation (MF.c:629-657).  Reproduced exactly,
 * including two properties of the reference: the scale max_cc accumulates
 * the weights of every template up to and including t (it is never reset,
 * MF.c:329,365), and the final tanh transform is applied to every output,
 * also outside the lag range (MF.c:405-408).
 * Returns 0, or -1 on bad arguments. */
int fmo_matched_filter_variable(const float *templates, const float *sst,
                                const int *moveouts, const float *data,
                                const float *weights, size_t step,
                                const int *n_tpl, size_t N, size_t T,
                                size_t S, size_t C, size_t n_corr, float *cc,
                                int normalize, int n_threads)
{
    const size_t nch = S * C;
    if (step == 0 || nch == 0)
        return -1;
#ifdef _OPENMP
    if (n_threads > 0)
        omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    float *cc_norm = (float *)malloc(nch * sizeof(float));
    if (!cc_norm)
        return -1;
    int max_len = 0;
    for (size_t k = 0; k < T * nch; k++)
        if (n_tpl[k] > max_len)
            max_len = n_tpl[k];
    float max_cc = 0.0f;
    for (size_t t = 0; t < T; t++) {
        const int *mo = moveouts + t * nch;
        const float *w = weights + t * nch;
        const float *ss = sst + t * nch;
        const int *nt = n_tpl + t * nch;
        const float *tp = templates + t * nch * (size_t)max_len;
        int lo = 0, hi = 0, used = 0;
        for (size_t ch = 0; ch < nch; ch++) {
            if (mo[ch] < lo)
                lo = mo[ch];
            if (mo[ch] > hi)
                hi = mo[ch];
            max_cc += w[ch];
            if (w[ch] != 0.0f)
                used += 1;
        }
        float norm_sum = 0.0f;
        for (size_t ch = 0; ch < nch; ch++) {
            cc_norm[ch] = (float)(1.0 / (double)sqrtf((float)(1.0 / (double)(nt[ch] - 3))) * (double)w[ch]);
            norm_sum += cc_norm[ch];
        }
        const size_t start = (size_t)(int)(ceilf(abs(lo) / (float)step)) * step;
        const long long stop = (long long)N - max_len - hi - (long long)step;
        long long n_lags = stop > (long long)start ? (stop - (long long)start + (long long)step - 1) / (long long)step : 0;
#pragma omp parallel for
        for (long long k = 0; k < n_lags; k++) {
            size_t i = start + (size_t)k * step;
            float acc = 0.0f;
            for (size_t ch = 0; ch < nch; ch++) {
                if (w[ch] == 0.0f)
                    continue;
                size_t off = i + (size_t)((long long)mo[ch]);
                float v = corr_direct(tp + ch * (size_t)max_len, ss[ch], data + ch * N + off,
                                      (size_t)nt[ch], normalize);
                acc = fmaf(atanhf(v - 10 * FLT_EPSILON), cc_norm[ch], acc);
            }
            cc[t * n_corr + i / step] = acc;
        }
        const float bias = used * FLT_EPSILON * 10;
#pragma omp parallel for
        for (long long i = 0; i < (long long)n_corr; i++)
            cc[t * n_corr + i] = (tanhf(cc[t * n_corr + i] / norm_sum) + bias) * max_cc;
    }
    free(cc_norm);
    return 0;
}

/* Number of OpenMP threads a parallel region would use (for reporting). */
int fmo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
