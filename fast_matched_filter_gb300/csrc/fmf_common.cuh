// fmf_common.cuh -- shared definitions of the GB300 matched-filter library.
//
// Terminology follows the reference (fast_matched_filter): a *template* t has
// one waveform per *channel* ch = station * C + component; the *moveout*
// mo[t][ch] shifts that channel's waveform in the continuous *data*; output
// index k ("lag") correlates template t against data samples
// k*step + mo[t][ch] + [0, L) of every channel.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/fmf_gb300.h"

namespace fmf {

// Stability threshold of the reference (matched_filter.cu:22, matched_filter.c:17):
// a channel contributes only when sst * (window energy) exceeds it.
constexpr float kThreshold = 0.000001f;

// Device view of one matched-filter problem.  Channel-major arrays are
// indexed [t][ch] (T x SC) or [ch][sample] (SC x N).
struct Problem {
    const float *tpl;     // (T, SC, L) templates; centred per channel for "full"
    const float *sst;     // (T, SC) caller-supplied sum of squares (raw templates)
    const float *tsum;    // (T, SC) sum of the centred template ("full"), else null
    const int *mo;        // (T, SC) moveouts
    const float *w;       // (T, SC) weights
    const float *data;    // (SC, N) data; centred per channel for "full"
    const float *stat_e;  // short: (SC, N) window energy; full: (SC, N) float pairs (centred
                          // energy, centred mean), one 8-byte load per lag; window starts at the index
    const int *k_lo;      // (T) first valid output index
    const int *k_hi;      // (T) one past the last valid output index (<= n_corr)
    float *out;           // (T, n_corr) or (T, n_corr, SC)
    int T, SC, L, N, step, n_corr;
    int normalize;        // 0 short, 1 full
    int network_sum;      // 1 weighted sum over channels, 0 per channel
    // Per-channel template lengths (Fisher-z network sum), else null:
    const int *ntap;      // (T, SC) taps of each channel (templates zero-padded to L)
    const long long *pre2q; // (SC, N+1) running sums of d^2 (centred d for full), exact, in units
                            // unit2[ch] (64-bit fixed point)
    const float *unit2;     // (SC) the fixed-point unit of each channel's running sums, a power of two
    const float2 *pre1f;    // (SC, N+1) running sums of centred d as hi + lo floats (full), else null
    const float *zweight; // (T, SC) Fisher-z weight of each channel
    // (T) each, or null: when set, the tensor-core kernel writes
    // (tanh(x / vp_norm[t]) + vp_bias[t]) * vp_scale[t] for every output x
    const float *vp_norm, *vp_bias, *vp_scale;
};

#ifdef __CUDACC__
// Window sums of a per-channel length n from running sums: of d^2 as exact
// 64-bit fixed point (the difference of two is exact), of d as float pairs
// P = hi + lo (hi = fl(P), lo = fl(P - hi), ~48 significant bits).

// a - b = s + e exactly (Knuth's TwoSum on a and -b).
__device__ __forceinline__ float two_diff(float a, float b, float &e)
{
    const float s = a - b, bb = s - a;
    e = (a - (s - bb)) - (b + bb);
    return s;
}

// (h, l) += (xh, xl): TwoSum of the high words, every rounding error and the
// low words accumulated in l (not renormalised).
__device__ __forceinline__ void pair_add(float &h, float &l, float xh, float xl)
{
    const float s = h + xh, bb = s - h;
    l += ((h - (s - bb)) + (xh - bb)) + xl;
    h = s;
}

// The pair (h, l) as hi = fl(h + l), lo = the rest (|h| >= |l|).
__device__ __forceinline__ float2 pair_normalise(float h, float l)
{
    const float hi = h + l;
    return make_float2(hi, l - (hi - h));
}

// A non-negative 64-bit integer d < 2^63 as a normalised float pair h + l
// (about 48 significant bits) with FP32/INT32 operations only: its 23-bit
// digits become exact floats by the 2^23 magic-number trick, the top two are
// added by TwoSum and the low one joins the error word.  (Forming the pair with
// int64 <-> float conversions takes three of them, which run at a fraction of
// the FP32 rate: the 'full' per-channel-length search ran 95 TMAC/s with them,
// 124 with this.)
__device__ __forceinline__ void fixed_pair(long long d, float &h, float &l)
{
    const unsigned long long x = d > 0 ? (unsigned long long)d : 0ull;
    const unsigned lo = (unsigned)x & 0x7fffffu, mid = (unsigned)(x >> 23) & 0x7fffffu;
    const unsigned top = (unsigned)(x >> 46);  // < 2^17
    const float magic = 8388608.0f;           // 2^23
    const float fl = __int_as_float(0x4b000000u | lo) - magic;
    const float fm = (__int_as_float(0x4b000000u | mid) - magic) * magic;
    const float ft = (__int_as_float(0x4b000000u | top) - magic) * (magic * magic);
    float e;
    const float s = two_diff(ft, -fm, e);  // ft + fm = s + e exactly
    const float t = e + fl;
    h = s + t;
    l = t - (h - s);
}

// 'short': sum of d^2 over the window [a, b) from the fixed-point running sums
// (one rounding: the conversion instruction is cheaper here than the split).
__device__ __forceinline__ float window_energy(long long pa, long long pb, float unit)
{
    return __ll2float_rn(pb - pa) * unit;
}

// 'full': centred energy v = S2 - S1^2 / n and mean S1 / n of a window whose
// sums are the float pairs S2 = s2h + s2l (of d^2) and S1 = s1h + s1l (of d),
// with S1^2 / n carried as an unevaluated float pair too (TwoSum, and FMA for
// the exact square and division residuals), so that v keeps float accuracy
// even when the window mean dominates (S2 / v large).
__device__ __forceinline__ void window_centred_sums(float s2h, float s2l, float s1h, float s1l,
                                                    float nf, float inv_n, float &v, float &mean)
{
    const float h = s1h + s1l, l = s1l - (h - s1h);  // S1 = h + l, |l| <= ulp(h) / 2
    mean = h * inv_n;
    const float p = h * h;
    const float pe = fmaf(2.0f * h, l, fmaf(h, h, -p));  // S1^2 = p + pe (+ l^2)
    const float qh = p * inv_n;
    const float ql = (fmaf(-qh, nf, p) + pe) * inv_n;    // S1^2 / n = qh + ql
    float ev;
    const float vh = two_diff(s2h, qh, ev);
    const float r = vh + ((ev + s2l) - ql);
    v = r > 0.0f ? r : 0.0f;
}

// The same from running sums: of d^2 in fixed point (a2, b2; the exact
// difference taken as a float pair), of d as float pairs (a1, b1).
__device__ __forceinline__ void window_centred(long long a2, long long b2, float unit, float2 a1,
                                               float2 b1, float nf, float inv_n, float &v, float &mean)
{
    float dh, dl;
    fixed_pair(b2 - a2, dh, dl);
    const float s2h = dh * unit, s2l = dl * unit;
    float e1;
    const float s1h = two_diff(b1.x, a1.x, e1);
    const float s1l = e1 + (b1.y - a1.y);
    window_centred_sums(s2h, s2l, s1h, s1l, nf, inv_n, v, mean);
}
#endif

}  // namespace fmf

// ---------------------------------------------------------------------------
// Host-side helpers shared by the translation units (defined in fmf_api.cu).
namespace fmf {
int set_error(int status, const char *fmt, ...);
void count_launch(int n = 1);
void reset_launch_count();  // at the start of every entry point (fmf_last_launch_count)
void keep_pool_cached();    // at the start of every entry point that allocates scratch
int check_launch(const char *what);
// The dynamic shared memory every variable-size kernel is allowed: the
// attribute is set to the largest a CTA may have, never to one call's need, so
// that calls from several host threads with different needs cannot lower it
// under one another's launch.
constexpr int kMaxDynamicSmem = 227 * 1024;
// Maps the host pages of a result buffer for writing before a copy into it
// (parallel; a no-op where the kernel refuses).
void populate_host(void *p, size_t bytes);
bool host_is_pinned(const void *p);  // page-locked or registered host memory

// Stream-ordered scratch allocations (cudaMallocAsync from the device's
// default pool).  The pool keeps freed blocks for reuse by later calls;
// fmf_release_cache() trims it.  Everything is freed, in stream order, when
// the Scratch goes out of scope.
struct Scratch {
    cudaStream_t s;
    std::vector<void *> ptr;
    explicit Scratch(cudaStream_t st) : s(st) {}
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    template <class T>
    int get(T **out, size_t count, const char *what)
    {
        void *p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, count * sizeof(T) + 16, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(e == cudaErrorMemoryAllocation ? FMF_ERR_OOM : FMF_ERR_CUDA,
                             "allocating %zu bytes for %s: %s", count * sizeof(T), what,
                             cudaGetErrorString(e));
        }
        ptr.push_back(p);
        *out = static_cast<T *>(p);
        return FMF_OK;
    }
    ~Scratch()
    {
        for (void *p : ptr)
            cudaFreeAsync(p, s);
    }
};

// Preprocessing shared by every form: per-template lag ranges, 'full'
// centring, double-float window statistics (fmf_api.cu).  Fills the epilogue fields of
// *P and the data the numerator kernels read (centred for 'full').
struct Args {
    const float *tpl, *sst, *data, *w;
    const int *mo;
    float *out;
    size_t step, L, N, T, S, C, n_corr;
    int normalize, sum_mode, precision, flags;
    // check_zeros count (optional): per template, the outputs equal to 0
    // whose last-axis index is below zero_stop (host or device pointer, as
    // the other arrays)
    unsigned long long *zero_counts = nullptr;
    long long zero_stop = 0;
};
int validate_args(const Args &a);
// Window statistics of every channel (fmf_prep.cu): blocks of kStatWindows
// windows; the shared memory a launch needs, and the launch itself.
constexpr int kStatWindows = 4096;
size_t window_stats_smem(int L, bool full);
int launch_window_stats(const float *data, int N, int L, int SC, const float *mu, float *dcen,
                        float *stat_e, cudaStream_t s);
int prepare_problem(const Args &a, Scratch &ws, cudaStream_t s, Problem *P, const float **data_for_tc);

// Tensor-core form (fmf_tc.cu).
constexpr int TC_MAX_PROBS = 64;
struct TcProb;
int tc_choose_nb(int L, int step, int split, int forced);
int tc_prepare(const Problem &P, const float *data_for_tc, int split, int nb, int tg, Scratch &ws,
               cudaStream_t s, TcProb *out);
int tc_run(const TcProb *probs, int n, int split, unsigned long long *queue, unsigned *err,
           cudaStream_t s);
size_t tc_prob_size();
void tc_subset(const TcProb *full, int t0, int nt, TcProb *out);
int launch_plain(const Problem &P, cudaStream_t stream);
int launch_plain_all(const Problem &P, cudaStream_t stream);
// FMF_PREC_AUTO: the precision a prepared search runs in (fmf_auto.cu); waits on s.
int choose_auto_precision(const Problem &P, Scratch &ws, cudaStream_t s, int *precision);
void set_last_precision(int precision);
int device_error_word(unsigned **out);

// Detection on network-summed rows (fmf_detect.cu).
int detect_device(const float *cc, int T, int n_corr, size_t ld, const int *begin, const int *end,
                  float n_mad, int min_sep, int max_det, float *med_out, float *mad_out,
                  float *thr_out, int *count_out, int *lag_out, float *val_out, Scratch &ws,
                  cudaStream_t s);
int validate_detect(size_t T, size_t n_corr, float n_mad, size_t min_sep, size_t max_det,
                    const void *count_out, const void *lag_out, const void *val_out);
int detect_finish_host(const int *count_host, size_t T);
int detect_capacity();
}  // namespace fmf
