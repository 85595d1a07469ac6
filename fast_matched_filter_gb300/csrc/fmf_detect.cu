// fmf_detect.cu -- detection on network-summed correlation rows, on the GPU.
//
// The callers of the matched filter threshold each template's summed cc
// trace and pick its peaks.  Done on the host this needs the whole (T, n_corr)
// result copied out (8.6 GB for 500 templates over a day at 100 Hz); done
// here only the detections leave the device.  There is no reference
// counterpart: the semantics are the usual robust threshold and scipy's peak
// finder, so a caller's numpy/scipy code gives the same answers.
//
// For each template row cc[t][0:n_corr) and its lag window [begin_t, end_t):
//   median = numpy.median of the window (float32: the mean of the two middle
//            values, summed in float32, for an even count)
//   mad    = numpy.median of |x - median| (float32 differences)
//   thr    = median + n_mad * mad (float32; multiply, then add -- no fused
//            multiply-add)
//   peaks  = scipy.signal.find_peaks(window, height=thr, distance=min_separation):
//            local maxima (a flat top counts once, at its middle sample rounded
//            down; the window's first and last samples never count) whose value
//            is >= thr; then, from the highest down (equal heights: the later lag
//            first), each peak still kept removes the peaks closer than
//            min_separation lags on either side.
//
// The order statistics are exact.  Each (median, then MAD) is a sample-select:
//   1. one block per row sorts a strided sample of the row's 32-bit
//      order-preserving keys and brackets the two middle ranks with a key
//      window [klo, khi] six binomial standard deviations wide;
//   2. one pass over the row counts the keys below klo and gathers the keys
//      inside the window (about 5 % of the row) into a candidate list;
//   3. if the window holds both middle ranks, a radix selection (three passes
//      of 11, 11 and 10 bits, each a shared-memory histogram of the keys that
//      match the bits chosen so far) runs over the candidates only; if not --
//      heavy ties, an adversarial row -- the same radix selection runs over
//      the whole row.  Rows no longer than the sample are sorted whole.
// The MAD pass's read of the row also notes the values at or above a lower
// bound of the threshold (from the MAD window: thr = med + n_mad * mad is
// monotone in mad) in a hot list, whose local maxima a small kernel gathers,
// so a call reads the rows twice (median, MAD + peaks) in the usual case; rows
// whose MAD window missed get a peak pass of their own.  Peaks are gathered
// into a list per template (capacity kDetCap) and filtered by one thread
// block per template: the candidates below the exact threshold dropped, a
// sort by lag, a sort by height, and the greedy distance filter.
//
// Every launch is stream-ordered and the state lives on the device, so a
// detection run needs no host round trip and can be captured in a graph.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "fmf_common.cuh"

namespace fmf {
namespace {

constexpr int kDetBins = 2048;            // histogram bins of the 11-bit passes
constexpr int kDetThreads = 256;          // histogram / peak kernels
constexpr int kDetSelectThreads = 1024;   // per-template filter kernel
constexpr int kDetChunk = 1024;           // templates per round of scratch
constexpr int kDetCap = 16384;            // candidate peaks per template row
constexpr int kDetSample = 16384;         // sampled keys per row (sample-select)

// source of a row's radix selection
constexpr int kSrcRow = 0;   // the row itself (fallback)
constexpr int kSrcCand = 1;  // the candidate keys gathered by det_count_kernel
constexpr int kSrcDone = 2;  // already exact (the row was sorted whole)

struct DetState {
    int begin, end;        // lag window of the row
    unsigned prefix[2];    // key bits chosen so far for the lower / upper middle rank
    int rank[2];           // rank still to find inside the chosen bucket
    float med, mad, thr;
    int n_cand;            // local maxima at or above thr (may exceed the capacity)
    float thr_lo;          // a lower bound of thr known before the MAD pass
    int peaks_ready;       // 1: the MAD counting pass noted the values >= thr_lo
    int n_hot;             // values >= thr_lo noted (may exceed the capacity)
    int src;               // kSrcRow / kSrcCand / kSrcDone
    unsigned klo, khi;     // sample window of the keys
    int n_lt, n_in;        // keys below klo, keys inside [klo, khi]
};

// Order-preserving image of a float: a < b  <=>  key(a) < key(b) (for non-NaN
// values; -0 sorts just below +0).
__device__ __forceinline__ unsigned order_key(float x)
{
    const unsigned u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_value(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Digit of pass p: bits [shift, shift + width) of the key.
__device__ __forceinline__ int pass_shift(int p) { return p == 0 ? 21 : (p == 1 ? 10 : 0); }
__device__ __forceinline__ unsigned pass_bins(int p) { return p == 2 ? 1024u : 2048u; }
__device__ __forceinline__ unsigned pass_high_mask(int p)
{
    return p == 0 ? 0u : (p == 1 ? 0xffe00000u : 0xfffffc00u);
}

// Split of a row at its first 16-byte boundary: `head` scalar elements, then
// `nvec` float4s, then `tail` scalar elements.
struct RowSplit {
    long long head, nvec, tail;
};

__device__ __forceinline__ RowSplit split_row(const float *row, long long n)
{
    RowSplit r;
    r.head = (long long)(((16u - ((unsigned)(size_t)row & 15u)) & 15u) >> 2);
    if (r.head > n)
        r.head = n;
    r.nvec = (n - r.head) >> 2;
    r.tail = n - r.head - 4 * r.nvec;
    return r;
}

__global__ void det_init_kernel(DetState *__restrict__ st, int T, int n_corr,
                                const int *__restrict__ begin, const int *__restrict__ end)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T)
        return;
    int b = 0, e = n_corr;
    if (begin) {
        b = min(max(begin[t], 0), n_corr);
        e = min(max(end[t], b), n_corr);
    }
    const int n = e - b;
    DetState s;
    s.begin = b;
    s.end = e;
    s.prefix[0] = s.prefix[1] = 0u;
    s.rank[0] = n > 0 ? (n - 1) / 2 : 0;
    s.rank[1] = n / 2;
    s.med = s.mad = s.thr = __int_as_float(0x7fc00000);  // NaN until computed
    s.n_cand = 0;
    s.thr_lo = __int_as_float(0x7fc00000);
    s.peaks_ready = 0;
    s.n_hot = 0;
    s.src = kSrcRow;
    s.klo = s.khi = 0u;
    s.n_lt = s.n_in = 0;
    st[t] = s;
}

// Key of a row value: mode 0 the value, mode 1 |value - median| (float32).
__device__ __forceinline__ unsigned sel_key(float v, int mode, float med)
{
    return order_key(mode == 0 ? v : fabsf(__fsub_rn(v, med)));
}

// The value of the two middle keys, as numpy's median of float32 data.
__device__ __forceinline__ float middle_value(unsigned ka, unsigned kb, int n)
{
    const float a = key_value(ka), b = key_value(kb);
    return (n & 1) ? a : __fmul_rn(__fadd_rn(a, b), 0.5f);
}

__device__ __forceinline__ void finish_select(DetState &s, int mode, float v, float n_mad)
{
    if (mode == 0) {
        s.med = v;
    } else {
        s.mad = v;
        s.thr = __fadd_rn(s.med, __fmul_rn(n_mad, v));
    }
}

// The key of rank r (0-based, ascending) among the first P keys of sk, by the
// block: three radix passes (11, 11 and 10 bits), each a shared-memory
// histogram of the keys that match the bits chosen so far, then one warp
// finding the bucket that holds the rank.  All threads of the block call it.
__device__ unsigned block_select(const unsigned *sk, int P, int r, unsigned *hist, int *shared_pick)
{
    unsigned prefix = 0u;
    for (int pass = 0; pass < 3; pass++) {
        const int shift = pass_shift(pass);
        const unsigned bins = pass_bins(pass), high = pass_high_mask(pass);
        for (int i = threadIdx.x; i < (int)bins; i += blockDim.x)
            hist[i] = 0u;
        __syncthreads();
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            const unsigned k = sk[i];
            if ((k & high) == prefix)
                atomicAdd(&hist[(k >> shift) & (bins - 1u)], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x, per = (int)bins / 32;
            unsigned sum = 0;
            for (int i = 0; i < per; i++)
                sum += hist[lane * per + i];
            unsigned inc = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o)
                    inc += y;
            }
            const unsigned exc = inc - sum;
            if ((unsigned)r >= exc && (unsigned)r < inc) {
                unsigned c = exc;
                int i = 0;
                for (; i < per - 1; i++) {
                    if ((unsigned)r < c + hist[lane * per + i])
                        break;
                    c += hist[lane * per + i];
                }
                shared_pick[0] = lane * per + i;
                shared_pick[1] = (int)c;
            }
        }
        __syncthreads();
        prefix |= (unsigned)shared_pick[0] << shift;
        r -= shared_pick[1];
        __syncthreads();
    }
    return prefix;
}

// Step 1 of the sample-select (one block per row): a strided sample of the
// row's keys, sorted; either the exact answer (row no longer than the
// sample) or the key window around the two middle ranks.
__global__ void __launch_bounds__(1024)
det_sample_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st, int mode,
                  float n_mad, float *__restrict__ saved)
{
    extern __shared__ unsigned long long sample_smem[];
    unsigned *sk = reinterpret_cast<unsigned *>(sample_smem);  // kDetSample keys
    const int t = blockIdx.x;
    DetState s = st[t];
    const long long n = s.end - s.begin;
    if (n <= 0)
        return;
    const float *row = cc + (size_t)t * ld + s.begin;
    const int m = n < kDetSample ? (int)n : kDetSample;
    int P = 1;
    while (P < m)
        P <<= 1;
    // sample positions floor(i * n / m) from a fixed-point step (no 64-bit division
    // per sample); any spread of positions serves, the selection is exact.  The
    // median pass gathers the sampled values from the row (scattered reads) and
    // keeps them in `saved`; the MAD pass reads them back contiguously.
    const unsigned long long stepq = ((unsigned long long)n << 20) / (unsigned long long)m;
    float *sv = saved + (size_t)t * kDetSample;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        unsigned key = 0xffffffffu;
        if (i < m) {
            float v;
            if (mode == 0) {
                long long pos = (long long)(((unsigned long long)i * stepq) >> 20);
                v = row[pos < n ? pos : n - 1];
                sv[i] = v;
            } else {
                v = sv[i];
            }
            key = sel_key(v, mode, s.med);
        }
        sk[i] = key;
    }
    __syncthreads();
    // two order statistics of the sample (the padding keys, all ones, rank last):
    // the exact middle values when the sample is the whole row; otherwise the keys
    // bracketing the two middle ranks -- the sample position of rank r is about
    // r*m/n, with a binomial standard deviation of at most sqrt(m)/2 = 64 positions:
    // bracket by 6 of them
    __shared__ unsigned hist[kDetBins];
    __shared__ int pick[2];
    const long long a = (n - 1) / 2, b = n / 2;
    constexpr int kPad = 6 * 64 + 16;
    const long long pa = a * m / n, pb = (b * m + n - 1) / n;
    const int r0 = m == n ? (int)a : (int)(pa - kPad > 0 ? pa - kPad : 0);
    const int r1 = m == n ? (int)b : (int)(pb + kPad < m - 1 ? pb + kPad : m - 1);
    const unsigned k0 = block_select(sk, P, r0, hist, pick);
    const unsigned k1 = r1 == r0 ? k0 : block_select(sk, P, r1, hist, pick);
    if (threadIdx.x != 0)
        return;
    s.prefix[0] = s.prefix[1] = 0u;
    s.rank[0] = (int)a;
    s.rank[1] = (int)b;
    s.n_lt = s.n_in = 0;
    if (m == n) {  // the whole row
        finish_select(s, mode, middle_value(k0, k1, (int)n), n_mad);
        s.src = kSrcDone;
    } else {
        s.klo = k0;
        s.khi = k1;
        s.src = kSrcCand;
        if (mode == 1) {
            // thr = med + n_mad * mad rises with mad (for n_mad >= 0; falls otherwise) and
            // float rounding keeps that order, so a MAD inside the window [klo, khi] gives
            // thr >= thr_lo: the counting pass gathers the local maxima >= thr_lo, a
            // superset of the peaks, and the filter keeps those >= thr
            const float d = key_value(n_mad >= 0.0f ? k0 : k1);
            s.thr_lo = __fadd_rn(s.med, __fmul_rn(n_mad, d));
            s.peaks_ready = 1;
        }
    }
    st[t] = s;
}

// A local maximum at row[i] = x (absolute index i in the window [b, e))
// at or above thr, appended (unordered) to the template's candidate list.
__device__ __forceinline__ void peak_at(const float *row, long long i, long long b, long long e, float x,
                                        float thr, DetState *st, int2 *cand, int cap, int t)
{
    if (!(x >= thr) || i < b + 1 || i >= e - 1)
        return;  // a flat top has the value of its rising sample
    if (!(row[i - 1] < x))
        return;
    long long j = i + 1;
    while (j < e - 1 && row[j] == x)
        j++;
    if (row[j] < x) {
        const int peak = (int)((i + j - 1) >> 1);
        const int slot = atomicAdd(&st[t].n_cand, 1);
        if (slot < cap)
            cand[(size_t)t * cap + slot] = make_int2(peak, __float_as_int(x));
    }
}

// A value of row t at window offset o at or above thr_lo, noted in the row's
// hot list (the rare path of the MAD counting pass: one atomic, one store;
// det_hot_kernel examines the neighbours later).
__device__ __forceinline__ void note_hot(DetState *st, int t, long long o, int *hot, int cap)
{
    const int slot = atomicAdd(&st[t].n_hot, 1);
    if (slot < cap)
        hot[(size_t)t * cap + slot] = (int)o;
}

// Step 2: one pass over the row: keys below klo counted, keys inside
// [klo, khi] appended to the row's candidate list (up to cap).  In the MAD
// pass (mode 1, PEAKS) the same read notes the offsets of the values at or
// above thr_lo in the row's hot list, so that no third read of the row is
// needed for the peaks.
template <bool PEAKS>
__global__ void __launch_bounds__(kDetThreads, 4)  // 32 warps per SM: enough loads in flight
det_count_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st,
                 unsigned *__restrict__ cand, long long cap, int mode, int *__restrict__ hot,
                 int hcap)
{
    const int t = blockIdx.y;
    const int src = st[t].src;
    const long long n = st[t].end - st[t].begin;
    if (src != kSrcCand || n <= 0)
        return;
    const unsigned klo = st[t].klo, khi = st[t].khi;
    const float med = st[t].med;
    const bool peaks = PEAKS && mode == 1 && st[t].peaks_ready != 0;
    const float thr_lo = st[t].thr_lo;
    const float *row = cc + (size_t)t * ld + st[t].begin;
    unsigned *list = cand + (size_t)t * cap;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kWarps = kDetThreads / 32;
    unsigned lt = 0;  // per-lane count of keys below klo
    // One warp step: each lane's up to 16 keys; the keys inside the window are
    // appended with one atomic per warp (a warp prefix sum places them).
    constexpr int kK = 16;
    const unsigned width = khi - klo;  // key - klo <= width  <=>  klo <= key <= khi
    // a lane's keys inside the window wait here (its own column), so that only
    // the few candidates are written out, in a loop over the set bits
    __shared__ unsigned stash[kWarps][kK][32];
    auto take = [&](const unsigned (&key)[kK], const bool (&ok)[kK], auto all_ok) {
        constexpr bool ALL = decltype(all_ok)::value;  // every key of the step is in the row
        unsigned in_mask = 0;
#pragma unroll
        for (int u = 0; u < kK; u++) {
            const bool o = ALL || ok[u];
            lt += (o && key[u] < klo) ? 1u : 0u;
            if (o && key[u] - klo <= width) {
                in_mask |= 1u << u;
                stash[warp][u][lane] = key[u];
            }
        }
        const int cnt = __popc(in_mask);
        int inc = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o)
                inc += y;
        }
        const int total = __shfl_sync(0xffffffffu, inc, 31);
        if (total == 0)
            return;
        int base = 0;
        if (lane == 31)
            base = atomicAdd(&st[t].n_in, total);
        base = __shfl_sync(0xffffffffu, base, 31);
        long long pos = (long long)base + inc - cnt;
        for (unsigned m = in_mask; m; m &= m - 1u, pos++)
            if (pos < cap)
                list[pos] = stash[warp][__ffs(m) - 1][lane];
    };
    const RowSplit rs = split_row(row, n);
    if (blockIdx.x == 0 && warp == 0) {
        unsigned key[kK];
        bool ok[kK];
        const long long i = lane < rs.head ? lane : rs.head + 4 * rs.nvec + (lane - rs.head);
        ok[0] = lane < rs.head + rs.tail;
        const float x = ok[0] ? row[i] : 0.0f;
        key[0] = ok[0] ? sel_key(x, mode, med) : 0u;
        if (peaks && ok[0] && x >= thr_lo)
            note_hot(st, t, i, hot, hcap);
#pragma unroll
        for (int u = 1; u < kK; u++) {
            ok[u] = false;
            key[u] = 0u;
        }
        take(key, ok, std::false_type{});
    }
    const float4 *vrow = reinterpret_cast<const float4 *>(row + rs.head);
    const long long steps = (rs.nvec + 127) / 128;  // 128 float4s per warp step
    const long long cstride = (long long)gridDim.x * kWarps;
    auto load4 = [&](long long c, float4 (&v)[4]) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long i = c * 128 + u * 32 + lane;
            v[u] = (c < steps && i < rs.nvec) ? vrow[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    float4 nv[4];
    long long c = (long long)blockIdx.x * kWarps + warp;
    load4(c, nv);
    for (; c < steps; c += cstride) {
        unsigned key[kK];
        bool ok[kK];
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
            v[u] = nv[u];
        load4(c + cstride, nv);  // the next step's values are in flight while this one is counted
        if (peaks) {  // values at or above thr_lo (rare)
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const long long q = c * 128 + u * 32 + lane;
                const float mx = fmaxf(fmaxf(v[u].x, v[u].y), fmaxf(v[u].z, v[u].w));
                if (q < rs.nvec && mx >= thr_lo) {
                    const long long o = rs.head + 4 * q;
                    if (v[u].x >= thr_lo)
                        note_hot(st, t, o, hot, hcap);
                    if (v[u].y >= thr_lo)
                        note_hot(st, t, o + 1, hot, hcap);
                    if (v[u].z >= thr_lo)
                        note_hot(st, t, o + 2, hot, hcap);
                    if (v[u].w >= thr_lo)
                        note_hot(st, t, o + 3, hot, hcap);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const bool okv = c * 128 + u * 32 + lane < rs.nvec;
            key[4 * u + 0] = sel_key(v[u].x, mode, med);
            key[4 * u + 1] = sel_key(v[u].y, mode, med);
            key[4 * u + 2] = sel_key(v[u].z, mode, med);
            key[4 * u + 3] = sel_key(v[u].w, mode, med);
            ok[4 * u + 0] = ok[4 * u + 1] = ok[4 * u + 2] = ok[4 * u + 3] = okv;
        }
        if (c * 128 + 128 <= rs.nvec)  // a whole step inside the row (warp-uniform)
            take(key, ok, std::true_type{});
        else
            take(key, ok, std::false_type{});
    }
    for (int o = 16; o > 0; o >>= 1)
        lt += __shfl_down_sync(0xffffffffu, lt, o);
    if (lane == 0 && lt)
        atomicAdd(&st[t].n_lt, (int)lt);
}

// Step 3: does the window hold both middle ranks?  Then select among the
// candidates; else fall back to the whole row -- and in the MAD pass, leave
// the peaks to a pass of their own (the gathered superset may miss some, or
// have overflowed its list).
__global__ void det_check_kernel(DetState *__restrict__ st, int T, long long cap, int mode, int pcap)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T || st[t].src != kSrcCand)
        return;
    DetState s = st[t];
    const long long n = s.end - s.begin;
    const long long a = (n - 1) / 2, b = n / 2;
    if (s.n_in <= cap && s.n_lt <= a && b < (long long)s.n_lt + s.n_in) {
        s.rank[0] = (int)(a - s.n_lt);
        s.rank[1] = (int)(b - s.n_lt);
    } else {
        s.src = kSrcRow;
        s.rank[0] = (int)a;
        s.rank[1] = (int)b;
        if (mode == 1)
            s.peaks_ready = 0;
    }
    if (mode == 1 && (!s.peaks_ready || s.n_hot > pcap)) {
        s.peaks_ready = 0;
        s.n_cand = 0;
    }
    s.prefix[0] = s.prefix[1] = 0u;
    st[t] = s;
}

// Histogram update by a whole warp: every lane calls it (lanes whose value
// does not count pass ok = false); lanes with the same digit add once.
// With `aggregate` (the first pass, whose keys share few digits) lanes with
// the same digit add once; otherwise (later passes, digits spread) each lane
// adds its own count.
__device__ __forceinline__ void hist_add(unsigned *h, float v, bool ok, int mode, float med, int shift,
                                         unsigned dmask, unsigned high, unsigned p0, unsigned p1,
                                         bool two, int lane, bool aggregate)
{
    const unsigned key = mode == 2 ? __float_as_uint(v) : sel_key(v, mode, med);
    const unsigned dig = (key >> shift) & dmask;
    const bool m0 = ok && (key & high) == p0;
    const bool m1 = two && ok && (key & high) == p1;
    if (!aggregate) {
        if (m0)
            atomicAdd(&h[dig], 1u);
        if (m1)
            atomicAdd(&h[kDetBins + dig], 1u);
        return;
    }
    if (__any_sync(0xffffffffu, m0)) {
        const unsigned g = __match_any_sync(0xffffffffu, m0 ? dig : 0xffffffffu);
        if (m0 && (__ffs(g) - 1) == lane)
            atomicAdd(&h[dig], __popc(g));
    }
    if (two) {
        if (__any_sync(0xffffffffu, m1)) {
            const unsigned g = __match_any_sync(0xffffffffu, m1 ? dig : 0xffffffffu);
            if (m1 && (__ffs(g) - 1) == lane)
                atomicAdd(&h[kDetBins + dig], __popc(g));
        }
    }
}

// One selection pass: histogram of the current digit over the elements whose
// higher key bits equal a rank's prefix.  mode 0 keys the values, mode 1 keys
// |x - median|.  Grid: (blocks per row, templates).  The row is read with
// 16-byte loads, two per lane in flight per step.
__global__ void __launch_bounds__(kDetThreads)
det_hist_kernel(const float *__restrict__ cc, size_t ld, const DetState *__restrict__ st,
                unsigned *__restrict__ hist, const unsigned *__restrict__ cand, long long cap, int pass,
                int mode)
{
    __shared__ unsigned h[2 * kDetBins];
    const int t = blockIdx.y;
    const DetState s = st[t];
    if (s.src == kSrcDone || s.end - s.begin <= 0)
        return;  // uniform over the block, before any barrier
    const bool keys = s.src == kSrcCand;  // candidate keys instead of row values
    const long long n = keys ? s.n_in : s.end - s.begin;
    for (int i = threadIdx.x; i < 2 * kDetBins; i += kDetThreads)
        h[i] = 0u;
    __syncthreads();
    const int shift = pass_shift(pass);
    const unsigned dmask = pass_bins(pass) - 1u;
    const unsigned high = pass_high_mask(pass);
    const unsigned p0 = s.prefix[0], p1 = s.prefix[1];
    const bool two = p0 != p1;  // the two middle ranks sit in different buckets
    const float med = s.med;
    // candidate keys are stored as the bits of a float whose order key they
    // are: key_value() turns them back, so both sources run the same code
    const float *row = keys ? reinterpret_cast<const float *>(cand + (size_t)t * cap)
                            : cc + (size_t)t * ld + s.begin;
    const int kmode = keys ? 2 : mode;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    constexpr int kWarps = kDetThreads / 32;
    const RowSplit rs = split_row(row, n);
    if (blockIdx.x == 0 && warp == 0) {  // the unaligned ends, at most 3 + 3 values
        const long long i = lane < rs.head ? lane : rs.head + 4 * rs.nvec + (lane - rs.head);
        const bool ok = lane < rs.head + rs.tail;
        const float v = ok ? row[i] : 0.f;
        hist_add(h, v, ok, kmode, med, shift, dmask, high, p0, p1, two, lane, pass == 0);
    }
    const float4 *vrow = reinterpret_cast<const float4 *>(row + rs.head);
    const long long steps = (rs.nvec + 63) / 64;  // 64 float4s per warp step
    for (long long c = (long long)blockIdx.x * kWarps + warp; c < steps; c += (long long)gridDim.x * kWarps) {
        float4 v[2];
        bool ok[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const long long i = c * 64 + u * 32 + lane;
            ok[u] = i < rs.nvec;
            v[u] = ok[u] ? vrow[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            hist_add(h, v[u].x, ok[u], kmode, med, shift, dmask, high, p0, p1, two, lane, pass == 0);
            hist_add(h, v[u].y, ok[u], kmode, med, shift, dmask, high, p0, p1, two, lane, pass == 0);
            hist_add(h, v[u].z, ok[u], kmode, med, shift, dmask, high, p0, p1, two, lane, pass == 0);
            hist_add(h, v[u].w, ok[u], kmode, med, shift, dmask, high, p0, p1, two, lane, pass == 0);
        }
    }
    __syncthreads();
    unsigned *gh = hist + (size_t)t * 2 * kDetBins;
    for (int i = threadIdx.x; i < (two ? 2 : 1) * kDetBins; i += kDetThreads) {
        const unsigned c = h[i];
        if (c)
            atomicAdd(gh + i, c);
    }
}

// Picks each rank's bucket from the pass's histogram (one warp per template),
// clears the histogram, and after the last pass turns the two keys into the
// median (mode 0) or the MAD and the threshold (mode 1).
__global__ void det_resolve_kernel(DetState *__restrict__ st, unsigned *__restrict__ hist, int pass,
                                   int mode, float n_mad)
{
    const int t = blockIdx.x;
    const int lane = threadIdx.x;
    DetState s = st[t];
    const int n = s.end - s.begin;
    if (n <= 0 || s.src == kSrcDone)
        return;
    unsigned *gh = hist + (size_t)t * 2 * kDetBins;
    const int per = (int)pass_bins(pass) / 32;  // bins per lane
    const int shift = pass_shift(pass);
    const bool two = s.prefix[0] != s.prefix[1];
    for (int r = 0; r < 2; r++) {
        const unsigned *h = gh + (two ? r : 0) * kDetBins;
        unsigned sum = 0;
        for (int i = 0; i < per; i++)
            sum += h[lane * per + i];
        unsigned inc = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o)
                inc += y;
        }
        const unsigned exc = inc - sum;
        const unsigned rk = (unsigned)s.rank[r];
        const unsigned found = __ballot_sync(0xffffffffu, rk >= exc && rk < inc);
        const int src = found ? __ffs(found) - 1 : 0;
        unsigned bin = 0, before = 0;
        if (lane == src) {
            unsigned c = exc;
            int i = 0;
            for (; i < per - 1; i++) {
                const unsigned hv = h[lane * per + i];
                if (rk < c + hv)
                    break;
                c += hv;
            }
            bin = (unsigned)(lane * per + i);
            before = c;
        }
        bin = __shfl_sync(0xffffffffu, bin, src);
        before = __shfl_sync(0xffffffffu, before, src);
        s.prefix[r] |= bin << shift;
        s.rank[r] = (int)(rk - before);
    }
    __syncwarp();
    for (int i = lane; i < 2 * kDetBins; i += 32)
        gh[i] = 0u;
    if (pass == 2)
        finish_select(s, mode, middle_value(s.prefix[0], s.prefix[1], n), n_mad);
    if (lane == 0)
        st[t] = s;
}

// The local maxima among a row's hot values (at or above thr_lo), one block
// per row: appended to the candidate list, a superset of the peaks that the
// select kernel filters by the exact threshold.  A superset that overflows
// the list hands the row to det_peaks_kernel (exact threshold).
__global__ void __launch_bounds__(kDetThreads)
det_hot_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st,
               const int *__restrict__ hot, int hcap, int2 *__restrict__ cand, int cap)
{
    const int t = blockIdx.x;
    if (!st[t].peaks_ready)
        return;  // uniform over the block
    const long long b = st[t].begin, e = st[t].end;
    const float thr_lo = st[t].thr_lo;
    const float *row = cc + (size_t)t * ld;
    const int n = min(st[t].n_hot, hcap);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const long long i = b + hot[(size_t)t * hcap + j];
        peak_at(row, i, b, e, row[i], thr_lo, st, cand, cap, t);
    }
    __syncthreads();
    if (threadIdx.x == 0 && st[t].n_cand > cap) {
        st[t].peaks_ready = 0;
        st[t].n_cand = 0;
    }
}

// Local maxima at or above the threshold, appended (unordered) to the
// template's candidate list, for the rows whose MAD pass did not gather them
// (rows sorted whole by the sample, MAD windows that missed, overflowing
// supersets).  Grid: (blocks per row, templates).  Samples are read with
// 16-byte loads; the rare sample at or above the threshold is examined with
// scalar loads.
__global__ void __launch_bounds__(kDetThreads)
det_peaks_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st,
                 int2 *__restrict__ cand, int cap)
{
    const int t = blockIdx.y;
    const long long b = st[t].begin, e = st[t].end;
    const float thr = st[t].thr;
    if (e - b < 3 || st[t].peaks_ready)
        return;
    const float *row = cc + (size_t)t * ld;
    const RowSplit rs = split_row(row + b, e - b);
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gtid < rs.head + rs.tail) {
        const long long i = b + (gtid < rs.head ? gtid : rs.head + 4 * rs.nvec + (gtid - rs.head));
        peak_at(row, i, b, e, row[i], thr, st, cand, cap, t);
    }
    const float4 *vrow = reinterpret_cast<const float4 *>(row + b + rs.head);
    const long long base = b + rs.head;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = gtid; v < rs.nvec; v += 2 * stride) {
        const float4 x0 = vrow[v];
        const bool has1 = v + stride < rs.nvec;
        const float4 x1 = has1 ? vrow[v + stride] : make_float4(0.f, 0.f, 0.f, 0.f);
        const long long i0 = base + 4 * v, i1 = base + 4 * (v + stride);
        peak_at(row, i0, b, e, x0.x, thr, st, cand, cap, t);
        peak_at(row, i0 + 1, b, e, x0.y, thr, st, cand, cap, t);
        peak_at(row, i0 + 2, b, e, x0.z, thr, st, cand, cap, t);
        peak_at(row, i0 + 3, b, e, x0.w, thr, st, cand, cap, t);
        if (has1) {
            peak_at(row, i1, b, e, x1.x, thr, st, cand, cap, t);
            peak_at(row, i1 + 1, b, e, x1.y, thr, st, cand, cap, t);
            peak_at(row, i1 + 2, b, e, x1.z, thr, st, cand, cap, t);
            peak_at(row, i1 + 3, b, e, x1.w, thr, st, cand, cap, t);
        }
    }
}

// Ascending bitonic sort of P (a power of two) keys in shared memory.
__device__ void bitonic_sort(unsigned long long *a, int P)
{
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long x = a[i], y = a[l];
                    if ((x > y) == ((i & k) == 0)) {
                        a[i] = y;
                        a[l] = x;
                    }
                }
            }
            __syncthreads();
        }
}

// Distance filter and output of one template (one block per template).
// Shared memory: keys (8 B), lags (4 B) and keep flags (1 B) per candidate.
__global__ void __launch_bounds__(kDetSelectThreads)
det_select_kernel(const DetState *__restrict__ st, const int2 *__restrict__ cand, int cap, int min_sep,
                  int max_det, float *med_out, float *mad_out, float *thr_out, int *count_out,
                  int *lag_out, float *val_out)
{
    extern __shared__ unsigned long long sk[];
    int *lag = reinterpret_cast<int *>(sk + cap);
    unsigned char *keep = reinterpret_cast<unsigned char *>(lag + cap);
    __shared__ int warp_tot[kDetSelectThreads / 32];
    const int t = blockIdx.x;
    const DetState s = st[t];
    if (threadIdx.x == 0) {
        if (med_out)
            med_out[t] = s.med;
        if (mad_out)
            mad_out[t] = s.mad;
        if (thr_out)
            thr_out[t] = s.thr;
    }
    const int m0 = s.n_cand;
    if (m0 > cap) {
        if (threadIdx.x == 0)
            count_out[t] = -1;  // capacity exceeded: no peaks reported for this row
        return;
    }
    int P = 1;
    while (P < m0)
        P <<= 1;
    const int2 *c = cand + (size_t)t * cap;
    // 1. the candidates at or above thr (the MAD pass gathers a superset: those at or
    // above a lower bound of thr), ordered by lag (lags are distinct); the others
    // sort last
    int kept = 0;
    for (int i0 = 0; i0 < P; i0 += blockDim.x) {
        const int i = i0 + threadIdx.x;
        const bool ok = i < m0 && __int_as_float(c[i].y) >= s.thr;
        if (i < P)
            sk[i] = ok ? ((unsigned long long)(unsigned)c[i].x << 32) | (unsigned)c[i].y : ~0ull;
        kept += __syncthreads_count(ok);
    }
    const int m = kept;
    bitonic_sort(sk, P);
    // 2. order by height, then by lag (position in lag order)
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const unsigned long long k = sk[i];
        if (i < m) {
            lag[i] = (int)(k >> 32);
            keep[i] = 1;
            sk[i] = ((unsigned long long)order_key(__uint_as_float((unsigned)k)) << 32) | (unsigned)i;
        } else {
            sk[i] = 0ull;
        }
    }
    __syncthreads();
    bitonic_sort(sk, P);
    // 3. greedy from the highest: each kept peak removes its close neighbours
    if (threadIdx.x == 0) {
        for (int q = P - 1; q >= P - m; q--) {
            const int j = (int)(unsigned)sk[q];
            if (!keep[j])
                continue;
            const int lj = lag[j];
            for (int k = j - 1; k >= 0 && lj - lag[k] < min_sep; k--)
                keep[k] = 0;
            for (int k = j + 1; k < m && lag[k] - lj < min_sep; k++)
                keep[k] = 0;
        }
    }
    __syncthreads();
    // 4. values back into lag order (sk[j] = value bits of the peak at lag position j)
    constexpr int kPer = 16;  // P <= 16384 = kPer * kDetSelectThreads
    unsigned long long held[kPer];
#pragma unroll
    for (int u = 0; u < kPer; u++) {
        const int q = threadIdx.x + u * kDetSelectThreads;
        held[u] = q < P ? sk[q] : 0ull;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPer; u++) {
        const int q = threadIdx.x + u * kDetSelectThreads;
        if (q < P && q >= P - m) {
            const int j = (int)(unsigned)held[u];
            sk[j] = __float_as_uint(key_value((unsigned)(held[u] >> 32)));
        }
    }
    __syncthreads();
    // 5. kept peaks in lag order: block-wide exclusive scan of the keep flags
    const int span = (m + kDetSelectThreads - 1) / kDetSelectThreads;
    const int i0 = threadIdx.x * span, i1 = min(i0 + span, m);
    int cnt = 0;
    for (int i = i0; i < i1; i++)
        cnt += keep[i];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o)
            inc += y;
    }
    if (lane == 31)
        warp_tot[wid] = inc;
    __syncthreads();
    int base = 0, total = 0;
    for (int w = 0; w < kDetSelectThreads / 32; w++) {
        if (w < wid)
            base += warp_tot[w];
        total += warp_tot[w];
    }
    int pos = base + inc - cnt;
    for (int i = i0; i < i1; i++) {
        if (!keep[i])
            continue;
        if (pos < max_det) {
            lag_out[(size_t)t * max_det + pos] = lag[i];
            val_out[(size_t)t * max_det + pos] = __uint_as_float((unsigned)sk[i]);
        }
        pos++;
    }
    if (threadIdx.x == 0)
        count_out[t] = total;
}

size_t select_smem(int cap) { return (size_t)cap * (8 + 4 + 1); }

}  // namespace

// Detection over T rows of device-resident cc (row stride ld floats), every
// pointer a device pointer.  Stream-ordered; no host synchronisation.
int detect_device(const float *cc, int T, int n_corr, size_t ld, const int *begin, const int *end,
                  float n_mad, int min_sep, int max_det, float *med_out, float *mad_out,
                  float *thr_out, int *count_out, int *lag_out, float *val_out, Scratch &ws,
                  cudaStream_t s)
{
    int rc;
    const int chunk = T < kDetChunk ? T : kDetChunk;
    DetState *st;
    unsigned *hist, *keys;
    int2 *cand;
    int *hot;
    float *saved;
    // candidate keys per row: the sample window holds about 5 % of a row
    const long long key_cap = n_corr < 65536 ? n_corr : std::max(65536LL, (long long)n_corr / 8);
    if ((rc = ws.get(&st, (size_t)chunk, "detection state")) ||
        (rc = ws.get(&hist, (size_t)chunk * 2 * kDetBins, "detection histograms")) ||
        (rc = ws.get(&keys, (size_t)chunk * key_cap, "candidate keys")) ||
        (rc = ws.get(&cand, (size_t)chunk * kDetCap, "candidate peaks")) ||
        (rc = ws.get(&hot, (size_t)chunk * kDetCap, "values above the threshold bound")) ||
        (rc = ws.get(&saved, (size_t)chunk * kDetSample, "sampled values")))
        return rc;
    cudaError_t e = cudaFuncSetAttribute(det_select_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)select_smem(kDetCap));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(det_sample_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(kDetSample * sizeof(unsigned)));
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "detection shared memory: %s", cudaGetErrorString(e));
    if ((e = cudaMemsetAsync(hist, 0, (size_t)chunk * 2 * kDetBins * sizeof(unsigned), s)) != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "clearing the detection histograms: %s", cudaGetErrorString(e));
    for (int t0 = 0; t0 < T; t0 += chunk) {
        const int nt = T - t0 < chunk ? T - t0 : chunk;
        const float *rows = cc + (size_t)t0 * ld;
        // enough blocks per row to fill the 152 SMs (8 resident blocks each) about eight
        // times over, so that the last, partial wave of blocks costs little
        long long per_row = (152LL * 8 * 8 + nt - 1) / nt;
        const long long row_cap = ((long long)n_corr + 1023) / 1024;
        if (per_row > row_cap)
            per_row = row_cap;
        if (per_row < 1)
            per_row = 1;
        const dim3 grid((unsigned)per_row, (unsigned)nt);
        det_init_kernel<<<(nt + 127) / 128, 128, 0, s>>>(st, nt, n_corr, begin ? begin + t0 : nullptr,
                                                         end ? end + t0 : nullptr);
        for (int mode = 0; mode < 2; mode++) {
            det_sample_kernel<<<nt, 1024, kDetSample * sizeof(unsigned), s>>>(rows, ld, st, mode, n_mad,
                                                                               saved);
            if (mode == 1)
                det_count_kernel<true><<<grid, kDetThreads, 0, s>>>(rows, ld, st, keys, key_cap, mode,
                                                                    hot, kDetCap);
            else
                det_count_kernel<false><<<grid, kDetThreads, 0, s>>>(rows, ld, st, keys, key_cap, mode,
                                                                     hot, kDetCap);
            det_check_kernel<<<(nt + 127) / 128, 128, 0, s>>>(st, nt, key_cap, mode, kDetCap);
            for (int pass = 0; pass < 3; pass++) {
                det_hist_kernel<<<grid, kDetThreads, 0, s>>>(rows, ld, st, hist, keys, key_cap, pass,
                                                             mode);
                det_resolve_kernel<<<nt, 32, 0, s>>>(st, hist, pass, mode, n_mad);
            }
        }
        det_hot_kernel<<<nt, kDetThreads, 0, s>>>(rows, ld, st, hot, kDetCap, cand, kDetCap);
        det_peaks_kernel<<<grid, kDetThreads, 0, s>>>(rows, ld, st, cand, kDetCap);
        det_select_kernel<<<nt, kDetSelectThreads, select_smem(kDetCap), s>>>(
            st, cand, kDetCap, min_sep, max_det, med_out ? med_out + t0 : nullptr,
            mad_out ? mad_out + t0 : nullptr, thr_out ? thr_out + t0 : nullptr, count_out + t0,
            lag_out + (size_t)t0 * max_det, val_out + (size_t)t0 * max_det);
        count_launch(22);
        if ((rc = check_launch("detection kernels")))
            return rc;
    }
    return FMF_OK;
}

int validate_detect(size_t T, size_t n_corr, float n_mad, size_t min_sep, size_t max_det,
                    const void *count_out, const void *lag_out, const void *val_out)
{
    if (T < 1 || n_corr < 1)
        return set_error(FMF_ERR_ARG, "detection: sizes must be positive (T=%zu n_corr=%zu)", T, n_corr);
    if (T > (size_t)INT_MAX || n_corr > (size_t)INT_MAX || max_det > (size_t)INT_MAX / 2 ||
        min_sep > (size_t)INT_MAX)
        return set_error(FMF_ERR_ARG, "detection: sizes exceed the 32-bit index range");
    if (min_sep < 1)
        return set_error(FMF_ERR_ARG, "detection: min_separation must be at least 1");
    if (!std::isfinite(n_mad))
        return set_error(FMF_ERR_ARG, "detection: n_mad must be finite");
    if (!count_out || (max_det > 0 && (!lag_out || !val_out)))
        return set_error(FMF_ERR_ARG, "detection: null output array");
    return FMF_OK;
}

// Host copies of the detection outputs: counts of -1 (capacity exceeded) turn
// into an error status.
int detect_finish_host(const int *count_host, size_t T)
{
    for (size_t t = 0; t < T; t++)
        if (count_host[t] < 0)
            return set_error(FMF_ERR_UNSUPPORTED,
                             "detection: template %zu has more than %d local maxima above its threshold; "
                             "raise n_mad",
                             t, kDetCap);
    return FMF_OK;
}

int detect_capacity() { return kDetCap; }

}  // namespace fmf
