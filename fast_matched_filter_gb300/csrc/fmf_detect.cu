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
// The order statistics are exact, from one read of each row in the usual
// case (a sample-select):
//   1. one block per row sorts a strided sample of the row: the key window
//      [klo, khi] around the two middle ranks (three binomial standard
//      deviations wide), so the median lies in [m_lo, m_hi], the values of
//      those keys; and from the sample's |x - m| about the window's middle, a
//      window [a_lo, a_hi] the MAD lies in, widened a little for the median's
//      own uncertainty;
//   2. one pass over the row counts the keys below klo and gathers the keys
//      inside [klo, khi] (about 2.5 % of the row), and classifies every value
//      for the MAD before the median is known: |x - m| < a_lo for every m in
//      [m_lo, m_hi] (counted), |x - m| > a_hi for every such m (dropped), or
//      either (listed: about 7 % of a Gaussian row); the same read notes the
//      values at or above a lower bound of the threshold
//      (m_lo + n_mad * a_lo: thr = med + n_mad * mad is monotone in both);
//   3. the median: if the window holds both middle ranks, a radix selection
//      over the candidates (passes of up to 11 bits over the key bits the
//      window's keys do not share, each a shared-memory histogram of the keys
//      that match the bits chosen so far); if not -- a window that missed
//      (about one row in 800), heavy ties, an adversarial row -- the same
//      selection over the whole row, by a fixed grid of blocks over the list
//      of such rows, so that the row is read at the rate of the whole GPU;
//   4. the MAD: the sample keyed by |x - med| narrows [a_lo, a_hi]; the listed
//      values keyed by |x - med| are counted below the window or gathered in
//      it, and selected as in 3.  A row whose median or MAD window missed, or
//      whose list overflowed, selects its MAD over the whole row and takes its
//      peaks in a pass of its own.  Rows no longer than the sample are sorted
//      whole.
// The values noted in step 2 are examined by a small kernel for the local
// maximum and plateau rules: a superset of the peaks, gathered into a list
// per template (capacity kDetCap) and filtered by one thread block per
// template: the candidates below the exact threshold dropped, a sort by lag,
// a sort by height, and the greedy distance filter.
//
// Every launch is stream-ordered and the state lives on the device, so a
// detection run needs no host round trip and can be captured in a graph.
#include <algorithm>
#include <cmath>

#include "fmf_common.cuh"

namespace fmf {
namespace {

constexpr int kDetBins = 2048;            // histogram bins of the 11-bit passes
constexpr int kDetThreads = 256;          // histogram / peak kernels
constexpr int kDetSelectThreads = 1024;   // per-template filter kernel
constexpr int kDetChunk = 1024;           // templates per round of scratch
constexpr int kDetCap = 16384;            // candidate peaks per template row
constexpr int kDetSample = 16384;         // sampled keys per row (sample-select)
constexpr int kDetBlocks = 152 * 8 * 8;   // blocks of a row pass: 8 waves of 8 per SM
constexpr int kSpill = 16;                // rows past a column's capacity (one step's appends)
constexpr int kDetRowBlocks = 152 * 4;    // the fixed grid of the passes over rows that fell back

// source of a row's radix selection
constexpr int kSrcRow = 0;   // the row itself (fallback)
constexpr int kSrcCand = 1;  // the candidate keys gathered by det_count_kernel
constexpr int kSrcDone = 2;  // already exact (the row was sorted whole)

struct DetState {
    int begin, end;        // lag window of the row
    unsigned prefix[2];    // key bits chosen so far for the lower / upper middle rank
    int rank[2];           // rank still to find inside the chosen bucket
    int top;               // key bits below the window's common high bits (0..32)
    float med, mad, thr;
    int n_cand;            // local maxima at or above thr (may exceed the capacity)
    float thr_lo;          // a lower bound of thr known before the counting pass
    int peaks_ready;       // 1: the counting pass noted the values >= thr_lo
    int n_hot;             // values >= thr_lo noted (may exceed the capacity)
    int src;               // kSrcRow / kSrcCand / kSrcDone
    unsigned klo, khi;     // key window of the current selection
    int n_lt, n_in;        // keys below klo, keys inside [klo, khi]
    // the MAD classes of the counting pass (one_read = 1): the median lies in
    // [m_lo, m_hi] and the MAD in [a_lo, a_hi] when both windows hold
    int one_read;
    float m_lo, m_hi, a_lo, a_hi;
    int has_below;         // [kb0, kb1] is not empty
    unsigned kb0, kb1;     // value keys with |x - m| < a_lo for every m in [m_lo, m_hi]
    unsigned kn0, kn1;     // value keys with |x - m| <= a_hi for some m in [m_lo, m_hi]
    int n_below;           // values in [kb0, kb1]
    int over_k, over_a;    // a lane's column of candidates / undecided values overflowed
};

// The lists of a row are written in columns, one per thread of the counting
// pass, so that appending takes no scan and no shared counter: thread l of
// warp w of block b puts its k-th entry at list + t * cap + ((b * 8 + w) *
// (C + kSpill) + k) * 32 + (l & 31), up to C entries (rows C.. of the warp's
// region take a step's overflow, unread), and its count at
// cnt[(t * S + b) * 256 + l] (more than C: overflowed).  Equal counts across a
// warp make coalesced stores and loads.
struct Lanes {
    int S;                 // counting blocks per row
    int Ck, Ca;            // column capacity: candidates of a selection / undecided values
    int *cnt_k, *cnt_a;    // entries per column (may exceed the capacity)
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

// Digit of selection pass p over the low `top` bits of the keys (the bits
// above are common to every key selected among): up to 11 bits at a time from
// the top; width 0 once the key is complete.
__device__ __forceinline__ void pass_digit(int top, int p, int &shift, int &width)
{
    int hi = top;
    shift = hi;
    width = 0;
    for (int q = 0; q <= p; q++) {
        width = hi < 11 ? hi : 11;
        shift = hi - width;
        hi = shift;
    }
}

// The bits at and above `bit` (none for bit 32).
__device__ __forceinline__ unsigned above_mask(int bit) { return bit >= 32 ? 0u : ~0u << bit; }

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
    s.top = 32;
    s.med = s.mad = s.thr = __int_as_float(0x7fc00000);  // NaN until computed
    s.n_cand = 0;
    s.thr_lo = __int_as_float(0x7fc00000);
    s.peaks_ready = 0;
    s.n_hot = 0;
    s.src = kSrcRow;
    s.klo = s.khi = 0u;
    s.n_lt = s.n_in = 0;
    s.one_read = 0;
    s.m_lo = s.m_hi = s.a_lo = s.a_hi = 0.0f;
    s.has_below = 0;
    s.kb0 = s.kb1 = s.kn0 = s.kn1 = 0u;
    s.n_below = 0;
    s.over_k = s.over_a = 0;
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

// The keys of ranks r0 <= r1 (0-based, ascending) among the first P keys of
// sk, by the block: three radix passes (11, 11 and 10 bits), each a
// shared-memory histogram per rank of the keys that match that rank's bits so
// far (one histogram while both ranks share them; warp-aggregated in the
// first pass, whose digits sampled keys mostly share), then one warp per rank
// finding the bucket that holds it.  All threads of the block call it.
__device__ void block_select2(const unsigned *sk, int P, int r0, int r1, unsigned *hist, int *pick,
                              unsigned &k0, unsigned &k1)
{
    unsigned pre[2] = {0u, 0u};
    int r[2] = {r0, r1};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int pass = 0; pass < 3; pass++) {
        int shift, width;
        pass_digit(32, pass, shift, width);
        const unsigned dmask = (1u << width) - 1u, high = above_mask(shift + width);
        const bool two = pre[0] != pre[1];
        for (int i = threadIdx.x; i < 2 * kDetBins; i += blockDim.x)
            hist[i] = 0u;
        __syncthreads();
        for (int i0 = 0; i0 < P; i0 += blockDim.x) {  // every lane runs every step
            const int i = i0 + threadIdx.x;
            const unsigned k = i < P ? sk[i] : 0u;
            const unsigned dig = (k >> shift) & dmask;
            for (int q = 0; q < (two ? 2 : 1); q++) {
                const bool m = i < P && (k & high) == pre[q];
                if (pass == 0) {
                    const unsigned g = __match_any_sync(0xffffffffu, m ? dig : 0xffffffffu);
                    if (m && (__ffs(g) - 1) == lane)
                        atomicAdd(&hist[q * kDetBins + dig], __popc(g));
                } else if (m) {
                    atomicAdd(&hist[q * kDetBins + dig], 1u);
                }
            }
        }
        __syncthreads();
        if (warp < 2) {
            const unsigned *h = hist + (two ? warp : 0) * kDetBins;
            const int per = kDetBins / 32;
            unsigned sum = 0;
            for (int i = 0; i < per; i++)
                sum += h[lane * per + i];
            unsigned inc = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o)
                    inc += y;
            }
            const unsigned exc = inc - sum, rk = (unsigned)(warp == 0 ? r[0] : r[1]);
            if (rk >= exc && rk < inc) {
                unsigned c = exc;
                int i = 0;
                for (; i < per - 1; i++) {
                    if (rk < c + h[lane * per + i])
                        break;
                    c += h[lane * per + i];
                }
                pick[2 * warp] = lane * per + i;
                pick[2 * warp + 1] = (int)c;
            }
        }
        __syncthreads();
        for (int q = 0; q < 2; q++) {
            pre[q] |= (unsigned)pick[2 * q] << shift;
            r[q] -= pick[2 * q + 1];
        }
        __syncthreads();
    }
    k0 = pre[0];
    k1 = pre[1];
}

// |x - m| in float32, as numpy computes the MAD's deviations.
__device__ __forceinline__ float dev(float x, float m) { return fabsf(__fsub_rn(x, m)); }

// |x - m| < a for every float m in [m_lo, m_hi]: |x - m| falls, then rises,
// in m (float rounding keeps both monotone), so the larger of the ends.
__device__ __forceinline__ bool below_all(float x, float m_lo, float m_hi, float a)
{
    return dev(x, m_lo) < a && dev(x, m_hi) < a;
}

// |x - m| <= a for some float m in [m_lo, m_hi]: 0 inside, else the nearer end.
__device__ __forceinline__ bool near_some(float x, float m_lo, float m_hi, float a)
{
    if (x < m_lo)
        return __fsub_rn(m_lo, x) <= a;
    if (x > m_hi)
        return __fsub_rn(x, m_hi) <= a;
    return x == x;  // inside (NaN is not)
}

// Both predicates hold on an interval of values (a sublevel set of a
// function that falls, then rises): its first and last keys, from a key c
// inside it, by bisection.
template <class F>
__device__ unsigned first_key(unsigned c, F pred)
{
    unsigned long long lo = 0, hi = c;  // pred false..true on [0, c], true at c
    while (lo < hi) {
        const unsigned long long mid = (lo + hi) >> 1;
        if (pred(key_value((unsigned)mid)))
            hi = mid;
        else
            lo = mid + 1;
    }
    return (unsigned)hi;
}
template <class F>
__device__ unsigned last_key(unsigned c, F pred)
{
    unsigned long long lo = c, hi = 0xffffffffull;  // pred true..false on [c, 2^32)
    while (lo < hi) {
        const unsigned long long mid = (lo + hi + 1) >> 1;
        if (pred(key_value((unsigned)mid)))
            lo = mid;
        else
            hi = mid - 1;
    }
    return (unsigned)lo;
}

// Step 1 and 4 of the sample-select (one block per row).  Mode 0: a strided
// sample of the row (kept in `saved`), sorted: the exact median and MAD for a
// row no longer than the sample; else the median's key window, the MAD's
// window about the median window's middle, and the MAD classes of the
// counting pass.  Mode 1 (the median now exact): the sample keyed by
// |x - med| narrows the MAD window for the listed values; rows that cannot
// use the list select their MAD over the whole row.
// sample positions either side of the middle ranks: 3 binomial standard deviations
// (+16), so that a window misses about one row in 800 -- such a row is selected
// over the whole row, a few reads of it at the rate of the whole GPU
constexpr int kPad = 3 * 64 + 16;

__global__ void __launch_bounds__(1024)
det_sample_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st, int mode,
                  float n_mad, float *__restrict__ saved)
{
    extern __shared__ unsigned long long sample_smem[];
    unsigned *sk = reinterpret_cast<unsigned *>(sample_smem);  // kDetSample keys
    __shared__ unsigned hist[2 * kDetBins];
    __shared__ int pick[4];
    const int t = blockIdx.x;
    const int begin = st[t].begin;
    const long long n = st[t].end - begin;
    if (n <= 0)
        return;
    const float *row = cc + (size_t)t * ld + begin;
    const int m = n < kDetSample ? (int)n : kDetSample;
    int P = 1;
    while (P < m)
        P <<= 1;
    const long long a = (n - 1) / 2, b = n / 2;
    float *sv = saved + (size_t)t * kDetSample;
    const float med = st[t].med;  // mode 1: exact
    // thread 0 alone updates the row's state, at the end (fields read here, at the top,
    // by every thread, are not written)
    auto whole_row_mad = [&]() {  // the MAD over the whole row, the peaks by a pass of their own
        DetState s = st[t];
        s.src = kSrcRow;
        s.top = 32;
        s.prefix[0] = s.prefix[1] = 0u;
        s.rank[0] = (int)a;
        s.rank[1] = (int)b;
        s.peaks_ready = 0;
        st[t] = s;
    };
    if (mode == 1) {
        const bool whole = m == n;  // sorted whole by the median's sample
        const bool list = !whole && st[t].one_read && !st[t].over_a && med >= st[t].m_lo &&
                          med <= st[t].m_hi;
        if (!whole && !list) {
            if (threadIdx.x == 0)
                whole_row_mad();
            return;
        }
    }
    // sample positions floor(i * n / m) from a fixed-point step (no 64-bit division
    // per sample); any spread of positions serves, the selection is exact
    // (blockDim.x = 1024, P <= kDetSample: kPer slots per thread, all loads issued
    // before the first store, so the scattered reads are in flight together)
    const unsigned long long stepq = ((unsigned long long)n << 20) / (unsigned long long)m;
    constexpr int kPer = kDetSample / 1024;
    float v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; j++) {
        const int i = threadIdx.x + j * 1024;
        v[j] = 0.0f;
        if (i < m) {
            if (mode == 0) {
                const long long pos = (long long)(((unsigned long long)i * stepq) >> 20);
                v[j] = row[pos < n ? pos : n - 1];
            } else {
                v[j] = sv[i];
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kPer; j++) {
        const int i = threadIdx.x + j * 1024;
        if (i < P) {
            if (mode == 0 && i < m)
                sv[i] = v[j];
            sk[i] = i < m ? order_key(mode == 0 ? v[j] : dev(v[j], med)) : 0xffffffffu;  // padding ranks last
        }
    }
    __syncthreads();
    // ranks of the window: the sample position of rank r is about r*m/n, with a
    // binomial standard deviation of at most sqrt(m)/2 = 64 positions
    const long long pa = a * m / n, pb = (b * m + n - 1) / n;
    const int r0 = m == n ? (int)a : (int)(pa - kPad > 0 ? pa - kPad : 0);
    const int r1 = m == n ? (int)b : (int)(pb + kPad < m - 1 ? pb + kPad : m - 1);
    unsigned k0, k1;
    block_select2(sk, P, r0, r1, hist, pick, k0, k1);
    if (m == n) {  // the whole row: exact
        if (threadIdx.x == 0) {
            DetState s = st[t];
            finish_select(s, mode, middle_value(k0, k1, (int)n), n_mad);
            s.src = kSrcDone;
            s.one_read = 0;
            s.peaks_ready = 0;
            st[t] = s;
        }
        return;
    }
    if (mode == 1) {  // the listed values' window: the sample's, inside [a_lo, a_hi]
        if (threadIdx.x == 0) {
            const unsigned klo = max(k0, order_key(st[t].a_lo)), khi = min(k1, order_key(st[t].a_hi));
            if (klo > khi) {  // cannot hold the MAD: the whole row
                whole_row_mad();
            } else {
                DetState s = st[t];
                s.klo = klo;
                s.khi = khi;
                s.src = kSrcCand;
                s.n_lt = s.n_below;
                s.n_in = 0;
                s.over_k = 0;
                st[t] = s;
            }
        }
        return;
    }
    // mode 0: the median lies in [m_lo, m_hi] if the window holds; the sample's
    // deviations from its middle give the MAD's window, widened by how far the
    // median can be from that middle
    // window ends without -0 (x + 0 is +0 for x = -0): the counting pass compares
    // floats, where -0 and +0 are one value, and keys its candidates as x + 0
    const float m_lo = __fadd_rn(key_value(k0), 0.0f), m_hi = __fadd_rn(key_value(k1), 0.0f);
    const float mid = __fadd_rn(__fmul_rn(0.5f, m_lo), __fmul_rn(0.5f, m_hi));
    __syncthreads();  // every thread is past its last read of the value keys
    for (int i = threadIdx.x; i < P; i += blockDim.x)
        sk[i] = i < m ? order_key(dev(sv[i], mid)) : 0xffffffffu;
    __syncthreads();
    unsigned ka0, ka1;
    block_select2(sk, P, r0, r1, hist, pick, ka0, ka1);
    if (threadIdx.x != 0)
        return;
    DetState s = st[t];
    s.klo = order_key(m_lo);
    s.khi = order_key(m_hi);
    s.src = kSrcCand;
    s.n_lt = s.n_in = 0;
    s.n_below = 0;
    s.over_k = s.over_a = 0;
    // the MAD moves with the median only at second order where the row is near
    // symmetric about it (d MAD / d m ~ f(m + MAD) - f(m - MAD)): a quarter of the
    // median window's half-width; a window that misses costs that row a pass over it
    const float wide = __fmul_rn(0.25f, fmaxf(__fsub_rn(mid, m_lo), __fsub_rn(m_hi, mid)));
    const float a_lo = fmaxf(__fsub_rn(key_value(ka0), wide), 0.0f);
    const float a_hi = __fadd_rn(key_value(ka1), wide);
    s.one_read = isfinite(m_lo) && isfinite(m_hi) && isfinite(a_lo) && isfinite(a_hi);
    if (s.one_read) {
        s.m_lo = m_lo;
        s.m_hi = m_hi;
        s.a_lo = a_lo;
        s.a_hi = a_hi;
        auto near = [&](float x) { return near_some(x, m_lo, m_hi, a_hi); };
        s.kn0 = first_key(order_key(m_lo), near);
        s.kn1 = last_key(order_key(m_lo), near);
        auto below = [&](float x) { return below_all(x, m_lo, m_hi, a_lo); };
        s.has_below = below(mid);  // the middle minimises the larger distance
        if (s.has_below) {
            s.kb0 = first_key(order_key(mid), below);
            s.kb1 = last_key(order_key(mid), below);
        }
        // thr = med + n_mad * mad rises with med and with mad (for n_mad >= 0; falls
        // with mad otherwise) and float rounding keeps that order, so med >= m_lo and
        // a MAD in [a_lo, a_hi] give thr >= thr_lo: the counting pass notes the values
        // >= thr_lo, whose local maxima are a superset of the peaks
        s.thr_lo = __fadd_rn(m_lo, __fmul_rn(n_mad, n_mad >= 0.0f ? a_lo : a_hi));
        s.peaks_ready = s.thr_lo == s.thr_lo;
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
// hot list (the rare path of the counting pass: one atomic, one store;
// det_hot_kernel examines the neighbours later).
__device__ __forceinline__ void note_hot(DetState *st, int t, long long o, int *hot, int cap)
{
    const int slot = atomicAdd(&st[t].n_hot, 1);
    if (slot < cap)
        hot[(size_t)t * cap + slot] = (int)o;
}

// Step 2, the one read of a row (ROW = true): values below the median window
// counted, values inside it appended to the thread's candidate column; the
// MAD classes (values in [b_lo, b_hi] counted, values in [n_lo, n_hi] outside
// it appended to the thread's column of undecided values); the offsets of the
// values at or above thr_lo noted in the row's hot list.  ROW = false, step 4:
// each thread walks its own column of undecided values keyed |x - med|: below
// the window counted, inside it appended to its candidate column.  Windows
// are compared as floats (rows are free of NaN; -0 compares as +0, and the
// readers key a candidate x as x + 0).  The per-value work is predicated, with
// no branch: the pass stays at the rate of the row's read.
template <bool ROW>
__global__ void __launch_bounds__(kDetThreads, 3)  // 24 warps per SM, 16 values per lane in flight
det_count_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st,
                 float *__restrict__ cand, long long cap, float *__restrict__ amb, long long amb_cap,
                 Lanes g, int *__restrict__ hot, int hcap)
{
    const int t = blockIdx.y;
    if (st[t].src != kSrcCand)
        return;  // uniform over the block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t col = ((size_t)t * g.S + blockIdx.x) * kDetThreads + threadIdx.x;
    const size_t region = (size_t)blockIdx.x * (kDetThreads / 32) + warp;
    float *kc = cand + (size_t)t * cap + region * (size_t)(g.Ck + kSpill) * 32 + lane;
    float *ac = amb + (size_t)t * amb_cap + region * (size_t)(g.Ca + kSpill) * 32 + lane;
    const float lo = key_value(st[t].klo), hi = key_value(st[t].khi);
    const float med = st[t].med;
    // the MAD classes as float intervals, empty (x >= +inf never holds) where the
    // row has none
    const bool classes = ROW && st[t].one_read;
    const bool has_below = classes && st[t].has_below;
    const float b_lo = has_below ? key_value(st[t].kb0) : INFINITY;
    const float b_hi = has_below ? key_value(st[t].kb1) : -INFINITY;
    const float n_lo = classes ? key_value(st[t].kn0) : INFINITY;
    const float n_hi = classes ? key_value(st[t].kn1) : -INFINITY;
    const bool peaks = ROW && st[t].peaks_ready;
    const float thr_lo = st[t].thr_lo;
    unsigned lt = 0, nb = 0;
    // offsets (floats) of the next entry of this thread's columns; a step's appends
    // past the capacity land in the spill rows, and the offset is clamped after it
    unsigned ko = 0, ao = 0;
    const unsigned kmax = (unsigned)g.Ck * 32u, amax = (unsigned)g.Ca * 32u;
    bool ovk = false, ova = false;
    auto take = [&](float x, bool ok) {
        lt += (unsigned)(ok & (x < lo));
        const bool in = ok & (x >= lo) & (x <= hi);
        if (in)
            kc[ko] = x;
        ko += in ? 32u : 0u;
        if constexpr (ROW) {
            const bool below = ok & (x >= b_lo) & (x <= b_hi);
            nb += (unsigned)below;
            const bool un = ok & !below & (x >= n_lo) & (x <= n_hi);
            if (un)
                ac[ao] = x;
            ao += un ? 32u : 0u;
        }
    };
    auto clamp = [&]() {  // after at most kSpill appends per column
        ovk |= ko > kmax;
        ko = min(ko, kmax);
        if constexpr (ROW) {
            ova |= ao > amax;
            ao = min(ao, amax);
        }
    };
    if constexpr (ROW) {
        const float *row = cc + (size_t)t * ld + st[t].begin;
        const long long n = st[t].end - st[t].begin;
        const RowSplit rs = split_row(row, n);
        if (blockIdx.x == 0 && warp == 0) {  // the unaligned ends, at most 3 + 3 values
            const long long i = lane < rs.head ? lane : rs.head + 4 * rs.nvec + (lane - rs.head);
            const bool ok = lane < rs.head + rs.tail;
            const float x = ok ? row[i] : 0.0f;
            if (peaks && ok && x >= thr_lo)
                note_hot(st, t, i, hot, hcap);
            take(x, ok);
            clamp();
        }
        // a warp step: 32 float4s from each quarter of the row, so that a lane's four
        // float4s lie far apart (on a smooth row, neighbouring values share their
        // class: a lane's appends then come in runs of at most 4)
        const float4 *vrow = reinterpret_cast<const float4 *>(row + rs.head);
        const long long quarter = (rs.nvec + 3) / 4;
        const long long steps = (quarter + 31) / 32;
        const long long cstride = (long long)gridDim.x * (kDetThreads / 32);
        auto load4 = [&](long long c, float4 (&v)[4]) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const long long q = c * 32 + lane, i = u * quarter + q;
                v[u] = (c < steps && q < quarter && i < rs.nvec) ? vrow[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        };
        float4 nv[4];
        long long c = (long long)blockIdx.x * (kDetThreads / 32) + warp;
        load4(c, nv);
        for (; c < steps; c += cstride) {
            float4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                v[u] = nv[u];
            load4(c + cstride, nv);  // the next step's values are in flight while this one is counted
            // values at or above thr_lo (rare): one vote per step on the lanes' largest
            // values (the zeros loaded past the row's end can only cost the slow path)
            float mx = -INFINITY;
#pragma unroll
            for (int u = 0; u < 4; u++)
                mx = fmaxf(mx, fmaxf(fmaxf(v[u].x, v[u].y), fmaxf(v[u].z, v[u].w)));
            if (peaks && __any_sync(0xffffffffu, mx >= thr_lo)) {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const long long q = c * 32 + lane, i = u * quarter + q;
                    const float m4 = fmaxf(fmaxf(v[u].x, v[u].y), fmaxf(v[u].z, v[u].w));
                    if (q < quarter && i < rs.nvec && m4 >= thr_lo) {
                        const long long o = rs.head + 4 * i;
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
            if (c * 32 + 32 <= quarter && 3 * quarter + c * 32 + 32 <= rs.nvec) {  // a whole step (warp-uniform)
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    take(v[u].x, true);
                    take(v[u].y, true);
                    take(v[u].z, true);
                    take(v[u].w, true);
                }
            } else {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const long long q = c * 32 + lane;
                    const bool ok = q < quarter && u * quarter + q < rs.nvec;
                    take(v[u].x, ok);
                    take(v[u].y, ok);
                    take(v[u].z, ok);
                    take(v[u].w, ok);
                }
            }
            clamp();
        }
    } else {
        // this thread's own column of undecided values, eight loads in flight
        const int m = min(g.cnt_a[col], g.Ca);
        const int mw = __reduce_max_sync(0xffffffffu, m);
        for (int k = 0; k < mw; k += 8) {
            float x[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                x[j] = k + j < m ? ac[(size_t)(k + j) * 32] : 0.0f;
#pragma unroll
            for (int j = 0; j < 8; j++)
                take(dev(x[j], med), k + j < m);
            clamp();
        }
    }
    const int nk = ovk ? g.Ck + 1 : (int)(ko / 32u);  // past the capacity: overflowed
    g.cnt_k[col] = nk;
    if (ROW)
        g.cnt_a[col] = ova ? g.Ca + 1 : (int)(ao / 32u);
    const bool over_k = __any_sync(0xffffffffu, ovk);
    const bool over_a = ROW && __any_sync(0xffffffffu, ova);
    const int sum_k = __reduce_add_sync(0xffffffffu, (unsigned)nk);
    for (int o = 16; o > 0; o >>= 1) {
        lt += __shfl_down_sync(0xffffffffu, lt, o);
        nb += __shfl_down_sync(0xffffffffu, nb, o);
    }
    if (lane == 0) {
        if (lt)
            atomicAdd(&st[t].n_lt, (int)lt);
        if (nb)
            atomicAdd(&st[t].n_below, (int)nb);
        if (sum_k)
            atomicAdd(&st[t].n_in, sum_k);
        if (over_k)
            atomicOr(&st[t].over_k, 1);
        if (over_a)
            atomicOr(&st[t].over_a, 1);
    }
}

// Step 3 (and 4): does the window hold both middle ranks?  Then select among
// the candidates, over the key bits they do not share; else fall back to the
// whole row -- for the median that also gives up the MAD classes of the
// counting pass (they assume the median inside [m_lo, m_hi]) and its hot
// values; for the MAD, the hot values (the superset may miss some, or have
// overflowed its list).
__global__ void det_check_kernel(DetState *__restrict__ st, int T, int mode, int pcap, float n_mad)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T || st[t].src != kSrcCand)
        return;
    DetState s = st[t];
    const long long n = s.end - s.begin;
    const long long a = (n - 1) / 2, b = n / 2;
    if (!s.over_k && s.n_lt <= a && b < (long long)s.n_lt + s.n_in) {
        s.rank[0] = (int)(a - s.n_lt);
        s.rank[1] = (int)(b - s.n_lt);
        const unsigned diff = s.klo ^ s.khi;
        s.top = diff ? 32 - __clz(diff) : 0;
        s.prefix[0] = s.prefix[1] = s.klo & above_mask(s.top);
        if (s.top == 0) {  // every candidate has the key klo
            finish_select(s, mode, middle_value(s.klo, s.klo, (int)n), n_mad);
            s.src = kSrcDone;
        }
    } else {
        s.src = kSrcRow;
        s.top = 32;
        s.prefix[0] = s.prefix[1] = 0u;
        s.rank[0] = (int)a;
        s.rank[1] = (int)b;
        s.peaks_ready = 0;
        if (mode == 0)
            s.one_read = 0;
    }
    if (mode == 1 && (!s.peaks_ready || s.n_hot > pcap))
        s.peaks_ready = 0;
    if (!s.peaks_ready)
        s.n_cand = 0;
    st[t] = s;
}

// Histogram update: every lane of the warp calls it (lanes whose value does
// not count pass ok = false).  With `aggregate` (the first pass over a whole
// row, whose keys share few digits) lanes with the same digit add once;
// otherwise (candidates, later passes: digits spread) each lane adds its own
// count.
__device__ __forceinline__ void hist_add(unsigned *h, float v, bool ok, int mode, float med, int shift,
                                         unsigned dmask, unsigned high, unsigned p0, unsigned p1,
                                         bool two, int lane, bool aggregate)
{
    // mode 2: a candidate, keyed as v + 0 (the counting pass compares floats, where
    // -0 and +0 are one value)
    const unsigned key = mode == 2 ? order_key(__fadd_rn(v, 0.0f)) : sel_key(v, mode, med);
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

// One selection pass over the candidates: histogram of the current digit over
// the candidates whose higher key bits equal a rank's prefix, each thread
// reading its own column as the counting pass wrote it.  Grid: (blocks per
// row, templates), as the counting pass.
__global__ void __launch_bounds__(kDetThreads)
det_hist_kernel(const DetState *__restrict__ st, unsigned *__restrict__ hist,
                const float *__restrict__ cand, long long cap, Lanes g, int pass)
{
    __shared__ unsigned h[2 * kDetBins];
    const int t = blockIdx.y;
    const DetState s = st[t];
    if (s.src != kSrcCand || s.end - s.begin <= 0)
        return;  // uniform over the block, before any barrier (rows that fell back:
                 // det_hist_row_kernel)
    if (pass > 0 && s.top <= 11 * pass)
        return;  // the key is complete
    for (int i = threadIdx.x; i < 2 * kDetBins; i += kDetThreads)
        h[i] = 0u;
    __syncthreads();
    int shift, width;
    pass_digit(s.top, pass, shift, width);
    const unsigned dmask = (1u << width) - 1u;
    const unsigned high = above_mask(shift + width);
    const unsigned p0 = s.prefix[0], p1 = s.prefix[1];
    const bool two = p0 != p1;  // the two middle ranks sit in different buckets
    const float med = s.med;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    constexpr int kWarps = kDetThreads / 32;
    {
        const size_t col = ((size_t)t * g.S + blockIdx.x) * kDetThreads + threadIdx.x;
        const size_t region = (size_t)blockIdx.x * kWarps + warp;
        const float *kc = cand + (size_t)t * cap + region * (size_t)(g.Ck + kSpill) * 32 + lane;
        const int m = g.cnt_k[col];  // <= Ck: no column overflowed
        const int mw = __reduce_max_sync(0xffffffffu, m);
        for (int k = 0; k < mw; k += 8) {  // eight loads in flight
            float x[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                x[j] = k + j < m ? kc[(size_t)(k + j) * 32] : 0.0f;
#pragma unroll
            for (int j = 0; j < 8; j++)
                hist_add(h, x[j], k + j < m, 2, med, shift, dmask, high, p0, p1, two, lane, false);
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

// The rows that need a pass over the whole row, compacted into list[0..*count)
// (one block): kind 0 those selecting over the whole row, kind 1 those whose
// peaks were not gathered by the counting pass (at least 3 lags).
__global__ void __launch_bounds__(1024)
det_collect_kernel(const DetState *__restrict__ st, int T, int kind, int *__restrict__ list,
                   int *__restrict__ count)
{
    __shared__ int n;
    if (threadIdx.x == 0)
        n = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const bool need = kind == 0 ? st[t].src == kSrcRow && st[t].end > st[t].begin
                                    : !st[t].peaks_ready && st[t].end - st[t].begin >= 3;
        if (need)
            list[atomicAdd(&n, 1)] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        *count = n;
}

// The same pass for the rows that fell back to selection over the whole row
// (a sample window that missed, a column that overflowed): every block of a
// fixed grid takes a slice of each such row in turn, so a row that fell back
// is read at the rate of the whole GPU, not of its own few blocks.  mode 0
// keys the values, mode 1 |x - median|; equal digits are aggregated per warp
// in the first pass (a row's keys share their high digits).
__global__ void __launch_bounds__(kDetThreads)
det_hist_row_kernel(const float *__restrict__ cc, size_t ld, const DetState *__restrict__ st,
                    const int *__restrict__ list, const int *__restrict__ count,
                    unsigned *__restrict__ hist, int pass, int mode)
{
    __shared__ unsigned h[2 * kDetBins];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kWarps = kDetThreads / 32;
    const int nrows = *count;
    for (int k = 0; k < nrows; k++) {
        const int t = list[k];
        const DetState s = st[t];
        const long long n = s.end - s.begin;
        if (n <= 0)
            continue;
        int shift, width;
        pass_digit(s.top, pass, shift, width);
        if (width == 0)
            continue;
        const unsigned dmask = (1u << width) - 1u;
        const unsigned high = above_mask(shift + width);
        const unsigned p0 = s.prefix[0], p1 = s.prefix[1];
        const bool two = p0 != p1;
        const bool agg = pass == 0;
        for (int i = threadIdx.x; i < 2 * kDetBins; i += kDetThreads)
            h[i] = 0u;
        __syncthreads();
        const float *row = cc + (size_t)t * ld + s.begin;
        const RowSplit rs = split_row(row, n);
        if (blockIdx.x == 0 && warp == 0) {  // the unaligned ends, at most 3 + 3 values
            const long long i = lane < rs.head ? lane : rs.head + 4 * rs.nvec + (lane - rs.head);
            const bool ok = lane < rs.head + rs.tail;
            const float v = ok ? row[i] : 0.f;
            hist_add(h, v, ok, mode, s.med, shift, dmask, high, p0, p1, two, lane, agg);
        }
        const float4 *vrow = reinterpret_cast<const float4 *>(row + rs.head);
        const long long steps = (rs.nvec + 63) / 64;  // 64 float4s per warp step
        for (long long c = (long long)blockIdx.x * kWarps + warp; c < steps;
             c += (long long)gridDim.x * kWarps) {
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
                hist_add(h, v[u].x, ok[u], mode, s.med, shift, dmask, high, p0, p1, two, lane, agg);
                hist_add(h, v[u].y, ok[u], mode, s.med, shift, dmask, high, p0, p1, two, lane, agg);
                hist_add(h, v[u].z, ok[u], mode, s.med, shift, dmask, high, p0, p1, two, lane, agg);
                hist_add(h, v[u].w, ok[u], mode, s.med, shift, dmask, high, p0, p1, two, lane, agg);
            }
        }
        __syncthreads();
        unsigned *gh = hist + (size_t)t * 2 * kDetBins;
        for (int i = threadIdx.x; i < (two ? 2 : 1) * kDetBins; i += kDetThreads) {
            const unsigned c = h[i];
            if (c)
                atomicAdd(gh + i, c);
        }
        __syncthreads();  // h is cleared for the next row
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
    int shift, width;
    pass_digit(s.top, pass, shift, width);
    if (width == 0)
        return;  // the key was complete after an earlier pass
    unsigned *gh = hist + (size_t)t * 2 * kDetBins;
    const int per = kDetBins / 32;  // bins per lane (digits of fewer bits leave the rest empty)
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
    if (shift == 0)
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
// template's candidate list, for the rows whose counting pass did not gather
// them (rows sorted whole by the sample, windows that missed, supersets that
// overflowed): every block of a fixed grid takes a slice of each such row in
// turn.  Samples are read with 16-byte loads; the rare sample at or above the
// threshold is examined with scalar loads.
__global__ void __launch_bounds__(kDetThreads)
det_peaks_kernel(const float *__restrict__ cc, size_t ld, DetState *__restrict__ st,
                 const int *__restrict__ list, const int *__restrict__ count, int2 *__restrict__ cand, int cap)
{
    const long long gtid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int nrows = *count;
#pragma unroll 1
    for (int k = 0; k < nrows; k++) {
        const int t = list[k];
        const long long b = st[t].begin, e = st[t].end;
        const float thr = st[t].thr;
        const float *row = cc + (size_t)t * ld;
        const RowSplit rs = split_row(row + b, e - b);
        if (gtid < rs.head + rs.tail) {
            const long long i = b + (gtid < rs.head ? gtid : rs.head + 4 * rs.nvec + (gtid - rs.head));
            peak_at(row, i, b, e, row[i], thr, st, cand, cap, t);
        }
        const float4 *vrow = reinterpret_cast<const float4 *>(row + b + rs.head);
        const long long base = b + rs.head;
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
    // 1. the candidates at or above thr (the counting pass gathers a superset: those at
    // or above a lower bound of thr), ordered by lag (lags are distinct); the others
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
    DetState *st = nullptr;
    unsigned *hist = nullptr;
    int2 *cand = nullptr;
    int *hot = nullptr, *col_cnt = nullptr, *row_list = nullptr;
    float *saved = nullptr, *amb = nullptr, *keys = nullptr;
    // candidates per row: a sample window holds about 2.5 % of a row; the values whose
    // MAD class waits for the median, about 7 % of a Gaussian row
    // (at least 2 * kSpill rows of every thread's columns, so a row's columns always fit)
    const long long key_cap = std::max(2LL * kSpill * kDetThreads,
                                       n_corr < 65536 ? n_corr : std::max(65536LL, (long long)n_corr / 8));
    const long long amb_cap = std::max(2LL * kSpill * kDetThreads,
                                       n_corr < 65536 ? n_corr : std::max(65536LL, (long long)n_corr / 4));
    if ((rc = ws.get(&st, (size_t)chunk, "detection state")) ||
        (rc = ws.get(&hist, (size_t)chunk * 2 * kDetBins, "detection histograms")) ||
        (rc = ws.get(&keys, (size_t)chunk * key_cap, "candidate keys")) ||
        (rc = ws.get(&amb, (size_t)chunk * amb_cap, "values of undecided MAD class")) ||
        (rc = ws.get(&cand, (size_t)chunk * kDetCap, "candidate peaks")) ||
        (rc = ws.get(&hot, (size_t)chunk * kDetCap, "values above the threshold bound")) ||
        (rc = ws.get(&saved, (size_t)chunk * kDetSample, "sampled values")) ||
        (rc = ws.get(&col_cnt, 2 * ((size_t)kDetBlocks + chunk) * kDetThreads, "list column counts")) ||
        (rc = ws.get(&row_list, (size_t)chunk + 1, "rows of whole-row passes")))
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
        // enough blocks per row to fill the SMs several times over, so that the last,
        // partial wave of blocks costs little -- but at least 1,024 values per thread,
        // so that its list columns hold many standard deviations above their mean fill
        long long per_row = ((long long)kDetBlocks + nt - 1) / nt;
        const long long row_cap = std::max(1LL, (long long)n_corr / (1024LL * kDetThreads));
        if (per_row > row_cap)
            per_row = row_cap;
        if (per_row < 1)
            per_row = 1;
        const dim3 grid((unsigned)per_row, (unsigned)nt);
        // one column per counting thread (nt * per_row <= kDetBlocks + nt blocks); rows
        // C .. C + kSpill - 1 of each warp's region take a step's overflow
        Lanes g;
        g.S = (int)per_row;
        g.Ck = (int)(key_cap / (per_row * kDetThreads) - kSpill);
        g.Ca = (int)(amb_cap / (per_row * kDetThreads) - kSpill);
        g.cnt_k = col_cnt;
        g.cnt_a = col_cnt + ((size_t)kDetBlocks + chunk) * kDetThreads;
        const int check_blocks = (nt + 127) / 128;
        det_init_kernel<<<(nt + 127) / 128, 128, 0, s>>>(st, nt, n_corr, begin ? begin + t0 : nullptr,
                                                         end ? end + t0 : nullptr);
        // the median: sample, the one read of the rows, selection over the candidates
        det_sample_kernel<<<nt, 1024, kDetSample * sizeof(unsigned), s>>>(rows, ld, st, 0, n_mad, saved);
        det_count_kernel<true><<<grid, kDetThreads, 0, s>>>(rows, ld, st, keys, key_cap, amb, amb_cap, g, hot,
                                                            kDetCap);
        det_check_kernel<<<check_blocks, 128, 0, s>>>(st, nt, 0, kDetCap, n_mad);
        int *const rcount = row_list + chunk;
        det_collect_kernel<<<1, 1024, 0, s>>>(st, nt, 0, row_list, rcount);
        for (int pass = 0; pass < 3; pass++) {
            det_hist_kernel<<<grid, kDetThreads, 0, s>>>(st, hist, keys, key_cap, g, pass);
            det_hist_row_kernel<<<kDetRowBlocks, kDetThreads, 0, s>>>(rows, ld, st, row_list, rcount, hist,
                                                                      pass, 0);
            det_resolve_kernel<<<nt, 32, 0, s>>>(st, hist, pass, 0, n_mad);
        }
        // the MAD: the sample about the exact median, the listed values, selection
        det_sample_kernel<<<nt, 1024, kDetSample * sizeof(unsigned), s>>>(rows, ld, st, 1, n_mad, saved);
        det_count_kernel<false><<<grid, kDetThreads, 0, s>>>(rows, ld, st, keys, key_cap, amb, amb_cap, g, hot,
                                                             kDetCap);
        det_check_kernel<<<check_blocks, 128, 0, s>>>(st, nt, 1, kDetCap, n_mad);
        det_collect_kernel<<<1, 1024, 0, s>>>(st, nt, 0, row_list, rcount);
        for (int pass = 0; pass < 3; pass++) {
            det_hist_kernel<<<grid, kDetThreads, 0, s>>>(st, hist, keys, key_cap, g, pass);
            det_hist_row_kernel<<<kDetRowBlocks, kDetThreads, 0, s>>>(rows, ld, st, row_list, rcount, hist,
                                                                      pass, 1);
            det_resolve_kernel<<<nt, 32, 0, s>>>(st, hist, pass, 1, n_mad);
        }
        det_hot_kernel<<<nt, kDetThreads, 0, s>>>(rows, ld, st, hot, kDetCap, cand, kDetCap);
        det_collect_kernel<<<1, 1024, 0, s>>>(st, nt, 1, row_list, rcount);
        det_peaks_kernel<<<kDetRowBlocks, kDetThreads, 0, s>>>(rows, ld, st, row_list, rcount, cand, kDetCap);
        det_select_kernel<<<nt, kDetSelectThreads, select_smem(kDetCap), s>>>(
            st, cand, kDetCap, min_sep, max_det, med_out ? med_out + t0 : nullptr,
            mad_out ? mad_out + t0 : nullptr, thr_out ? thr_out + t0 : nullptr, count_out + t0,
            lag_out + (size_t)t0 * max_det, val_out + (size_t)t0 * max_det);
        count_launch(31);
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
