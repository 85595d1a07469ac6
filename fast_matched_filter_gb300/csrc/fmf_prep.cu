// fmf_prep.cu -- per-call preprocessing kernels.
//
//  * template_range_kernel : valid output range [k_lo, k_hi) of each template
//    (reference: matched_filter.c:53-76 start/stop, matched_filter.cu:302-308
//    n_corr_t).
//  * template_center_kernel: "full" only -- template minus its FP64 mean and
//    the FP64 sum of the centred values.  sum(t*(d-m)) equals
//    sum((t-tbar)*(d-m)) exactly, so centring changes no result; it removes
//    the template's DC term from the products the numerator sums.
//  * channel_centre_kernel : "full" only -- the constant subtracted from each
//    data channel, the median of evenly spaced samples (robust to transients).
//  * template_energy_kernel: the template energies sum(t^2) when the caller
//    passes none, computed as the reference wrapper computes them for
//    float32 templates (numpy.sum(templates**2, axis=-1),
//    fast_matched_filter.py:256-261): float32 squares summed in numpy's
//    pairwise order, so the values are bit-identical.
//  * window_stats_kernel   : sliding-window statistics of every channel for
//    windows of L samples starting at each sample index:
//      short: E = sum d^2                      (matched_filter.c:622)
//      full : m = sum d'/L, V = sum d'^2 - (sum d')^2/L   (d' = d - mu)
//    each window's sums composed from parts inside the window (the end of
//    its first 32-sample chunk, whole chunks, the start of its last chunk) in
//    double-float FP32 arithmetic, so that no window sum is the difference of
//    running sums and a large transient before a quiet window costs it no
//    digits (the reference's FP64 running sums lose 2^-53 of everything summed
//    before the window, matched_filter.c:29-31, 660-705).
#include "fmf_common.cuh"

namespace fmf {

__global__ void template_range_kernel(const int *__restrict__ mo, int T, int SC,
                                      int L, int N, int step, int n_corr,
                                      int *__restrict__ k_lo, int *__restrict__ k_hi)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T)
        return;
    int lo = 0, hi = 0;
    const int *m = mo + (size_t)t * SC;
    for (int ch = 0; ch < SC; ch++) {
        lo = min(lo, m[ch]);
        hi = max(hi, m[ch]);
    }
    long long first = lo < 0 ? ((long long)(-lo) + step - 1) / step : 0;
    long long last = (long long)N - L - hi;
    long long a = 0, b = 0;
    if (last >= 0) {
        b = last / step + 1;
        if (b > n_corr)
            b = n_corr;
        a = first < b ? first : b;
    }
    k_lo[t] = (int)a;
    k_hi[t] = (int)b;
}

__device__ __forceinline__ double block_sum_f64(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0)
        red[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); i++)
            s += red[i];
        red[32] = s;
    }
    __syncthreads();
    return red[32];
}

// numpy's float32 pairwise sum of the squares of a[0:n) (the reduction
// numpy.sum applies along a contiguous axis): fewer than 8 values -- a running
// sum from -0; up to 128 -- eight interleaved partial sums, combined as
// ((r0 + r1) + (r2 + r3)) + ((r4 + r5) + (r6 + r7)), then the values past the
// last multiple of 8 in order; more -- the sum of the two halves split at n/2
// rounded down to a multiple of 8.  Explicit round-to-nearest operations: no
// fused multiply-add may change a rounding.
__device__ float pairwise_leaf_sq(const float *a, int n)
{
    if (n < 8) {
        float r = -0.0f;
        for (int i = 0; i < n; i++)
            r = __fadd_rn(r, __fmul_rn(a[i], a[i]));
        return r;
    }
    float r[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
        r[k] = __fmul_rn(a[k], a[k]);
    int i = 8;
    for (; i < n - (n % 8); i += 8) {
#pragma unroll
        for (int k = 0; k < 8; k++)
            r[k] = __fadd_rn(r[k], __fmul_rn(a[i + k], a[i + k]));
    }
    float res = __fadd_rn(__fadd_rn(__fadd_rn(r[0], r[1]), __fadd_rn(r[2], r[3])),
                          __fadd_rn(__fadd_rn(r[4], r[5]), __fadd_rn(r[6], r[7])));
    for (; i < n; i++)
        res = __fadd_rn(res, __fmul_rn(a[i], a[i]));
    return res;
}

__device__ float pairwise_sq(const float *a, int n)
{
    // the recursion of numpy's pairwise sum, unrolled with an explicit stack
    // (depth <= 32 for any int n): post-order over the split tree
    int off[32], len[32], stage[32];
    float left[32];
    int sp = 0;
    off[0] = 0;
    len[0] = n;
    stage[0] = 0;
    float ret = 0.f;
    while (sp >= 0) {
        const int o = off[sp], m = len[sp];
        if (m <= 128) {
            ret = pairwise_leaf_sq(a + o, m);
            sp--;
        } else {
            int m2 = m / 2;
            m2 -= m2 % 8;
            if (stage[sp] == 0) {  // descend left
                stage[sp] = 1;
                sp++;
                off[sp] = o;
                len[sp] = m2;
                stage[sp] = 0;
                continue;
            }
            if (stage[sp] == 1) {  // left done: descend right
                left[sp] = ret;
                stage[sp] = 2;
                sp++;
                off[sp] = o + m2;
                len[sp] = m - m2;
                stage[sp] = 0;
                continue;
            }
            ret = __fadd_rn(left[sp], ret);  // both done
            sp--;
        }
    }
    return ret;
}

// one thread per (template, channel) row
__global__ void template_energy_kernel(const float *__restrict__ tpl, int rows, int L,
                                       float *__restrict__ sst)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows)
        sst[r] = pairwise_sq(tpl + (size_t)r * L, L);
}

// check_zeros count of the reference wrapper (fast_matched_filter.py:322-361)
// on the device: counts[t] += number of zeros among out[t][i] with
// i % last_axis < stop, over a row of row_len values.  Grid (blocks, T).
__global__ void zero_count_kernel(const float *__restrict__ out, long long row_len, long long last_axis,
                                  long long stop, unsigned long long *__restrict__ counts)
{
    const int t = blockIdx.y;
    const float *row = out + (size_t)t * row_len;
    const long long span = last_axis == row_len ? stop : row_len;  // network sum: lags < stop
    unsigned c = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < span;
         i += (long long)gridDim.x * blockDim.x)
        c += (row[i] == 0.0f && i % last_axis < stop) ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c)
        atomicAdd(counts + t, (unsigned long long)c);
}

// grid = T*SC blocks of 128 threads
__global__ void template_center_kernel(const float *__restrict__ tpl, int L,
                                       float *__restrict__ tcen,
                                       float *__restrict__ tsum)
{
    __shared__ double red[33];
    size_t row = blockIdx.x;
    const float *src = tpl + row * L;
    float *dst = tcen + row * L;
    double s = 0.0;
    for (int j = threadIdx.x; j < L; j += blockDim.x)
        s += (double)src[j];
    double mean = block_sum_f64(s, red) / (double)L;
    float mf = (float)mean;
    double s2 = 0.0;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        float v = src[j] - mf;
        dst[j] = v;
        s2 += (double)v;
    }
    double tot = block_sum_f64(s2, red);
    if (threadIdx.x == 0)
        tsum[row] = (float)tot;
}

// grid = SC blocks of 1024 threads: the centre c[ch] that 'full' subtracts
// from each data channel.  Any constant gives the same coefficients (the
// centred templates sum to zero, so sum t'(d - m) = sum t'(d - c - (m - c))),
// but the size of d - c sets the rounding of the numerator's products, of the
// tensor-core split most of all (2^-16 of each operand).  The channel mean
// moves with a large transient (a 1,000-sample burst at 1e3 shifts a 40,000-
// sample channel's mean by ~80 times a 1e-2 noise); the median of 8192
// evenly spaced samples stays at the level of the quiet data.  It is one of
// the samples, so d - c is exact in FP32 wherever c/2 <= d <= 2c.
constexpr int kCentreSample = 8192;
__global__ void __launch_bounds__(1024) channel_centre_kernel(const float *__restrict__ data, int N,
                                                              float *__restrict__ centre)
{
    __shared__ float v[kCentreSample];
    const float *src = data + (size_t)blockIdx.x * N;
    const int S = min(N, kCentreSample);
    for (int k = threadIdx.x; k < kCentreSample; k += blockDim.x)
        v[k] = k < S ? src[(long long)k * N / S] : INFINITY;
    __syncthreads();
    for (int k = 2; k <= kCentreSample; k <<= 1) {  // bitonic sort, ascending
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < kCentreSample; i += blockDim.x) {
                const int p = i ^ j;
                if (p > i) {
                    const float a = v[i], b = v[p];
                    if (((i & k) == 0) == (a > b)) {
                        v[i] = b;
                        v[p] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0)
        centre[blockIdx.x] = v[(S - 1) / 2];
}

// ---------------------------------------------------------------- window statistics
// Each window's sums are composed from parts that all lie inside the window,
// never taken as the difference of running sums: with samples in 32-sample
// chunks, the window [u, u + L) is
//     (u to the end of u's chunk) + (whole chunks) + (start of the last chunk to u + L),
// each part summed in double-float FP32 arithmetic (squares split exactly by
// FMA, TwoSum additions with the rounding errors carried in the low word).
// A difference of running sums loses the digits of everything summed before
// the window -- after a large transient, a quiet window holds 1e-10 of the
// running energy -- whereas here the sums of d^2 have only non-negative parts
// (about 44 significant bits whatever came before) and the sums of d' are
// accurate to 2^-44 of the window's own sum of |d'|.

constexpr int kStatThreads = 256;
constexpr int kStatGroup = 16;  // consecutive windows per thread
static_assert(kStatWindows == kStatThreads * kStatGroup, "one group of windows per thread");

// padded shared-memory index: one spare slot per 32, so that threads 16 or 32
// samples apart hit different banks
__device__ __forceinline__ int stat_pad(int i) { return i + (i >> 5); }

// Staged samples per block: the windows' span plus a zero tail read by the last
// group's loops, a multiple of the 32-sample chunk.
__host__ __device__ __forceinline__ int stat_span(int L) { return (kStatWindows + L + 63) & ~31; }

// Shared-memory carve (in floats, each part 16-byte aligned): squares, values
// ('full'), chunk sums of both, staged outputs.
struct StatLayout {
    int s2, s1, q2, q1, out, total;
    __host__ __device__ StatLayout(int L, bool full)
    {
        const int span = stat_span(L), padded = span + (span >> 5);
        const int nq = span >> 5, pw = kStatWindows + (kStatWindows >> 5);
        auto al = [](int x) { return (x + 3) & ~3; };
        s2 = 0;
        s1 = al(s2 + 2 * padded);
        q2 = al(s1 + (full ? padded : 0));
        q1 = al(q2 + 2 * nq);
        out = al(q1 + (full ? 2 * nq : 0));
        total = al(out + (full ? 2 : 1) * pw);
    }
};

size_t window_stats_smem(int L, bool full) { return (size_t)StatLayout(L, full).total * sizeof(float); }

// grid = (ceil(N / kStatWindows), SC), kStatThreads threads, dynamic smem =
// window_stats_smem(L, FULL).  short: stat_e[ch][u] = sum of d^2 over
// [u, u + L); FULL: (centred energy, mean) of d' = d - mu[ch] as float pairs,
// and the centred data into dcen.  Windows past N - L are not written.  One
// instantiation per mode: the 'short' one keeps no sums of d' in registers,
// so three blocks share an SM.
template <bool FULL>
__global__ void __launch_bounds__(kStatThreads, FULL ? 2 : 3)
window_stats_kernel(const float *__restrict__ data, int N, int L, const float *__restrict__ mu,
                    float *__restrict__ dcen, float *__restrict__ stat_e)
{
    extern __shared__ float4 stat_smem[];
    constexpr bool full = FULL;
    const StatLayout lay(L, full);
    float *base = reinterpret_cast<float *>(stat_smem);
    float2 *s2 = reinterpret_cast<float2 *>(base + lay.s2);
    float *s1 = base + lay.s1;
    float2 *q2 = reinterpret_cast<float2 *>(base + lay.q2);
    float2 *q1 = reinterpret_cast<float2 *>(base + lay.q1);
    float *out1 = base + lay.out;
    float2 *out2 = reinterpret_cast<float2 *>(base + lay.out);

    const int ch = blockIdx.y;
    const long long c0 = (long long)blockIdx.x * kStatWindows;
    const int len = (int)min((long long)kStatWindows + L - 1, (long long)N - c0);
    const int nwin = min(kStatWindows, len - L + 1);
    const int span = stat_span(L), nq = span >> 5;
    const float m = full ? mu[ch] : 0.0f;
    const float *src = data + (size_t)ch * N + c0;
    constexpr int kLoads = 4;  // loads in flight per thread before their use
    for (int i0 = threadIdx.x; i0 < span; i0 += kLoads * kStatThreads) {
        float x[kLoads];
#pragma unroll
        for (int j = 0; j < kLoads; j++) {
            const int i = i0 + j * kStatThreads;
            x[j] = i < len ? __ldg(src + i) : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < kLoads; j++) {
            const int i = i0 + j * kStatThreads;
            if (i < span) {
                const float v = i < len ? x[j] - m : 0.0f;
                if (full && i < kStatWindows && i < len)
                    dcen[(size_t)ch * N + c0 + i] = v;
                const float sq = v * v;
                s2[stat_pad(i)] = make_float2(sq, fmaf(v, v, -sq));  // v^2 exactly
                if (full)
                    s1[stat_pad(i)] = v;
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nq; k += kStatThreads) {  // chunk sums
        float h2 = 0.0f, l2 = 0.0f, h1 = 0.0f, l1 = 0.0f;
#pragma unroll 8
        for (int j = 0; j < 32; j++) {
            const float2 x = s2[stat_pad(32 * k + j)];
            pair_add(h2, l2, x.x, x.y);
            if (full)
                pair_add(h1, l1, s1[stat_pad(32 * k + j)], 0.0f);
        }
        q2[k] = make_float2(h2, l2);
        if (full)
            q1[k] = make_float2(h1, l1);
    }
    __syncthreads();

    const float Lf = (float)L, invL = 1.0f / Lf;
    auto emit = [&](int u, float h2, float l2, float h1, float l1) {
        if (full) {
            float v, mean;
            window_centred_sums(h2, l2, h1, l1, Lf, invL, v, mean);
            out2[stat_pad(u)] = make_float2(v, mean);
        } else {
            out1[stat_pad(u)] = h2 + l2;
        }
    };
    if (L >= 32) {
        // windows u0 .. u0 + 15 of this thread: all start in chunk a and end
        // past it, so suffix (in chunk a) + whole chunks + tail never overlap
        const int u0 = threadIdx.x * kStatGroup;
        if (u0 < nwin) {
            const int a = u0 >> 5;
            float sh2[kStatGroup], sl2[kStatGroup], sh1[kStatGroup], sl1[kStatGroup];
            float h2 = 0.0f, l2 = 0.0f, h1 = 0.0f, l1 = 0.0f;
            for (int j = u0 + kStatGroup; j < 32 * a + 32; j++) {
                const float2 x = s2[stat_pad(j)];
                pair_add(h2, l2, x.x, x.y);
                if (full)
                    pair_add(h1, l1, s1[stat_pad(j)], 0.0f);
            }
#pragma unroll
            for (int r = kStatGroup - 1; r >= 0; r--) {  // suffix sums, last start first
                const float2 x = s2[stat_pad(u0 + r)];
                pair_add(h2, l2, x.x, x.y);
                sh2[r] = h2;
                sl2[r] = l2;
                if (full) {
                    pair_add(h1, l1, s1[stat_pad(u0 + r)], 0.0f);
                    sh1[r] = h1;
                    sl1[r] = l1;
                }
            }
            const int e0 = u0 + L;  // end (exclusive) of window u0
            float mh2 = 0.0f, ml2 = 0.0f, mh1 = 0.0f, ml1 = 0.0f;  // whole chunks
            for (int k = a + 1; k < (e0 >> 5); k++) {
                pair_add(mh2, ml2, q2[k].x, q2[k].y);
                if (full)
                    pair_add(mh1, ml1, q1[k].x, q1[k].y);
            }
            float rh2 = 0.0f, rl2 = 0.0f, rh1 = 0.0f, rl1 = 0.0f;  // tail in the last chunk
            for (int j = e0 & ~31; j < e0; j++) {
                const float2 x = s2[stat_pad(j)];
                pair_add(rh2, rl2, x.x, x.y);
                if (full)
                    pair_add(rh1, rl1, s1[stat_pad(j)], 0.0f);
            }
#pragma unroll
            for (int r = 0; r < kStatGroup; r++) {
                const int e = e0 + r;
                if (r > 0 && (e & 31) == 0) {  // the tail's chunk is whole: move it to the middle
                    const int k = (e >> 5) - 1;
                    pair_add(mh2, ml2, q2[k].x, q2[k].y);
                    rh2 = rl2 = 0.0f;
                    if (full) {
                        pair_add(mh1, ml1, q1[k].x, q1[k].y);
                        rh1 = rl1 = 0.0f;
                    }
                }
                if (u0 + r < nwin) {
                    float th2 = sh2[r], tl2 = sl2[r], th1 = 0.0f, tl1 = 0.0f;
                    pair_add(th2, tl2, mh2, ml2);
                    pair_add(th2, tl2, rh2, rl2);
                    if (full) {
                        th1 = sh1[r];
                        tl1 = sl1[r];
                        pair_add(th1, tl1, mh1, ml1);
                        pair_add(th1, tl1, rh1, rl1);
                    }
                    emit(u0 + r, th2, tl2, th1, tl1);
                }
                const float2 x = s2[stat_pad(e)];
                pair_add(rh2, rl2, x.x, x.y);
                if (full)
                    pair_add(rh1, rl1, s1[stat_pad(e)], 0.0f);
            }
        }
    } else {  // windows shorter than a chunk: direct sums
        for (int u = threadIdx.x; u < nwin; u += kStatThreads) {
            float h2 = 0.0f, l2 = 0.0f, h1 = 0.0f, l1 = 0.0f;
            for (int j = u; j < u + L; j++) {
                const float2 x = s2[stat_pad(j)];
                pair_add(h2, l2, x.x, x.y);
                if (full)
                    pair_add(h1, l1, s1[stat_pad(j)], 0.0f);
            }
            emit(u, h2, l2, h1, l1);
        }
    }
    __syncthreads();
    for (int u = threadIdx.x; u < nwin; u += kStatThreads) {  // coalesced stores
        const size_t o = (size_t)ch * N + c0 + u;
        if (full)
            reinterpret_cast<float2 *>(stat_e)[o] = out2[stat_pad(u)];
        else
            stat_e[o] = out1[stat_pad(u)];
    }
}

int launch_window_stats(const float *data, int N, int L, int SC, const float *mu, float *dcen,
                        float *stat_e, cudaStream_t s)
{
    const bool full = mu != nullptr;
    const size_t smem = window_stats_smem(L, full);
    void (*kern)(const float *, int, int, const float *, float *, float *) =
        full ? window_stats_kernel<true> : window_stats_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynamicSmem);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "window statistics shared memory (%zu bytes): %s", smem,
                         cudaGetErrorString(e));
    dim3 grid((N + kStatWindows - 1) / kStatWindows, SC);
    kern<<<grid, kStatThreads, smem, s>>>(data, N, L, mu, dcen, stat_e);
    count_launch();
    return FMF_OK;
}

}  // namespace fmf
