// fmf_prep.cu -- per-call preprocessing kernels.
//
//  * template_range_kernel : valid output range [k_lo, k_hi) of each template
//    (reference: matched_filter.c:53-76 start/stop, matched_filter.cu:302-308
//    n_corr_t).
//  * template_center_kernel: "full" only -- template minus its FP64 mean and
//    the FP64 sum of the centred values.  sum(t*(d-m)) equals
//    sum((t-tbar)*(d-m)) exactly, so centring changes no result; it removes
//    the template's DC term from the products the numerator sums.
//  * channel_mean_kernel   : "full" only -- mean of each data channel (double-float sum),
//    rounded to float; d - mu is exact in FP32 wherever mu/2 <= d <= 2 mu.
//  * template_energy_kernel: the template energies sum(t^2) when the caller
//    passes none, computed as the reference wrapper computes them for
//    float32 templates (numpy.sum(templates**2, axis=-1),
//    fast_matched_filter.py:256-261): float32 squares summed in numpy's
//    pairwise order, so the values are bit-identical.
//  * window_stats_kernel   : sliding-window statistics of every channel for
//    windows of L samples starting at each sample index:
//      short: E = sum d^2                      (matched_filter.c:622)
//      full : m = sum d'/L, V = sum d'^2 - (sum d')^2/L   (d' = d - mu)
//    computed from a prefix sum local to each block of windows (so the
//    differenced values are of the size of the block's energy, not of the
//    whole trace's) held as double-float pairs in FP32 arithmetic: squares
//    split exactly by FMA, TwoSum additions with the rounding errors carried
//    in the low word, window differences by TwoSum; about 44 significant bits,
//    the accuracy of an FP64 scan at FP32 speed (FP64 runs at ~2 operations
//    per clock per SM on this part, which made this kernel FP64-bound).
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

// grid = SC blocks of 1024 threads: the mean of each data channel, rounded
// to float, from double-float sums (FP32 arithmetic, fixed order); each
// thread keeps four 16-byte loads in flight.
__global__ void channel_mean_kernel(const float *__restrict__ data, int N,
                                    float *__restrict__ mu)
{
    __shared__ float2 red[32];
    const float *src = data + (size_t)blockIdx.x * N;
    float h = 0.0f, l = 0.0f;
    // the floats before the first 16-byte boundary of the row (any caller pointer), then
    // float4 groups
    const int head = (int)min((long long)N, (long long)(((16 - ((uintptr_t)src & 15)) & 15) >> 2));
    for (int i = threadIdx.x; i < head; i += blockDim.x)
        pair_add(h, l, src[i], 0.0f);
    const float4 *v4 = reinterpret_cast<const float4 *>(src + head);
    const int n4 = (N - head) >> 2;
    constexpr int U = 4;
    for (int i0 = threadIdx.x; i0 < n4; i0 += U * blockDim.x) {
        float4 x[U];
#pragma unroll
        for (int u = 0; u < U; u++)
            x[u] = i0 + u * (int)blockDim.x < n4 ? v4[i0 + u * blockDim.x] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < U; u++) {
            pair_add(h, l, x[u].x, 0.0f);
            pair_add(h, l, x[u].y, 0.0f);
            pair_add(h, l, x[u].z, 0.0f);
            pair_add(h, l, x[u].w, 0.0f);
        }
    }
    for (int i = head + 4 * n4 + threadIdx.x; i < N; i += blockDim.x)
        pair_add(h, l, src[i], 0.0f);
    for (int o = 16; o > 0; o >>= 1) {
        const float yh = __shfl_down_sync(0xffffffffu, h, o), yl = __shfl_down_sync(0xffffffffu, l, o);
        pair_add(h, l, yh, yl);
    }
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = make_float2(h, l);
    __syncthreads();
    if (threadIdx.x == 0) {
        float th = 0.0f, tl = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++)
            pair_add(th, tl, red[i].x, red[i].y);
        mu[blockIdx.x] = (float)(((double)th + (double)tl) / (double)N);
    }
}

// In-place inclusive scan of a[1..len] (a[0] = 0) as double-float pairs, by the
// block: a contiguous segment per thread, then the segment totals by warp
// shuffles and one thread over the warps.
__device__ void block_scan_pair(float2 *a, int len, float2 *part)
{
    const int nt = blockDim.x;
    const int seg = (len + nt - 1) / nt;
    const int b = 1 + threadIdx.x * seg;
    const int e = min(len + 1, b + seg);
    float h = 0.0f, l = 0.0f;
    for (int i = b; i < e; i++) {
        const float2 x = a[i];
        pair_add(h, l, x.x, x.y);
        a[i] = make_float2(h, l);
    }
    // inclusive warp scan of the segment totals
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float xh = h, xl = l;
    for (int o = 1; o < 32; o <<= 1) {
        const float yh = __shfl_up_sync(0xffffffffu, xh, o), yl = __shfl_up_sync(0xffffffffu, xl, o);
        if (lane >= o)
            pair_add(xh, xl, yh, yl);
    }
    if (lane == 31)
        part[wid] = make_float2(xh, xl);
    // exclusive value of this thread within its warp
    float eh = __shfl_up_sync(0xffffffffu, xh, 1), el = __shfl_up_sync(0xffffffffu, xl, 1);
    if (lane == 0)
        eh = el = 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) {
        float rh = 0.0f, rl = 0.0f;
        for (int i = 0; i < (nt >> 5); i++) {
            const float2 v = part[i];
            part[i] = make_float2(rh, rl);
            pair_add(rh, rl, v.x, v.y);
        }
    }
    __syncthreads();
    float oh = part[wid].x, ol = part[wid].y;
    pair_add(oh, ol, eh, el);
    for (int i = b; i < e; i++) {
        float2 x = a[i];
        pair_add(x.x, x.y, oh, ol);
        a[i] = x;
    }
    __syncthreads();
}

// grid = (ceil(N / B), SC), block 256, dynamic smem = (B + L + 1) * 8 * (full ? 2 : 1)
__global__ void window_stats_kernel(const float *__restrict__ data, int N, int L,
                                    int B, const float *__restrict__ mu,
                                    float *__restrict__ dcen,
                                    float *__restrict__ stat_e)
{
    extern __shared__ float2 shp[];
    __shared__ float2 part[33];
    const int ch = blockIdx.y;
    const long long c0 = (long long)blockIdx.x * B;
    const int len = (int)min((long long)B + L, (long long)N - c0);
    const bool full = mu != nullptr;
    float2 *P2 = shp;
    float2 *P1 = shp + (B + L + 1);
    const float *src = data + (size_t)ch * N + c0;
    const float m = full ? mu[ch] : 0.0f;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        const float v = src[i] - m;
        if (full && i < B)
            dcen[(size_t)ch * N + c0 + i] = v;
        const float sq = v * v;
        P2[i + 1] = make_float2(sq, fmaf(v, v, -sq));  // v^2 exactly
        if (full)
            P1[i + 1] = make_float2(v, 0.0f);
    }
    if (threadIdx.x == 0) {
        P2[0] = make_float2(0.0f, 0.0f);
        if (full)
            P1[0] = make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    block_scan_pair(P2, len, part);
    if (full)
        block_scan_pair(P1, len, part);
    const int nwin = min(B, len - L + 1);
    const float Lf = (float)L, invL = 1.0f / Lf;
    for (int u = threadIdx.x; u < nwin; u += blockDim.x) {
        const size_t o = (size_t)ch * N + c0 + u;
        if (full) {
            float v, mean;
            window_centred(P2[u], P2[u + L], P1[u], P1[u + L], Lf, invL, v, mean);
            reinterpret_cast<float2 *>(stat_e)[o] = make_float2(v, mean);
        } else {
            float e;
            const float2 a2 = P2[u], b2 = P2[u + L];
            const float h = two_diff(b2.x, a2.x, e);
            stat_e[o] = h + (e + (b2.y - a2.y));
        }
    }
}

}  // namespace fmf
