// fmf_variable.cu -- per-channel template lengths with a Fisher-z network sum.
//
// GPU form of the reference's CPU-only arch 'variable_precise'
// (matched_filter.c:321-412, 569-606): channel ch of template t uses its
// first n[t][ch] taps (templates stored zero-padded to the longest, L); each
// channel's coefficient is the 'precise' one (window mean removed for 'full',
// threshold on sqrt(sst * ssd), matched_filter.c:629-657); the network value
// is sum_ch atanh(cc - 10 eps) * z[t][ch] with z = sqrt(n - 3) * w, and every
// output of template t then becomes
// (tanh(value / sum_ch z) + used * eps * 10) * scale[t].
// scale[t] is the reference's max_cc, which accumulates the weights of
// templates 0..t (it is never reset, matched_filter.c:329,365); it is
// reproduced as is.  Valid outputs: start <= k*step < stop with
// start = ceil(|min(0, min mo)| / step) * step and
// stop = N - L - max(0, max mo) - step (matched_filter.c:384-385); the final
// transform applies to every output (matched_filter.c:405-408).
//
// Kernels: metadata (Fisher-z weights per (t, ch), lag ranges and weight sums
// per template, the cumulative scale in one thread, each in the reference's
// float operation order),
// masked/centred templates, double-float prefix sums of d^2 and d stored as float
// pairs (global, so that any window length is a few FP32 operations), the
// numerator kernel with its
// variable-length epilogue -- the plain FP32 kernel (fmf_plain.cu) or the
// tensor-core kernel (fmf_tc.cu), whose issuers stop each channel's K range
// at its own length -- and the final transform.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "fmf_common.cuh"

namespace fmf {

__global__ void channel_mean_kernel(const float *, int, float *);
int collect_device_errors();

// Fisher-z weight of every (t, ch), one thread each, in the reference's mix
// of float and double operations: z = sqrt(n - 3) * w as
// 1 / sqrt(1 / (n - 3)) * w.
__global__ void vp_zweight_kernel(const float *__restrict__ w, const int *__restrict__ ntap, long long n,
                                  float *__restrict__ zweight)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        zweight[i] = (float)(1.0 / (double)sqrtf((float)(1.0 / (double)(ntap[i] - 3))) * (double)w[i]);
}

// One thread per template: lag range, sum of the Fisher-z weights (channel
// order, float), used-channel bias.
__global__ void vp_meta_kernel(const int *__restrict__ mo, const float *__restrict__ w,
                               const float *__restrict__ zweight, int T, int SC, int L, int N, int step,
                               int n_corr, int *k_lo, int *k_hi, float *norm_sum, float *bias)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T)
        return;
    const int *m = mo + (size_t)t * SC;
    const float *wt = w + (size_t)t * SC;
    const float *zt = zweight + (size_t)t * SC;
    int lo = 0, hi = 0, used = 0;
    float zs = 0.0f;
    for (int ch = 0; ch < SC; ch++) {
        lo = min(lo, m[ch]);
        hi = max(hi, m[ch]);
        if (wt[ch] != 0.0f)
            used += 1;
        zs += zt[ch];
    }
    const long long start = (long long)(int)ceilf((float)abs(lo) / (float)step) * step;
    const long long stop = (long long)N - L - hi - step;
    long long a = 0, b = 0;
    if (stop > start) {
        a = start / step;
        b = (stop - 1) / step + 1;
        if (b > n_corr)
            b = n_corr;
        if (a > b)
            a = b;
    }
    k_lo[t] = (int)a;
    k_hi[t] = (int)b;
    norm_sum[t] = zs;
    bias[t] = used * FLT_EPSILON * 10;
}

// scale[t] = the reference's max_cc after template t: one float sum of the
// weights of templates 0..t in (t, ch) order (never reset,
// matched_filter.c:329,365).  One block: the weights of whole templates pass
// through shared memory, thread 0 adds them in order.
constexpr int kScaleChunk = 8192;
__global__ void vp_scale_kernel(const float *__restrict__ w, int T, int SC, float *__restrict__ scale)
{
    __shared__ float buf[kScaleChunk];
    const int per = SC <= kScaleChunk ? kScaleChunk / SC : 0;  // whole templates per chunk
    float max_cc = 0.0f;
    if (per == 0) {  // more channels than one chunk holds: straight from global memory
        if (threadIdx.x == 0)
            for (int t = 0; t < T; t++) {
                for (int ch = 0; ch < SC; ch++)
                    max_cc += w[(size_t)t * SC + ch];
                scale[t] = max_cc;
            }
        return;
    }
    for (int t0 = 0; t0 < T; t0 += per) {
        const int nt = min(per, T - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < nt * SC; i += blockDim.x)
            buf[i] = w[(size_t)t0 * SC + i];
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int tt = 0; tt < nt; tt++) {
                const float *b = buf + tt * SC;
#pragma unroll 8
                for (int ch = 0; ch < SC; ch++)
                    max_cc += b[ch];
                scale[t0 + tt] = max_cc;
            }
        }
    }
}

// grid = T*SC blocks: template ch of t restricted to its first n taps (zero
// beyond); for 'full' minus its FP64 mean over those taps, with the FP64 sum
// of the result.
__global__ void vp_template_kernel(const float *__restrict__ tpl, const int *__restrict__ ntap, int L,
                                   int full, float *__restrict__ tout, float *__restrict__ tsum)
{
    __shared__ double red[33];
    const size_t row = blockIdx.x;
    const int n = min(max(ntap[row], 0), L);
    const float *src = tpl + row * L;
    float *dst = tout + row * L;
    float mf = 0.0f;
    if (full) {
        double s = 0.0;
        for (int j = threadIdx.x; j < n; j += blockDim.x)
            s += (double)src[j];
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0)
            red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++)
                tot += red[i];
            red[32] = n > 0 ? tot / n : 0.0;
        }
        __syncthreads();
        mf = (float)red[32];
        __syncthreads();
    }
    double s2 = 0.0;
    for (int j = threadIdx.x; j < L; j += blockDim.x) {
        const float v = j < n ? src[j] - mf : 0.0f;
        dst[j] = v;
        s2 += (double)v;
    }
    if (full) {
        for (int o = 16; o > 0; o >>= 1)
            s2 += __shfl_down_sync(0xffffffffu, s2, o);
        if ((threadIdx.x & 31) == 0)
            red[threadIdx.x >> 5] = s2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double tot = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); i++)
                tot += red[i];
            tsum[row] = (float)tot;
        }
    }
}

constexpr int kPrefixBlock = 2048;

// Prefix sums of d'^2 and d' (d' = d - mu) per channel in three phases, all in
// double-float FP32 arithmetic (squares split exactly by FMA, TwoSum
// additions; FP64 runs at ~2 operations per clock per SM on this part):
// block sums, their exclusive scan per channel, then the scan inside each
// block plus its offset.  Stored as normalised float pairs hi = fl(P),
// lo = P - hi (~44-48 significant bits), so that the correlation epilogues
// form window sums in FP32 arithmetic, exact to float rounding while the
// window holds more than ~2^-24 of the channel's energy up to that point.

// Phase 1, grid (blocks, SC), 256 threads: block sums.
__global__ void prefix_block_kernel(const float *__restrict__ data, int N, const float *__restrict__ mu,
                                    float2 *__restrict__ bs2, float2 *__restrict__ bs1, int nblk)
{
    __shared__ float2 r2[32], r1[32];
    const int ch = blockIdx.y, blk = blockIdx.x;
    const float m = mu ? mu[ch] : 0.0f;
    const float *src = data + (size_t)ch * N;
    float h2 = 0.0f, l2 = 0.0f, h1 = 0.0f, l1 = 0.0f;
    for (int i = blk * kPrefixBlock + threadIdx.x; i < min(N, (blk + 1) * kPrefixBlock); i += blockDim.x) {
        const float v = src[i] - m, sq = v * v;
        pair_add(h2, l2, sq, fmaf(v, v, -sq));
        pair_add(h1, l1, v, 0.0f);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float a = __shfl_down_sync(0xffffffffu, h2, o), b = __shfl_down_sync(0xffffffffu, l2, o);
        const float c = __shfl_down_sync(0xffffffffu, h1, o), d = __shfl_down_sync(0xffffffffu, l1, o);
        pair_add(h2, l2, a, b);
        pair_add(h1, l1, c, d);
    }
    if ((threadIdx.x & 31) == 0) {
        r2[threadIdx.x >> 5] = make_float2(h2, l2);
        r1[threadIdx.x >> 5] = make_float2(h1, l1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f, b = 0.0f, c = 0.0f, d = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            pair_add(a, b, r2[i].x, r2[i].y);
            pair_add(c, d, r1[i].x, r1[i].y);
        }
        bs2[(size_t)ch * nblk + blk] = pair_normalise(a, b);
        bs1[(size_t)ch * nblk + blk] = pair_normalise(c, d);
    }
}

// Phase 2, one thread per channel: exclusive scan of the block sums
// (renormalised at every step).
__global__ void prefix_offsets_kernel(float2 *bs2, float2 *bs1, int nblk, int SC)
{
    const int ch = blockIdx.x * blockDim.x + threadIdx.x;
    if (ch >= SC)
        return;
    float2 a = make_float2(0.0f, 0.0f), b = make_float2(0.0f, 0.0f);
    float2 *p2 = bs2 + (size_t)ch * nblk, *p1 = bs1 + (size_t)ch * nblk;
    constexpr int G = 8;  // loads of a group issued before the dependent additions
    for (int i0 = 0; i0 < nblk; i0 += G) {
        float2 x[G], y[G];
#pragma unroll
        for (int j = 0; j < G; j++) {
            x[j] = i0 + j < nblk ? p2[i0 + j] : make_float2(0.0f, 0.0f);
            y[j] = i0 + j < nblk ? p1[i0 + j] : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int j = 0; j < G; j++) {
            if (i0 + j < nblk) {
                p2[i0 + j] = a;
                p1[i0 + j] = b;
            }
            pair_add(a.x, a.y, x[j].x, x[j].y);
            a = pair_normalise(a.x, a.y);
            pair_add(b.x, b.y, y[j].x, y[j].y);
            b = pair_normalise(b.x, b.y);
        }
    }
}

// Phase 3, grid (blocks, SC), 256 threads: inclusive scan of the block plus
// its offset -> P2[ch][i + 1] = sum_{x <= i} d'^2 (P2[ch][0] = 0) and, for
// 'full', P1 of d' and the centred data.
__global__ void prefix_write_kernel(const float *__restrict__ data, int N, const float *__restrict__ mu,
                                    const float2 *__restrict__ bs2, const float2 *__restrict__ bs1,
                                    int nblk, float2 *__restrict__ pre2f, float2 *__restrict__ pre1f,
                                    float *__restrict__ dcen)
{
    __shared__ float2 part2[32], part1[32];
    const int ch = blockIdx.y, blk = blockIdx.x;
    const float m = mu ? mu[ch] : 0.0f;
    const float *src = data + (size_t)ch * N;
    const int i0 = blk * kPrefixBlock;
    constexpr int per = kPrefixBlock / 256;  // 8 consecutive samples per thread
    float2 v2[per], v1[per];                 // running pairs of this thread
    float h2 = 0.0f, l2 = 0.0f, h1 = 0.0f, l1 = 0.0f;
#pragma unroll
    for (int e = 0; e < per; e++) {
        const int i = i0 + threadIdx.x * per + e;
        float v = 0.0f;
        if (i < N) {
            v = src[i] - m;
            if (dcen)
                dcen[(size_t)ch * N + i] = v;
        }
        const float sq = v * v;
        pair_add(h2, l2, sq, fmaf(v, v, -sq));
        pair_add(h1, l1, v, 0.0f);
        v2[e] = make_float2(h2, l2);
        v1[e] = make_float2(h1, l1);
    }
    // inclusive warp scan of the thread totals, then the exclusive value of this thread
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float x2 = h2, y2 = l2, x1 = h1, y1 = l1;
    for (int o = 1; o < 32; o <<= 1) {
        const float a = __shfl_up_sync(0xffffffffu, x2, o), b = __shfl_up_sync(0xffffffffu, y2, o);
        const float c = __shfl_up_sync(0xffffffffu, x1, o), d = __shfl_up_sync(0xffffffffu, y1, o);
        if (lane >= o) {
            pair_add(x2, y2, a, b);
            pair_add(x1, y1, c, d);
        }
    }
    if (lane == 31) {
        part2[wid] = make_float2(x2, y2);
        part1[wid] = make_float2(x1, y1);
    }
    float e2h = __shfl_up_sync(0xffffffffu, x2, 1), e2l = __shfl_up_sync(0xffffffffu, y2, 1);
    float e1h = __shfl_up_sync(0xffffffffu, x1, 1), e1l = __shfl_up_sync(0xffffffffu, y1, 1);
    if (lane == 0)
        e2h = e2l = e1h = e1l = 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) {  // warp offsets, starting from the block's offset
        const float2 o2 = bs2[(size_t)ch * nblk + blk], o1 = bs1[(size_t)ch * nblk + blk];
        float a = o2.x, b = o2.y, c = o1.x, d = o1.y;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            const float2 p = part2[k], q = part1[k];
            part2[k] = make_float2(a, b);
            part1[k] = make_float2(c, d);
            pair_add(a, b, p.x, p.y);
            pair_add(c, d, q.x, q.y);
        }
    }
    __syncthreads();
    float oh2 = part2[wid].x, ol2 = part2[wid].y, oh1 = part1[wid].x, ol1 = part1[wid].y;
    pair_add(oh2, ol2, e2h, e2l);
    pair_add(oh1, ol1, e1h, e1l);
    float2 *p2 = pre2f + (size_t)ch * (N + 1);
    float2 *p1 = pre1f ? pre1f + (size_t)ch * (N + 1) : nullptr;
    if (blk == 0 && threadIdx.x == 0) {
        p2[0] = make_float2(0.0f, 0.0f);
        if (p1)
            p1[0] = make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int e = 0; e < per; e++) {
        const int i = i0 + threadIdx.x * per + e;
        if (i < N) {
            float a = oh2, b = ol2;
            pair_add(a, b, v2[e].x, v2[e].y);
            p2[i + 1] = pair_normalise(a, b);
            if (p1) {
                float c = oh1, d = ol1;
                pair_add(c, d, v1[e].x, v1[e].y);
                p1[i + 1] = pair_normalise(c, d);
            }
        }
    }
}

// out[t][k] = (tanh(out / norm_sum[t]) + bias[t]) * scale[t] for every k < n_corr
__global__ void vp_finalize_kernel(float *__restrict__ out, int T, int n_corr,
                                   const float *__restrict__ norm_sum, const float *__restrict__ bias,
                                   const float *__restrict__ scale)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)T * n_corr)
        return;
    const int t = (int)(idx / n_corr);
    out[idx] = (tanhf(out[idx] / norm_sum[t]) + bias[t]) * scale[t];
}

// ------------------------------------------------------------------ host driver
struct VArgs {
    const float *tpl, *sst, *data, *w;
    const int *mo, *ntap;
    float *out;
    size_t step, N, T, S, C, n_corr;
    int normalize, flags;
};

// Templates [t0, t0 + nt) of a prepared per-channel-length search.
static Problem var_subset(const Problem &P, int t0, int nt)
{
    Problem Q = P;
    const size_t o = (size_t)t0 * P.SC;
    Q.tpl += o * P.L;
    Q.sst += o;
    if (Q.tsum)
        Q.tsum += o;
    Q.mo += o;
    Q.w += o;
    Q.ntap += o;
    Q.zweight += o;
    Q.k_lo += t0;
    Q.k_hi += t0;
    Q.out += (size_t)t0 * P.n_corr;
    Q.T = nt;
    return Q;
}

// A second stream and one event per template chunk, released on scope exit.
struct CopyStream {
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev[9] = {};
    cudaError_t init(int n)
    {
        cudaError_t e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
        for (int i = 0; i <= n && e == cudaSuccess; i++)
            e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
        return e;
    }
    ~CopyStream()
    {
        if (s2) {
            cudaStreamSynchronize(s2);
            cudaStreamDestroy(s2);
        }
        for (cudaEvent_t e : ev)
            if (e)
                cudaEventDestroy(e);
    }
};

// With host_out, the result goes to host memory in template chunks of
// tapering size (8,8,8,8,4,2,1,1 of 40 parts), each chunk's copy on a second
// stream overlapping the later chunks' kernels (all of which are queued before
// the first copy, which blocks the host when host_out is pageable).
static int variable_device(const VArgs &a, int L, cudaStream_t s, float *host_out = nullptr)
{
    int rc;
    const int T = (int)a.T, SC = (int)(a.S * a.C), N = (int)a.N;
    const bool full = a.normalize == 1;
    Scratch ws(s);
    int *k_lo;
    float *zweight, *consts, *tmask, *tsum = nullptr, *mu = nullptr, *dcen = nullptr;
    float2 *bs2, *bs1;
    float2 *pre2f, *pre1f = nullptr;
    const int nblk = (N + kPrefixBlock - 1) / kPrefixBlock;
    if ((rc = ws.get(&k_lo, 2 * (size_t)T, "template ranges")) ||
        (rc = ws.get(&zweight, (size_t)T * SC, "Fisher-z weights")) ||
        (rc = ws.get(&consts, 3 * (size_t)T, "transform constants")) ||
        (rc = ws.get(&tmask, (size_t)T * SC * L, "masked templates")) ||
        (rc = ws.get(&pre2f, (size_t)SC * (N + 1), "prefix sums")) ||
        (rc = ws.get(&bs2, 2 * (size_t)SC * nblk, "block sums")))
        return rc;
    bs1 = bs2 + (size_t)SC * nblk;
    if (full && ((rc = ws.get(&tsum, (size_t)T * SC, "template sums")) ||
                 (rc = ws.get(&mu, (size_t)SC, "channel means")) ||
                 (rc = ws.get(&dcen, (size_t)SC * N, "centred data")) ||
                 (rc = ws.get(&pre1f, (size_t)SC * (N + 1), "prefix sums of d"))))
        return rc;
    int *k_hi = k_lo + T;
    float *norm_sum = consts, *bias = consts + T, *scale = consts + 2 * T;

    const long long n_tc = (long long)T * SC;
    vp_zweight_kernel<<<(unsigned)((n_tc + 255) / 256), 256, 0, s>>>(a.w, a.ntap, n_tc, zweight);
    vp_meta_kernel<<<(T + 127) / 128, 128, 0, s>>>(a.mo, a.w, zweight, T, SC, L, N, (int)a.step,
                                                   (int)a.n_corr, k_lo, k_hi, norm_sum, bias);
    vp_scale_kernel<<<1, 256, 0, s>>>(a.w, T, SC, scale);
    vp_template_kernel<<<(unsigned)((size_t)T * SC), 128, 0, s>>>(a.tpl, a.ntap, L, full ? 1 : 0, tmask, tsum);
    if (full)
        channel_mean_kernel<<<SC, 1024, 0, s>>>(a.data, N, mu);
    prefix_block_kernel<<<dim3(nblk, SC), 256, 0, s>>>(a.data, N, mu, bs2, bs1, nblk);
    prefix_offsets_kernel<<<(SC + 127) / 128, 128, 0, s>>>(bs2, bs1, nblk, SC);
    prefix_write_kernel<<<dim3(nblk, SC), 256, 0, s>>>(a.data, N, mu, bs2, bs1, nblk, pre2f, pre1f, dcen);
    count_launch(full ? 8 : 7);
    if ((rc = check_launch("variable-length preprocessing")))
        return rc;

    Problem P;
    P.tpl = tmask;
    P.sst = a.sst;
    P.tsum = tsum;
    P.mo = a.mo;
    P.w = a.w;
    P.data = full ? dcen : a.data;
    P.stat_e = nullptr;
    P.k_lo = k_lo;
    P.k_hi = k_hi;
    P.out = a.out;
    P.T = T;
    P.SC = SC;
    P.L = L;
    P.N = N;
    P.step = (int)a.step;
    P.n_corr = (int)a.n_corr;
    P.normalize = a.normalize;
    P.network_sum = 1;
    P.ntap = a.ntap;
    P.pre2f = pre2f;
    P.pre1f = pre1f;
    P.zweight = zweight;
    P.vp_norm = P.vp_bias = P.vp_scale = nullptr;
    const int precision = FMF_FLAG_PRECISION_OF(a.flags);
    const size_t row_bytes = a.n_corr * sizeof(float);
    const int n_chunks = (!host_out || (size_t)T * row_bytes < ((size_t)64 << 20)) ? 1 : (T < 8 ? T : 8);
    int bounds[9];
    {
        static const int wts[8] = {8, 8, 8, 8, 4, 2, 1, 1};
        const bool taper = n_chunks == 8 && T >= 40;
        int acc = 0;
        bounds[0] = 0;
        for (int c = 0; c < n_chunks; c++) {
            acc += taper ? wts[c] : 1;
            bounds[c + 1] = (int)(((long long)T * acc) / (taper ? 40 : n_chunks));
        }
        bounds[n_chunks] = T;
    }
    unsigned *err = nullptr;
    int split = 0;
    std::vector<unsigned char> tcfull;
    if (precision != FMF_PREC_FP32) {
        const int forced = ((a.flags >> 8) & 0xff) * 16;
        if (forced != 0 && forced != 32 && forced != 64 && forced != 128)
            return set_error(FMF_ERR_ARG, "tensor-core tile of %d lag blocks (32, 64 or 128)", forced);
        P.vp_norm = norm_sum;  // the final transform fused into the output write
        P.vp_bias = bias;
        P.vp_scale = scale;
        split = precision == FMF_PREC_SPLIT_BF16;
        const int nb = tc_choose_nb(L, (int)a.step, split, forced);
        if (nb == 0)
            return set_error(FMF_ERR_SMEM, "template length %d, step %zu: tensor-core tile does not fit "
                                           "shared memory", L, a.step);
        tcfull.resize(tc_prob_size());
        if ((rc = device_error_word(&err)) ||
            (rc = tc_prepare(P, P.data, split, nb, (a.flags >> 16) & 0xff, ws, s,
                             reinterpret_cast<TcProb *>(tcfull.data()))))
            return rc;
    }
    CopyStream cs;
    cudaError_t e = host_out ? cs.init(n_chunks) : cudaSuccess;
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "copy stream: %s", cudaGetErrorString(e));
    for (int c = 0; c < n_chunks; c++) {
        const int t0 = bounds[c], nt = bounds[c + 1] - bounds[c];
        if (nt > 0) {
            if (!tcfull.empty()) {
                std::vector<unsigned char> sub(tc_prob_size());
                unsigned long long *queue;
                tc_subset(reinterpret_cast<const TcProb *>(tcfull.data()), t0, nt,
                          reinterpret_cast<TcProb *>(sub.data()));
                if ((rc = ws.get(&queue, 1, "tile queue")) ||
                    (rc = tc_run(reinterpret_cast<const TcProb *>(sub.data()), 1, split, queue, err, s)))
                    return rc;
            } else {
                if ((rc = launch_plain_all(var_subset(P, t0, nt), s)))
                    return rc;
                const long long n = (long long)nt * a.n_corr;
                vp_finalize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
                    a.out + (size_t)t0 * a.n_corr, nt, (int)a.n_corr, norm_sum + t0, bias + t0, scale + t0);
                count_launch();
                if ((rc = check_launch("variable-length transform")))
                    return rc;
            }
        }
        if (host_out && (e = cudaEventRecord(cs.ev[c], s)) != cudaSuccess)
            return set_error(FMF_ERR_CUDA, "chunk event: %s", cudaGetErrorString(e));
    }
    if (!host_out)
        return FMF_OK;
    for (int c = 0; c < n_chunks; c++) {
        const int t0 = bounds[c], nt = bounds[c + 1] - bounds[c];
        if (nt <= 0)
            continue;
        if ((e = cudaStreamWaitEvent(cs.s2, cs.ev[c], 0)) != cudaSuccess ||
            (e = cudaMemcpyAsync(host_out + (size_t)t0 * a.n_corr, a.out + (size_t)t0 * a.n_corr,
                                 (size_t)nt * row_bytes, cudaMemcpyDeviceToHost, cs.s2)) != cudaSuccess)
            return set_error(FMF_ERR_CUDA, "copying the result: %s", cudaGetErrorString(e));
    }
    // the scratch is freed on s: s waits for the last copy
    if ((e = cudaEventRecord(cs.ev[n_chunks], cs.s2)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(s, cs.ev[n_chunks], 0)) != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "copying the result: %s", cudaGetErrorString(e));
    return FMF_OK;
}

static int variable_entry(const VArgs &a, void *stream)
{
    set_error(FMF_OK, "");
    reset_launch_count();
    if (!a.tpl || !a.sst || !a.mo || !a.data || !a.w || !a.ntap || !a.out)
        return set_error(FMF_ERR_ARG, "null array argument");
    if (a.step < 1 || a.T < 1 || a.S < 1 || a.C < 1 || a.n_corr < 1 || a.N < 1)
        return set_error(FMF_ERR_ARG, "sizes must be positive");
    if (a.N > (size_t)INT_MAX / 2 || a.n_corr > (size_t)INT_MAX || a.S * a.C > (size_t)INT_MAX ||
        a.T > (size_t)INT_MAX || a.step > (size_t)INT_MAX / 2)
        return set_error(FMF_ERR_ARG, "sizes exceed the 32-bit index range of this build");
    if (a.normalize != 0 && a.normalize != 1)
        return set_error(FMF_ERR_ARG, "normalize must be 0 or 1");
    const int precision = FMF_FLAG_PRECISION_OF(a.flags);
    if (precision != FMF_PREC_FP32 && precision != FMF_PREC_SPLIT_BF16 && precision != FMF_PREC_BF16)
        return set_error(FMF_ERR_ARG, "unknown precision %d", precision);
    if (a.flags & FMF_FLAG_DEVICE_POINTERS) {  // read in place: 4-byte elements
        const void *ptrs[7] = {a.tpl, a.sst, a.mo, a.data, a.w, a.ntap, a.out};
        for (const void *p : ptrs)
            if ((uintptr_t)p & 3)
                return set_error(FMF_ERR_ARG, "device array %p is not 4-byte aligned", p);
    }
    keep_pool_cached();
    cudaGetLastError();
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n_meta = a.T * a.S * a.C;
    const bool dev = (a.flags & FMF_FLAG_DEVICE_POINTERS) != 0;
    // the longest template (stride of the template array)
    int L = 0;
    if (dev) {
        int *tmp = (int *)malloc(n_meta * sizeof(int));
        if (!tmp)
            return set_error(FMF_ERR_OOM, "host memory for the template lengths");
        cudaError_t e = cudaMemcpyAsync(tmp, a.ntap, n_meta * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            free(tmp);
            return set_error(FMF_ERR_CUDA, "reading the template lengths: %s", cudaGetErrorString(e));
        }
        for (size_t i = 0; i < n_meta; i++)
            L = tmp[i] > L ? tmp[i] : L;
        free(tmp);
    } else {
        for (size_t i = 0; i < n_meta; i++)
            L = a.ntap[i] > L ? a.ntap[i] : L;
    }
    if (L < 1 || (size_t)L > a.N)
        return set_error(FMF_ERR_ARG, "longest template %d not in [1, N]", L);
    if (a.n_corr > (a.N - L) / a.step + 1)
        return set_error(FMF_ERR_ARG, "n_corr exceeds (N - longest template)/step + 1");
    if (dev)
        return variable_device(a, L, s);

    int rc;
    const size_t SC = a.S * a.C;
    const size_t cnt[7] = {a.T * SC * L, a.T * SC, a.T * SC, SC * a.N, a.T * SC, a.T * SC, a.T * a.n_corr};
    float *buf[7];
    {
        Scratch io(s);
        for (int i = 0; i < 7; i++)
            if ((rc = io.get(&buf[i], cnt[i], "input/output copies")))
                return rc;
        const void *src[6] = {a.tpl, a.sst, a.mo, a.data, a.w, a.ntap};
        for (int i = 0; i < 6; i++) {
            cudaError_t e = cudaMemcpyAsync(buf[i], src[i], cnt[i] * 4, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess)
                return set_error(FMF_ERR_CUDA, "copying inputs: %s", cudaGetErrorString(e));
        }
        VArgs d = a;
        d.tpl = buf[0];
        d.sst = buf[1];
        d.mo = reinterpret_cast<const int *>(buf[2]);
        d.data = buf[3];
        d.w = buf[4];
        d.ntap = reinterpret_cast<const int *>(buf[5]);
        d.out = buf[6];
        if ((rc = variable_device(d, L, s, a.out)))
            return rc;
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "variable-length search: %s", cudaGetErrorString(e));
    return precision != FMF_PREC_FP32 ? collect_device_errors() : FMF_OK;
}

}  // namespace fmf

extern "C" {

int fmf_matched_filter_variable_ex(const float *templates, const float *sum_square_templates,
                                   const int *moveouts, const float *data, const float *weights,
                                   size_t step, const int *n_samples_template, size_t n_samples_data,
                                   size_t n_templates, size_t n_stations, size_t n_components,
                                   size_t n_corr, float *cc_sum, int normalize, int flags, void *stream)
{
    fmf::VArgs a;
    a.tpl = templates;
    a.sst = sum_square_templates;
    a.mo = moveouts;
    a.data = data;
    a.w = weights;
    a.ntap = n_samples_template;
    a.out = cc_sum;
    a.step = step;
    a.N = n_samples_data;
    a.T = n_templates;
    a.S = n_stations;
    a.C = n_components;
    a.n_corr = n_corr;
    a.normalize = normalize;
    a.flags = flags;
    return fmf::variable_entry(a, stream);
}

int fmf_matched_filter_variable(const float *templates, const float *sum_square_templates,
                                const int *moveouts, const float *data, const float *weights,
                                size_t step, const int *n_samples_template, size_t n_samples_data,
                                size_t n_templates, size_t n_stations, size_t n_components,
                                size_t n_corr, float *cc_sum, int normalize)
{
    return fmf_matched_filter_variable_ex(templates, sum_square_templates, moveouts, data, weights, step,
                                          n_samples_template, n_samples_data, n_templates, n_stations,
                                          n_components, n_corr, cc_sum, normalize, 0, nullptr);
}

}  // extern "C"
