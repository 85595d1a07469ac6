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
// masked/centred templates, running sums over the whole trace of d^2 (exact
// 64-bit fixed point) and of d (float pairs), so that any window length is a
// few operations, the
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

__global__ void channel_centre_kernel(const float *, int, float *);
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

// Running sums per channel for windows of any length, in three phases (block
// sums, their exclusive scan per channel, the scan inside each block plus its
// offset):
//  * of d'^2 (d' = d - mu; d for 'short') as 64-bit integers in a unit q of
//    the channel (a power of two, its energy times 2^-60): each square, split
//    exactly by FMA into two floats, is rounded to the unit, and the integer
//    sums are exact, so a window's energy is an exact difference -- only the
//    rounding of its own n squares remains, at most n q, whatever was summed
//    before it.  (A floating-point running sum loses the digits of everything
//    summed before the window: after a large transient a quiet window holds
//    1e-10 of the channel's running energy.)
//  * of d' ('full') as normalised float pairs hi = fl(P), lo = P - hi summed in
//    double-float FP32 arithmetic: the window sum of d' enters the centred
//    energy multiplied by the window mean, so its cancellation error stays far
//    below float rounding of the energy.

// The fixed-point unit q[ch] of the running sums of d'^2: 2^(e - 60) with the
// channel energy below 2^e, so that no running sum exceeds 2^61 units
// (clamped to the normal float range).  Two kernels: the energy of every
// block of kPrefixBlock samples (double-float, all SMs busy), then the sum of
// a channel's block energies in block order (so the unit does not depend on
// scheduling) and the unit.
// grid (blocks, SC), 256 threads
__global__ void channel_energy_kernel(const float *__restrict__ data, int N, const float *__restrict__ mu,
                                      float *__restrict__ part, int nblk)
{
    __shared__ float2 red[8];
    const int ch = blockIdx.y, blk = blockIdx.x;
    const float m = mu ? mu[ch] : 0.0f;
    const float *src = data + (size_t)ch * N;
    const int i0 = blk * kPrefixBlock, i1 = min(N, i0 + kPrefixBlock);
    constexpr int per = kPrefixBlock / 256;  // loads in flight per thread
    float x[per];
#pragma unroll
    for (int e = 0; e < per; e++) {
        const int i = i0 + e * 256 + threadIdx.x;
        x[e] = i < i1 ? __ldg(src + i) - m : 0.0f;
    }
    float h = 0.0f, l = 0.0f;
#pragma unroll
    for (int e = 0; e < per; e++) {
        const float sq = x[e] * x[e];
        pair_add(h, l, sq, fmaf(x[e], x[e], -sq));
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float yh = __shfl_down_sync(0xffffffffu, h, o), yl = __shfl_down_sync(0xffffffffu, l, o);
        pair_add(h, l, yh, yl);
    }
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = make_float2(h, l);
    __syncthreads();
    if (threadIdx.x == 0) {
        float th = 0.0f, tl = 0.0f;
        for (int i = 0; i < 8; i++)
            pair_add(th, tl, red[i].x, red[i].y);
        part[(size_t)ch * nblk + blk] = th + tl;
    }
}

// grid SC, 32 threads: the channel's block energies summed in block order (each
// lane a contiguous run, then the lanes in order), and its unit
__global__ void channel_unit_kernel(const float *__restrict__ part, int nblk, float *__restrict__ unit)
{
    const int ch = blockIdx.x, lane = threadIdx.x;
    const float *p = part + (size_t)ch * nblk;
    const int per = (nblk + 31) / 32, b0 = lane * per, b1 = min(nblk, b0 + per);
    float h = 0.0f, l = 0.0f;
    for (int b = b0; b < b1; b++)
        pair_add(h, l, p[b], 0.0f);
    for (int o = 1; o < 32; o <<= 1) {  // lane 0 ends with lanes 0..31 in order
        const float yh = __shfl_down_sync(0xffffffffu, h, o), yl = __shfl_down_sync(0xffffffffu, l, o);
        if ((lane & (2 * o - 1)) == 0)
            pair_add(h, l, yh, yl);
    }
    if (lane == 0) {
        int e = 0;
        // the sum rounded up by a margin, so that the float total cannot undershoot it
        frexpf((h + l) * 1.0001f, &e);
        unit[ch] = h + l > 0.0f ? ldexpf(1.0f, max(e - 60, -126)) : 1.0f;
    }
}

// d'^2 in units of 1 / inv_unit, as the two roundings of its exact float split
__device__ __forceinline__ long long fixed_square(float v, float inv_unit)
{
    const float sq = v * v;
    return __float2ll_rn(sq * inv_unit) + __float2ll_rn(fmaf(v, v, -sq) * inv_unit);
}

// Phase 1, grid (blocks, SC), 256 threads: block sums.
__global__ void prefix_block_kernel(const float *__restrict__ data, int N, const float *__restrict__ mu,
                                    const float *__restrict__ unit, long long *__restrict__ bs2,
                                    float2 *__restrict__ bs1, int nblk)
{
    __shared__ long long r2[32];
    __shared__ float2 r1[32];
    const int ch = blockIdx.y, blk = blockIdx.x;
    const float m = mu ? mu[ch] : 0.0f, inv_unit = 1.0f / unit[ch];
    const float *src = data + (size_t)ch * N;
    long long s2 = 0;
    float h1 = 0.0f, l1 = 0.0f;
    const int i0 = blk * kPrefixBlock, i1 = min(N, i0 + kPrefixBlock);
    constexpr int per = kPrefixBlock / 256;  // loads in flight per thread
    float x[per];
#pragma unroll
    for (int e = 0; e < per; e++) {
        const int i = i0 + e * 256 + threadIdx.x;
        x[e] = i < i1 ? __ldg(src + i) - m : 0.0f;
    }
#pragma unroll
    for (int e = 0; e < per; e++) {
        s2 += fixed_square(x[e], inv_unit);
        pair_add(h1, l1, x[e], 0.0f);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s2 += __shfl_down_sync(0xffffffffu, s2, o);
        const float c = __shfl_down_sync(0xffffffffu, h1, o), d = __shfl_down_sync(0xffffffffu, l1, o);
        pair_add(h1, l1, c, d);
    }
    if ((threadIdx.x & 31) == 0) {
        r2[threadIdx.x >> 5] = s2;
        r1[threadIdx.x >> 5] = make_float2(h1, l1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long a = 0;
        float c = 0.0f, d = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            a += r2[i];
            pair_add(c, d, r1[i].x, r1[i].y);
        }
        bs2[(size_t)ch * nblk + blk] = a;
        bs1[(size_t)ch * nblk + blk] = pair_normalise(c, d);
    }
}

// Phase 2, one warp per channel: exclusive scan of the block sums -- each lane
// a contiguous run of blocks, the run totals scanned across the lanes (fixed
// order, so the float pairs round the same way every time).
__global__ void prefix_offsets_kernel(long long *bs2, float2 *bs1, int nblk, int SC)
{
    const int ch = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (ch >= SC)
        return;  // whole warps
    long long *p2 = bs2 + (size_t)ch * nblk;
    float2 *p1 = bs1 + (size_t)ch * nblk;
    const int per = (nblk + 31) / 32, b0 = min(nblk, lane * per), b1 = min(nblk, b0 + per);
    long long a = 0;
    float h = 0.0f, l = 0.0f;
    for (int b = b0; b < b1; b++) {  // this lane's run total
        a += p2[b];
        const float2 y = p1[b];
        pair_add(h, l, y.x, y.y);
    }
    // inclusive scan of the run totals over the lanes, then this lane's exclusive offset
    long long ia = a;
    float ih = h, il = l;
    for (int o = 1; o < 32; o <<= 1) {
        const long long ya = __shfl_up_sync(0xffffffffu, ia, o);
        const float yh = __shfl_up_sync(0xffffffffu, ih, o), yl = __shfl_up_sync(0xffffffffu, il, o);
        if (lane >= o) {
            ia += ya;
            float th = yh, tl = yl;  // earlier lanes first
            pair_add(th, tl, ih, il);
            ih = th;
            il = tl;
        }
    }
    long long ea = __shfl_up_sync(0xffffffffu, ia, 1);
    float eh = __shfl_up_sync(0xffffffffu, ih, 1), el = __shfl_up_sync(0xffffffffu, il, 1);
    if (lane == 0) {
        ea = 0;
        eh = el = 0.0f;
    }
    float2 b = pair_normalise(eh, el);
    for (int k = b0; k < b1; k++) {
        const long long x = p2[k];
        const float2 y = p1[k];
        p2[k] = ea;
        p1[k] = b;
        ea += x;
        pair_add(b.x, b.y, y.x, y.y);
        b = pair_normalise(b.x, b.y);
    }
}

// Phase 3, grid (blocks, SC), 256 threads: inclusive scan of the block plus
// its offset -> P2[ch][i + 1] = sum_{x <= i} d'^2 in units (P2[ch][0] = 0)
// and, for 'full', P1 of d' and the centred data.
__global__ void prefix_write_kernel(const float *__restrict__ data, int N, const float *__restrict__ mu,
                                    const float *__restrict__ unit, const long long *__restrict__ bs2,
                                    const float2 *__restrict__ bs1, int nblk,
                                    long long *__restrict__ pre2q, float2 *__restrict__ pre1f,
                                    float *__restrict__ dcen)
{
    __shared__ long long part2[32];
    __shared__ float2 part1[32];
    const int ch = blockIdx.y, blk = blockIdx.x;
    const float m = mu ? mu[ch] : 0.0f, inv_unit = 1.0f / unit[ch];
    const float *src = data + (size_t)ch * N;
    const int i0 = blk * kPrefixBlock;
    constexpr int per = kPrefixBlock / 256;  // 8 consecutive samples per thread
    long long v2[per];                       // running sums of this thread
    float2 v1[per];
    long long s2 = 0;
    float h1 = 0.0f, l1 = 0.0f;
#pragma unroll
    for (int e = 0; e < per; e++) {
        const int i = i0 + threadIdx.x * per + e;
        float v = 0.0f;
        if (i < N) {
            v = src[i] - m;
            if (dcen)
                dcen[(size_t)ch * N + i] = v;
        }
        s2 += fixed_square(v, inv_unit);
        pair_add(h1, l1, v, 0.0f);
        v2[e] = s2;
        v1[e] = make_float2(h1, l1);
    }
    // inclusive warp scan of the thread totals, then the exclusive value of this thread
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long x2 = s2;
    float x1 = h1, y1 = l1;
    for (int o = 1; o < 32; o <<= 1) {
        const long long a = __shfl_up_sync(0xffffffffu, x2, o);
        const float c = __shfl_up_sync(0xffffffffu, x1, o), d = __shfl_up_sync(0xffffffffu, y1, o);
        if (lane >= o) {
            x2 += a;
            pair_add(x1, y1, c, d);
        }
    }
    if (lane == 31) {
        part2[wid] = x2;
        part1[wid] = make_float2(x1, y1);
    }
    long long e2 = __shfl_up_sync(0xffffffffu, x2, 1);
    float e1h = __shfl_up_sync(0xffffffffu, x1, 1), e1l = __shfl_up_sync(0xffffffffu, y1, 1);
    if (lane == 0) {
        e2 = 0;
        e1h = e1l = 0.0f;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // warp offsets, starting from the block's offset
        long long a = bs2[(size_t)ch * nblk + blk];
        const float2 o1 = bs1[(size_t)ch * nblk + blk];
        float c = o1.x, d = o1.y;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            const long long p = part2[k];
            const float2 q = part1[k];
            part2[k] = a;
            part1[k] = make_float2(c, d);
            a += p;
            pair_add(c, d, q.x, q.y);
        }
    }
    __syncthreads();
    const long long o2 = part2[wid] + e2;
    float oh1 = part1[wid].x, ol1 = part1[wid].y;
    pair_add(oh1, ol1, e1h, e1l);
    long long *p2 = pre2q + (size_t)ch * (N + 1);
    float2 *p1 = pre1f ? pre1f + (size_t)ch * (N + 1) : nullptr;
    if (blk == 0 && threadIdx.x == 0) {
        p2[0] = 0;
        if (p1)
            p1[0] = make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int e = 0; e < per; e++) {
        const int i = i0 + threadIdx.x * per + e;
        if (i < N) {
            p2[i + 1] = o2 + v2[e];
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
    int *k_lo = nullptr;
    float *zweight = nullptr, *consts = nullptr, *tmask = nullptr, *tsum = nullptr, *mu = nullptr,
          *dcen = nullptr;
    long long *bs2 = nullptr, *pre2q = nullptr;
    float2 *bs1 = nullptr, *pre1f = nullptr;
    float *unit = nullptr, *epart = nullptr;
    const int nblk = (N + kPrefixBlock - 1) / kPrefixBlock;
    if ((rc = ws.get(&k_lo, 2 * (size_t)T, "template ranges")) ||
        (rc = ws.get(&zweight, (size_t)T * SC, "Fisher-z weights")) ||
        (rc = ws.get(&consts, 3 * (size_t)T, "transform constants")) ||
        (rc = ws.get(&tmask, (size_t)T * SC * L, "masked templates")) ||
        (rc = ws.get(&pre2q, (size_t)SC * (N + 1), "running sums of d^2")) ||
        (rc = ws.get(&unit, (size_t)SC, "fixed-point units")) ||
        (rc = ws.get(&epart, (size_t)SC * nblk, "block energies")) ||
        (rc = ws.get(&bs2, (size_t)SC * nblk, "block sums")) ||
        (rc = ws.get(&bs1, (size_t)SC * nblk, "block sums")))
        return rc;
    if (full && ((rc = ws.get(&tsum, (size_t)T * SC, "template sums")) ||
                 (rc = ws.get(&mu, (size_t)SC, "channel centres")) ||
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
        channel_centre_kernel<<<SC, 1024, 0, s>>>(a.data, N, mu);
    channel_energy_kernel<<<dim3(nblk, SC), 256, 0, s>>>(a.data, N, mu, epart, nblk);
    channel_unit_kernel<<<SC, 32, 0, s>>>(epart, nblk, unit);
    prefix_block_kernel<<<dim3(nblk, SC), 256, 0, s>>>(a.data, N, mu, unit, bs2, bs1, nblk);
    prefix_offsets_kernel<<<(SC + 3) / 4, 128, 0, s>>>(bs2, bs1, nblk, SC);  // a warp per channel
    prefix_write_kernel<<<dim3(nblk, SC), 256, 0, s>>>(a.data, N, mu, unit, bs2, bs1, nblk, pre2q,
                                                        pre1f, dcen);
    count_launch(full ? 10 : 9);
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
    P.pre2q = pre2q;
    P.unit2 = unit;
    P.pre1f = pre1f;
    P.zweight = zweight;
    P.vp_norm = P.vp_bias = P.vp_scale = nullptr;
    int precision = FMF_FLAG_PRECISION_OF(a.flags);
    if (precision == FMF_PREC_AUTO && (rc = choose_auto_precision(P, ws, s, &precision)))
        return rc;
    set_last_precision(precision);
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
                unsigned long long *queue = nullptr;
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
    const bool out_pinned = host_is_pinned(host_out);
    for (int c = 0; c < n_chunks; c++) {
        const int t0 = bounds[c], nt = bounds[c + 1] - bounds[c];
        if (nt <= 0)
            continue;
        if (!out_pinned)
            populate_host(host_out + (size_t)t0 * a.n_corr, (size_t)nt * row_bytes);  // while kernels run
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
    // FMF_FLAG_PRECISION is two bits: every value is a precision (FMF_PREC_AUTO included)
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
    return fmf_last_precision() != FMF_PREC_FP32 ? collect_device_errors() : FMF_OK;  // the form that ran
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
