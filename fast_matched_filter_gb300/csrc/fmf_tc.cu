// fmf_tc.cu -- tensor-core (tcgen05 / TMEM) matched filter, split-BF16 form.
//
// Same outputs as the plain form (fmf_plain.cu); the numerator sum_j t[j]*d[k*step+mo+j]
// runs on the 5th-generation tensor cores.  Every per-channel correlation is
// a Toeplitz x Hankel product, laid out so that neither matrix is built in
// full:
//
//   Output index i = I0 + Q*a + b of one template and channel (I0 a multiple
//   of Q = 128, a = lag block, b = phase in [0, Q)) needs data samples
//   p + Q*a + b + j with p = I0 + mo.  Writing p = Q*r0 + s (0 <= s < Q) and
//   k = s + b + j,
//       X[i] = sum_k A[Q-1-b][k] * B[a][k],
//       A[m][k] = t[k + m - (Q-1+s)]          (template Toeplitz, M = 128 rows)
//       B[a][k] = d[Q*(r0 + a) + k]            (data Hankel, N = NB lag blocks)
//   with K = s + L + Q - 1 (rounded to 16; the leading s & ~15 columns are
//   skipped because they multiply zeros).
//
//   * B is a view of the data stored "column-blocked": per channel, for each
//     16-byte column block cb of a Q-sample row, all rows are contiguous,
//     G[cb][row][8].  In the canonical no-swizzle K-major layout (8-row x
//     16-byte core matrices) rows are then 16 bytes apart, so B for any row
//     offset and any K step is a descriptor (start = cb*R*16 + row*16,
//     leading-dimension offset R*16, stride offset 128) -- no Hankel copy.
//   * A is a view of 8 shifted copies of the template interleaved in
//     128-byte blocks, W[n][e][c] = t[8n + e + c - (Q-1+s)]: core matrix
//     (row group g, K group k') of A is block W[g + k'], so both descriptor
//     offsets are 128 bytes.  W is 8/Q of the Toeplitz matrix.
//   * step > 1: taps j = step*q + phi read the decimated stream
//     d_psi[x] = d[step*x + psi]; each phase is a unit-step correlation with
//     its own template taps and moveout, accumulated into the same TMEM tile.
//   * Split-BF16: operands are bf16 hi + lo (x = hi + lo to 2^-16 relative);
//     three MMAs per K step (hi*hi, hi*lo, lo*hi) accumulate in FP32 in TMEM.
//
// Persistent CTAs (one per SM) take items (one template x NB*Q consecutive
// outputs, all channels) from a tile queue:
//   warp 0      producer: claims items, cp.async.bulk (TMA bulk copies) of the
//               data rows and template blocks of one (channel, phase) stage
//               into stage buffer b (b = parity of the channel's running
//               index), mbarrier complete_tx;
//   warps 1, 2  MMA issuers: one thread each issues tcgen05.mma for the
//               channels of its parity, from its stage buffer into its FP32
//               accumulator in TMEM, and commits to the barriers (a single
//               issuing thread cannot keep the tensor pipe busy);
//   warp 1      also allocates the TMEM (two accumulators + the network sum);
//   warps 4-11  epilogue: tcgen05.ld of the accumulator, normalisation by the
//               window statistics, threshold, weighted network sum in TMEM
//               (channel order, fused multiply-add), outputs.
// Instantiations: tc_persistent<VAR, PARTS>.  VAR: per-channel template
// lengths (the issuers cut each channel's K range at its own taps; 16 epilogue
// warps, warps 4-19, form window sums from per-channel running sums and add
// atanh(cc) * z).  PARTS: the items of a small search are split into channel
// parts whose partial sums a second kernel adds in order.
// Every wait is bounded (globaltimer); on timeout the CTA raises an error
// word, stops issuing, waits for its own copies/MMAs (bounded) and frees TMEM.
#include <cfloat>
#include <type_traits>

#include <cuda_bf16.h>

#include "fmf_common.cuh"

namespace fmf {

constexpr int TC_Q = 128;
constexpr int TC_CB = TC_Q / 8;
// Epilogue warps (2 per TMEM lane quarter; 4 per quarter for per-channel
// template lengths, whose epilogue does more arithmetic per output and needs
// more warps to hide its latency) + producer, 2 MMA issuers, 1 idle warp.
constexpr int tc_epi_warps(bool var) { return var ? 16 : 8; }
constexpr int tc_threads(bool var) { return 32 * (4 + tc_epi_warps(var)); }
constexpr int TC_TG = 16;  // templates interleaved per group of CTAs (L2 reuse of data rows)
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // 2 s per wait


// One search of a persistent launch (tile-queue items [item_begin, item_begin + n_tiles*T)).
struct TcProb {
    Problem P;                    // sizes, epilogue inputs, output
    const uint16_t *g_hi, *g_lo;  // bf16 bits, data streams [SC][step][CB][rows_total][8]
    const uint16_t *w_hi, *w_lo;  // bf16 bits, template blocks [T][SC][step][NW][64]
    const int *mu;                // [T][SC][step] moveout of each phase in its stream
    const int *psi;               // [T][SC][step] stream of each phase
    long long item_begin;         // first tile-queue item of this search
    int R;                        // data rows per stage
    int NW;                       // 128-byte template blocks per (template, channel, phase)
    int rows_total;               // rows per (channel, stream) in the data streams
    int row_front;                // rows of zero padding before sample 0
    int n_tiles;                  // output tiles of nb*128 indices
    int tg;                       // templates interleaved per group of items
    int nb;                       // lag blocks per tile (MMA N): 32, 64 or 128
    int parts;                    // k >= 1: the channels of a (tile, template) in k
                                  // ranges [j SC / k, (j + 1) SC / k) on k CTAs (items
                                  // j = 0..k-1 adjacent); their network sums go to
                                  // part_out[j][t][lag] and are added in order j after
                                  // the launch (a fixed order: deterministic results)
    float *part_out;
};

struct TcBatch {
    TcProb prob[TC_MAX_PROBS];
    int n_probs;
    int split;                    // 1: hi/lo, three products; 0: single bf16 product
    int stage_bytes;              // bytes of one pipeline stage (largest search)
    long long total_items;
    unsigned long long *queue;    // tile-queue head, zero before the launch
    unsigned *err;                // device error word
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait on an mbarrier phase.  Returns false when the CTA aborted or
// when this wait gave up after `limit_ns` (then it raises the error word and
// the abort flag).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                          unsigned *err, unsigned code,
                                          unsigned long long limit_ns = TC_WAIT_NS)
{
    if (mbar_try(bar, parity))
        return true;
    unsigned long long t0 = gtimer();
    for (unsigned it = 1;; it++) {
        if (mbar_try(bar, parity))
            return true;
        if ((it & 63) == 0) {
            if (*abort_flag)
                return false;
            if (gtimer() - t0 > limit_ns) {
                atomicOr(err, code);
                *abort_flag = 1;
                return false;
            }
        }
    }
}

// Warp-uniform form: lane 0 waits, the result is broadcast to the warp.
__device__ __forceinline__ bool mbar_wait_warp(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                               unsigned *err, unsigned code)
{
    int ok = 0;
    if ((threadIdx.x & 31) == 0)
        ok = mbar_wait(bar, parity, abort_flag, err, code) ? 1 : 0;
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor, no swizzle (layout type 0), version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 32 bits, 16 consecutive columns per thread
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; i++)
        v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float *v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15]))
        : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float *v)
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// CH consecutive accumulator columns of this warp's 32 lanes (CH = 8 or 16)
template <int CH>
__device__ __forceinline__ void tmem_ldc(uint32_t taddr, float *v)
{
    if constexpr (CH == 16)
        tmem_ld16(taddr, v);
    else
        tmem_ld8(taddr, v);
}
template <int CH>
__device__ __forceinline__ void tmem_stc(uint32_t taddr, const float *v)
{
    if constexpr (CH == 16)
        tmem_st16(taddr, v);
    else
        tmem_st8(taddr, v);
}

// ------------------------------------------------------------------ preprocessing
__device__ __forceinline__ void split_bf16(float x, uint16_t &hi, uint16_t &lo)
{
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(l);
}

// G[ch][psi][cb][r][e] = split(d[ch][step*(Q*(r - row_front) + 8*cb + e) + psi]), zero outside [0, N).
// One thread per 16-byte row chunk.
__global__ void tc_data_kernel(const float *__restrict__ data, int N, int SC, int step,
                               int rows_total, int row_front, uint16_t *__restrict__ g_hi,
                               uint16_t *__restrict__ g_lo)
{
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)SC * step * TC_CB * rows_total;
    if (idx >= total)
        return;
    int r = (int)(idx % rows_total);
    long long rest = idx / rows_total;
    int cb = (int)(rest % TC_CB);
    rest /= TC_CB;
    int psi = (int)(rest % step);
    int ch = (int)(rest / step);
    long long x0 = (long long)TC_Q * (r - row_front) + 8 * cb;
    const float *src = data + (size_t)ch * N;
    uint16_t h[8], l[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
        long long pos = (long long)step * (x0 + e) + psi;
        float v = (x0 + e >= 0 && pos < N) ? src[pos] : 0.0f;
        split_bf16(v, h[e], l[e]);
    }
    uint4 hv, lv;
    hv.x = h[0] | ((uint32_t)h[1] << 16);
    hv.y = h[2] | ((uint32_t)h[3] << 16);
    hv.z = h[4] | ((uint32_t)h[5] << 16);
    hv.w = h[6] | ((uint32_t)h[7] << 16);
    lv.x = l[0] | ((uint32_t)l[1] << 16);
    lv.y = l[2] | ((uint32_t)l[3] << 16);
    lv.z = l[4] | ((uint32_t)l[5] << 16);
    lv.w = l[6] | ((uint32_t)l[7] << 16);
    reinterpret_cast<uint4 *>(g_hi)[idx] = hv;
    if (g_lo)
        reinterpret_cast<uint4 *>(g_lo)[idx] = lv;
}

// W[t][ch][phi][n][e][c] = split(tphi[8n + e + c - (Q-1+s)]), tphi[q] = tpl[step*q + phi],
// s = mu mod Q, mu = floor((mo + phi) / step), psi = mo + phi - step*mu.
// One thread per (block n, row e).
__global__ void tc_template_kernel(const float *__restrict__ tpl, const int *__restrict__ mo, int T,
                                   int SC, int L, int step, int NW, uint16_t *__restrict__ w_hi,
                                   uint16_t *__restrict__ w_lo, int *__restrict__ mu_out,
                                   int *__restrict__ psi_out)
{
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)T * SC * step * NW * 8;
    if (idx >= total)
        return;
    int e = (int)(idx & 7);
    long long rest = idx >> 3;
    int n = (int)(rest % NW);
    long long meta = rest / NW;  // (t*SC + ch)*step + phi
    int phi = (int)(meta % step);
    long long row = meta / step;  // t*SC + ch
    int m = mo[row] + phi;
    int mu = m >= 0 ? m / step : -((-m + step - 1) / step);
    int psi = m - step * mu;
    int s = ((mu % TC_Q) + TC_Q) % TC_Q;
    if (n == 0 && e == 0) {
        mu_out[meta] = mu;
        psi_out[meta] = psi;
    }
    const float *tp = tpl + row * L;
    uint16_t h[8], l[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
        int q = 8 * n + e + c - (TC_Q - 1 + s);
        int j = step * q + phi;
        float v = (q >= 0 && j < L) ? tp[j] : 0.0f;
        split_bf16(v, h[c], l[c]);
    }
    uint4 hv, lv;
    hv.x = h[0] | ((uint32_t)h[1] << 16);
    hv.y = h[2] | ((uint32_t)h[3] << 16);
    hv.z = h[4] | ((uint32_t)h[5] << 16);
    hv.w = h[6] | ((uint32_t)h[7] << 16);
    lv.x = l[0] | ((uint32_t)l[1] << 16);
    lv.y = l[2] | ((uint32_t)l[3] << 16);
    lv.z = l[4] | ((uint32_t)l[5] << 16);
    lv.w = l[6] | ((uint32_t)l[7] << 16);
    reinterpret_cast<uint4 *>(w_hi)[idx] = hv;
    if (w_lo)
        reinterpret_cast<uint4 *>(w_lo)[idx] = lv;
}

// ------------------------------------------------------------------ persistent kernel
// Decodes a tile-queue item: search p, output tile, template t.  Items of one
// search are ordered so that groups of `tg` templates sweep the tiles together.
template <bool PARTS>
__device__ __forceinline__ void decode_item(const TcBatch &B, long long item, int &p, int &tile, int &t,
                                            int &c_begin, int &c_end, int &part)
{
    int lo = 0, hi = B.n_probs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B.prob[mid].item_begin <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    p = lo;
    const TcProb &pr = B.prob[p];
    long long local = item - pr.item_begin;
    c_begin = 0;
    c_end = pr.P.SC;
    part = 0;
    if (PARTS) {  // the parts of a (tile, template) are adjacent items
        const int k = pr.parts;
        part = (int)(local % k);
        local /= k;
        c_begin = (int)((long long)part * pr.P.SC / k);
        c_end = (int)((long long)(part + 1) * pr.P.SC / k);
    }
    const long long per_group = (long long)pr.n_tiles * pr.tg;
    const int grp = (int)(local / per_group);
    const long long rem = local - (long long)grp * per_group;
    const int tg0 = grp * pr.tg;
    const int tgn = min(pr.tg, pr.P.T - tg0);
    tile = (int)(rem / tgn);
    t = tg0 + (int)(rem % tgn);
}

constexpr int TC_NB_MAX = 128;  // largest tile; TMEM columns: D0 [0,128), D1 [128,256), sum [256,384)
constexpr int TC_NACC = 2;      // accumulator buffers

// 1/sqrt(x), one approximate MUFU operation; subnormal x is flushed to zero
// (result +inf).
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// atanh(y) in FP32 for the Fisher-z network sum, at most a few ulp from the
// exact value (the accuracy of the CUDA library's atanhf) with far fewer
// instructions for the common small arguments:
//  |y| <= 1/4: the Maclaurin series y + y^3/3 + ... + y^13/13 (the first
//    omitted term is below 2^-25 of the result);
//  1/4 < |y| < 1: atanh(a) = ln(q) / 2 with q = (1 + a) / (1 - a); q = 2^k m
//    with m in [sqrt(1/2), sqrt(2)) and ln(m) = 2 atanh(s), s = (m - 1) / (m + 1),
//    |s| <= 0.1716, from the same series to s^9/9;
//  |y| = 1 gives +-inf, |y| > 1 and NaN give NaN.
__device__ __forceinline__ float atanh_series(float y)
{
    const float z = y * y;
    float p = fmaf(1.0f / 13.0f, z, 1.0f / 11.0f);
    p = fmaf(p, z, 1.0f / 9.0f);
    p = fmaf(p, z, 1.0f / 7.0f);
    p = fmaf(p, z, 1.0f / 5.0f);
    p = fmaf(p, z, 1.0f / 3.0f);
    return fmaf(y * z, p, y);
}

__device__ __forceinline__ float atanh_reduced(float y)
{
    const float a = fabsf(y);
    if (!(a < 1.0f))  // 1, above 1, NaN
        return a == 1.0f ? copysignf(INFINITY, y) : __int_as_float(0x7fc00000);
    const float q = __fdividef(1.0f + a, 1.0f - a);  // in (5/3, 2^25] for a > 1/4
    const int bits = __float_as_int(q);
    const int k = (bits - 0x3f3504f3) >> 23;  // 0x3f3504f3 = sqrt(1/2)
    const float m = __int_as_float(bits - (k << 23));
    const float s = __fdividef(m - 1.0f, m + 1.0f);
    const float z = s * s;
    float p = fmaf(1.0f / 9.0f, z, 1.0f / 7.0f);
    p = fmaf(p, z, 1.0f / 5.0f);
    p = fmaf(p, z, 1.0f / 3.0f);
    float r = fmaf(s * z, p, s);                         // ln(m) / 2
    r = fmaf((float)k, 0.5f * 0.693145751953125f, r);    // + k ln2 / 2 (ln2 in two parts)
    r = fmaf((float)k, 0.5f * 1.4286068203094172e-06f, r);
    return copysignf(r, y);
}

// Called by all 32 lanes of a warp together: the series on every lane, the
// reduction only when some lane of the warp needs it (no divergent branch;
// the common case, every |y| <= 1/4, skips it).
__device__ __forceinline__ float fisher_atanh(float y)
{
    const bool big = !(fabsf(y) <= 0.25f);  // NaN included
    float r = atanh_series(y);
    if (__any_sync(0xffffffffu, big)) {
        const float g = atanh_reduced(y);
        r = big ? g : r;
    }
    return r;
}

// every lane of every warp takes part (the tail reads a dummy value)
__global__ void fisher_atanh_kernel(const float *__restrict__ y, float *__restrict__ out, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const float r = fisher_atanh(i < n ? y[i] : 0.0f);
    if (i < n)
        out[i] = r;
}

int launch_fisher_atanh(const float *y, float *out, long long n, cudaStream_t s)
{
    if (n <= 0)
        return FMF_OK;
    fisher_atanh_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(y, out, n);
    count_launch();
    return check_launch("fisher_atanh_kernel");
}

// VAR: per-channel template lengths (Problem::ntap set in every search of the
// batch), a separate instantiation so that the fixed-length epilogue keeps
// its registers.  PARTS: every search runs its items as channel parts
// (TcProb::parts), a separate instantiation for the same reason.  NORM: 0 every
// search 'short', 1 every search 'full', -1 each search's own (a batch mixing
// both); the fixed modes drop the other mode's epilogue code.
template <bool VAR, bool PARTS, int NORM>
__global__ void __launch_bounds__(tc_threads(VAR), 1) tc_persistent(const __grid_constant__ TcBatch B)
{
    constexpr int TC_EPI_WARPS = tc_epi_warps(VAR);
    extern __shared__ __align__(1024) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int split = B.split;

    uint8_t *bar_base = smem + 2 * (size_t)B.stage_bytes;
    const uint32_t full0 = smem_u32(bar_base), empty0 = full0 + 16, dfull0 = full0 + 32,
                   dempty0 = full0 + 48, fin = full0 + 64, ifull0 = full0 + 72, iempty0 = full0 + 104;
    long long *ring = reinterpret_cast<long long *>(bar_base + 136);  // 4 item slots
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bar_base + 168);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bar_base + 172);

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; i++) {
            mbar_init(full0 + 8 * i, 1);
            mbar_init(empty0 + 8 * i, 1);
            mbar_init(dfull0 + 8 * i, 1);
            mbar_init(dempty0 + 8 * i, TC_EPI_WARPS);
        }
        mbar_init(fin, 2);  // one commit per MMA issuer
        for (int i = 0; i < 4; i++) {
            mbar_init(ifull0 + 8 * i, 1);
            mbar_init(iempty0 + 8 * i, 2 + TC_EPI_WARPS);  // MMA issuers + epilogue warps
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    constexpr uint32_t TMEM_COLS = 512;  // D0, D1, sum at columns 0, 128, 256 (one CTA per SM)
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_holder)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    const long long total = B.total_items;

    if (warp == 0) {
        // ---------------------------------------------------------- producer + tile queue
        // Stage buffer b holds the stages of the channels whose running index g
        // (over the active channels of all items, in order) has parity b; MMA
        // issuer b consumes them.  uses[b] counts the stages put in buffer b.
        int uses[2] = {0, 0};
        long long g = 0;
        bool ok = true;
        for (long long q = 0; ok; q++) {
            const int slot = (int)(q & 3);
            long long item = total;
            if (lane == 0) {
                bool got = q < 4 || mbar_wait(iempty0 + 8 * slot, (uint32_t)(((q >> 2) - 1) & 1), abort_flag,
                                              B.err, 1u);
                if (got && !*abort_flag)
                    item = (long long)atomicAdd(B.queue, 1ull);
                ring[slot] = item;
                mbar_arrive(ifull0 + 8 * slot);
            }
            item = __shfl_sync(0xffffffffu, item, 0);  // warp-uniform decision
            if (item >= total)
                break;
            int p, tile, t, c_begin, c_end, part;
            decode_item<PARTS>(B, item, p, tile, t, c_begin, c_end, part);
            const TcProb &pr = B.prob[p];
            const Problem &P = pr.P;
            const int nb = pr.nb;
            const long long I0 = (long long)tile * TC_Q * nb;
            if (!(I0 < P.k_hi[t] && I0 + (long long)TC_Q * nb > P.k_lo[t]))
                continue;
            const int SC = P.SC, step = P.step, R = pr.R, NW = pr.NW;
            const uint32_t data_bytes = (uint32_t)TC_CB * R * 16, wbytes = (uint32_t)NW * 128;
            const uint32_t w_off = (split ? 2u : 1u) * data_bytes;
            const float *w = P.w + (size_t)t * SC;
            // one stage: phase phi of channel ch into buffer b
            auto load_stage = [&](int ch, int phi, int b) -> bool {
                if (uses[b] >= 1 &&
                    !mbar_wait_warp(empty0 + 8 * b, (uses[b] - 1) & 1, abort_flag, B.err, 2u))
                    return false;
                const long long meta = ((long long)t * SC + ch) * step + phi;
                const int mu = pr.mu[meta], psi = pr.psi[meta];
                const int sres = ((mu % TC_Q) + TC_Q) % TC_Q;
                const long long r0 = (I0 + mu - sres) / TC_Q + pr.row_front;
                const uint32_t st = smem_u32(smem + (size_t)b * B.stage_bytes);
                if (lane == 0)
                    mbar_expect_tx(full0 + 8 * b, (split ? 2u : 1u) * (data_bytes + wbytes));
                __syncwarp();
                const int cb = lane & 15, hl = lane >> 4;
                if (hl == 0 || split) {
                    const uint16_t *src = (hl ? pr.g_lo : pr.g_hi) +
                                          ((((long long)ch * step + psi) * TC_CB + cb) * pr.rows_total + r0) * 8;
                    bulk_g2s(st + hl * data_bytes + cb * (uint32_t)R * 16, src, (uint32_t)R * 16,
                             full0 + 8 * b);
                }
                if (lane < (split ? 2 : 1)) {
                    const uint16_t *src = (lane ? pr.w_lo : pr.w_hi) + meta * NW * 64;
                    bulk_g2s(st + w_off + lane * wbytes, src, wbytes, full0 + 8 * b);
                }
                uses[b]++;
                return true;
            };
            auto next_active = [&](int ch) {
                while (ch < c_end && w[ch] == 0.0f)
                    ch++;
                return ch;
            };
            // active channels in order; with step > 1 two consecutive channels
            // have their phases interleaved, so that both buffers stay fed
            int ch = next_active(c_begin);
            while (ok && ch < c_end) {
                const int ch2 = step > 1 ? next_active(ch + 1) : c_end;
                const bool pair = ch2 < c_end;
                const int b = (int)(g & 1);
                for (int phi = 0; ok && phi < step; phi++) {
                    ok = load_stage(ch, phi, b);
                    if (ok && pair)
                        ok = load_stage(ch2, phi, b ^ 1);
                }
                g += pair ? 2 : 1;
                ch = next_active((pair ? ch2 : ch) + 1);
            }
        }
        // do not leave with copies in flight
        if (lane == 0)
            for (int b = 0; b < 2; b++)
                if (uses[b] >= 1)
                    mbar_wait(full0 + 8 * b, (uses[b] - 1) & 1, abort_flag, B.err, 0u);
        __syncwarp();
    } else if (warp == 1 || warp == 2) {
        // ---------------------------------------------------------- MMA issuers
        // Two issuing threads (one per warp, on two SM sub-partitions): one
        // thread cannot issue tcgen05.mma fast enough to keep the tensor pipe
        // busy.  Issuer m takes the active channels of parity m (running index
        // c over all items), stage buffer m and accumulator m.
        const int m = warp - 1;
        if (lane == 0) {
            int used = 0;  // stages consumed from buffer m
            long long c = 0;
            for (long long q = 0;; q++) {
                const int slot = (int)(q & 3);
                if (!mbar_wait(ifull0 + 8 * slot, (uint32_t)((q >> 2) & 1), abort_flag, B.err, 32u))
                    goto mma_done;
                const long long item = ring[slot];
                mbar_arrive(iempty0 + 8 * slot);
                if (item >= total)
                    break;
                int p, tile, t, c_begin, c_end, part;
                decode_item<PARTS>(B, item, p, tile, t, c_begin, c_end, part);
                const TcProb &pr = B.prob[p];
                const Problem &P = pr.P;
                const int nb = pr.nb;
                const long long I0 = (long long)tile * TC_Q * nb;
                if (!(I0 < P.k_hi[t] && I0 + (long long)TC_Q * nb > P.k_lo[t]))
                    continue;
                // kind::f16 descriptor: F32 accumulate, BF16 A and B, K-major, N = nb, M = 128
                const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(nb >> 3) << 17) |
                                       ((uint32_t)(TC_Q >> 4) << 24);
                const int SC = P.SC, step = P.step;
                const uint32_t data_bytes = (uint32_t)TC_CB * pr.R * 16, wbytes = (uint32_t)pr.NW * 128;
                const uint32_t w_off = (split ? 2u : 1u) * data_bytes;
                const uint32_t lbo_b = (uint32_t)pr.R * 16;
                const float *w = P.w + (size_t)t * SC;
                for (int ch = c_begin; ch < c_end; ch++) {
                    if (w[ch] == 0.0f)
                        continue;
                    if ((c & 1) != m) {  // the other issuer's channel
                        c++;
                        continue;
                    }
                    const int d = m;  // accumulator m, reused every second channel
                    if (c >= TC_NACC &&
                        !mbar_wait(dempty0 + 8 * d, ((c / TC_NACC) - 1) & 1, abort_flag, B.err, 4u))
                        goto mma_done;
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(d * TC_NB_MAX);
                    uint32_t acc = 0;
                    for (int phi = 0; phi < step; phi++, used++) {
                        const int s = m;
                        if (!mbar_wait(full0 + 8 * s, used & 1, abort_flag, B.err, 8u))
                            goto mma_done;
                        tc_fence_after();
                        const long long meta = ((long long)t * SC + ch) * step + phi;
                        const int mu = pr.mu[meta];
                        const int sres = ((mu % TC_Q) + TC_Q) % TC_Q;
                        int lphi = (P.L - phi + step - 1) / step;
                        if constexpr (VAR) {  // per-channel length: the taps past it are zeros, skip them
                            const int n = P.ntap[(size_t)t * SC + ch];
                            const int own = n > phi ? (n - phi + step - 1) / step : 0;
                            lphi = min(lphi, own);
                        }
                        const int k_first = sres & ~15;
                        const int k_end = (sres + lphi + TC_Q - 1 + 15) & ~15;
                        const uint32_t zhi = smem_u32(smem + (size_t)s * B.stage_bytes);
                        const uint32_t whi = zhi + w_off;
                        // Descriptors advance by additions: the start-address field (bits 0-13,
                        // 16-byte units) of an address below 256 KB never carries into the
                        // next field.  A: +256 bytes per K step (two 128-byte template blocks);
                        // B: +2 column blocks per K step inside a 128-wide K block, then the
                        // next data row (+16 bytes) from column block 0.
                        uint64_t ah = sdesc(whi + (uint32_t)(k_first >> 3) * 128u, 128, 128);
                        const uint64_t a_lo = wbytes >> 4, b_lo = data_bytes >> 4;
                        const uint64_t b0 = sdesc(zhi, lbo_b, 128);
                        const uint64_t b_step = (2u * lbo_b) >> 4;
                        int k = k_first;
                        while (k < k_end) {
                            const int blk_end = min(k_end, (k & ~(TC_Q - 1)) + TC_Q);
                            uint64_t bh = b0 + (((uint32_t)((k & (TC_Q - 1)) >> 3) * lbo_b +
                                                 (uint32_t)(k / TC_Q) * 16u) >> 4);
                            for (; k < blk_end; k += 16) {
                                mma_bf16(dt, ah, bh, idesc, acc);
                                acc = 1;
                                if (split) {
                                    mma_bf16(dt, ah, bh + b_lo, idesc, 1);
                                    mma_bf16(dt, ah + a_lo, bh, idesc, 1);
                                }
                                ah += 16;
                                bh += b_step;
                            }
                        }
                        mma_commit(empty0 + 8 * s);
                    }
                    mma_commit(dfull0 + 8 * d);
                    c++;
                }
            }
        mma_done:
            mma_commit(fin);
            mbar_wait(fin, 0, abort_flag, B.err, 0u);
        }
        __syncwarp();
    } else if (warp >= 4) {
        // ---------------------------------------------------------- epilogue
        // TC_EPI_WARPS warps: warp w reads TMEM lane quarter w % 4 (rows
        // 32*(w%4) + lane) and the NC columns [a0, a0 + NC) of the accumulators;
        // the network sum of its outputs lives in TMEM columns 2*NB + [a0, a0 + NC).
        constexpr int CH = VAR ? 8 : 16;  // columns per TMEM access and per batch of statistics loads
        const int quarter = warp & 3;
        const int cgroup = (warp - 4) >> 2;  // column group of this warp
        const int m = 32 * quarter + lane;   // accumulator row
        const int b = TC_Q - 1 - m;          // phase of that row
        const uint32_t lane_base = tmem + ((uint32_t)(32 * quarter) << 16);
        int c = 0;
        for (long long q = 0;; q++) {
            const int slot = (int)(q & 3);
            long long item = total;
            if (lane == 0) {
                if (mbar_wait(ifull0 + 8 * slot, (uint32_t)((q >> 2) & 1), abort_flag, B.err, 64u)) {
                    item = ring[slot];
                    mbar_arrive(iempty0 + 8 * slot);
                }
            }
            item = __shfl_sync(0xffffffffu, item, 0);
            if (item >= total)
                break;
            int p, tile, t, c_begin, c_end, part;
            decode_item<PARTS>(B, item, p, tile, t, c_begin, c_end, part);
            const TcProb &pr = B.prob[p];
            // per-item fields, once, into registers
            const int nb = pr.nb;
            const int NC = nb / (TC_EPI_WARPS / 4);  // columns of this thread (multiple of CH)
            const int a0 = cgroup * NC;
            const uint32_t s_cols = lane_base + (uint32_t)(TC_NACC * TC_NB_MAX + a0);
            const int SC = pr.P.SC, step = pr.P.step, n_corr = pr.P.n_corr, N = pr.P.N;
            const bool full = NORM >= 0 ? NORM == 1 : pr.P.normalize != 0;
            const bool nsum = pr.P.network_sum != 0;
            const float *__restrict__ stat_e = pr.P.stat_e;
            const float *__restrict__ sstp = pr.P.sst;
            const float *__restrict__ tsump = pr.P.tsum;
            float *outp = pr.P.out;
            const long long I0 = (long long)tile * TC_Q * nb;
            const int klo = pr.P.k_lo[t], khi = pr.P.k_hi[t];
            const bool busy = I0 < khi && I0 + (long long)TC_Q * nb > klo;
            // valid lag blocks of this thread: klo <= I0 + Q*a + b < khi
            const long long kb = I0 + b;
            const int a_lo = (int)max(0LL, (klo - kb + TC_Q - 1) / TC_Q) - a0;
            const int a_hi = (int)min((long long)nb, (khi - kb + TC_Q - 1) / TC_Q) - a0;
            const bool any = busy && a_hi > a_lo;
            // the whole warp's outputs of this item are valid (the usual case)
            const bool interior = __all_sync(0xffffffffu, a_lo <= 0 && a_hi >= NC);
            const long long qs = (long long)TC_Q * step;
            const int qs32 = TC_Q * step;
            const float *w = pr.P.w + (size_t)t * SC;
            const int *mo = pr.P.mo + (size_t)t * SC;
            bool first = true;
            for (int ch = c_begin; busy && ch < c_end; ch++) {
                const float wc = w[ch];
                if (wc == 0.0f)
                    continue;
                const int d = c % TC_NACC;
                const size_t row = (size_t)t * SC + ch;
                const float sst = sstp[row];
                const float ts = full ? tsump[row] : 0.0f;
                const long long u0 = (kb + (long long)TC_Q * a0) * step + mo[ch];
                // short: window energies; full: (centred energy, mean) pairs
                const float *__restrict__ se = VAR ? nullptr : stat_e + (size_t)ch * N + u0;
                const float2 *__restrict__ sem =
                    VAR ? nullptr : reinterpret_cast<const float2 *>(stat_e) + (size_t)ch * N + u0;
                float *oc = outp + ((size_t)t * n_corr + kb + (long long)TC_Q * a0) * SC + ch;
                // statistics: all loads of a chunk issued together (indices clamped into the
                // valid range) before any use; the first chunk before waiting for the accumulator
                float e[CH], mm[CH];
                auto load_chunk = [&](int c0) {
#pragma unroll
                    for (int i = 0; i < CH; i++) {
                        const int ac = min(max(c0 + i, a_lo), a_hi - 1);
                        if (full) {
                            const float2 em = any ? __ldg(sem + ac * qs) : make_float2(0.0f, 0.0f);
                            e[i] = em.x;
                            mm[i] = em.y;
                        } else {
                            e[i] = any ? __ldg(se + ac * qs) : 0.0f;
                            mm[i] = 0.0f;
                        }
                    }
                };
                if constexpr (!VAR)
                    load_chunk(0);
                // per-channel lengths: the channel's own length and Fisher-z weight, its
                // running sums (d^2 in fixed point, and d for full) at the first window of
                // the thread
                [[maybe_unused]] int ntap = 0;
                [[maybe_unused]] float zw = 0.0f, nf = 0.0f, inv_n = 0.0f, unit = 0.0f;
                [[maybe_unused]] const long long *pf = nullptr;
                [[maybe_unused]] const float2 *pg = nullptr;
                if constexpr (VAR) {
                    ntap = pr.P.ntap[row];
                    zw = pr.P.zweight[row];
                    unit = pr.P.unit2[ch];
                    pf = pr.P.pre2q + (size_t)ch * (N + 1) + u0;
                    pg = full ? pr.P.pre1f + (size_t)ch * (N + 1) + u0 : nullptr;
                    nf = (float)ntap;
                    inv_n = 1.0f / nf;
                }
                if (!mbar_wait_warp(dfull0 + 8 * d, (c / TC_NACC) & 1, abort_flag, B.err, 16u))
                    goto epilogue_done;
                tc_fence_after();
                const uint32_t dcols = lane_base + (uint32_t)(d * TC_NB_MAX + a0);
#pragma unroll 1
                for (int c0 = 0; c0 < NC; c0 += CH) {
                    if constexpr (!VAR) {
                        if (c0 > 0)
                            load_chunk(c0);
                    }
                    float x[CH], sv[CH];
                    tmem_ldc<CH>(dcols + c0, x);
                    if (nsum && !first)
                        tmem_ldc<CH>(s_cols + c0, sv);
                    tmem_wait_ld();
                    if (c0 + CH >= NC) {
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0)
                            mbar_arrive(dempty0 + 8 * d);
                    }
                    if constexpr (VAR) {
                        // window sums of the channel's own length from the running sums,
                        // the 'precise' threshold on the square root, and
                        // atanh(cc - 10 eps) * z into the network sum
                        // CHECK: some output of the warp lies outside the valid lags (clamped
                        // indices, masked sums); otherwise every one is valid
                        auto var_chunk = [&](auto check) {
                            constexpr bool CHECK = decltype(check)::value;
                            auto var_value = [&](int i, float num, float ssd) {
                                const int a = c0 + i;
                                // the threshold on sqrt(sst * ssd), as p * rsqrt(p); p = 0 gives
                                // NaN there, and p below the normal range (flushed) cannot pass it
                                const float p = sst * ssd, r = rsqrt_ftz(p);
                                const float cc = p * r > kThreshold ? num * r : 0.0f;
                                const float prev = first ? 0.0f : sv[i];
                                const float z = fmaf(fisher_atanh(cc - 10.0f * FLT_EPSILON), zw, prev);
                                sv[i] = (!CHECK || (a >= a_lo && a < a_hi)) ? z : prev;
                            };
                            // element offsets of the windows (32-bit: at most NB * Q * step)
                            auto off = [&](int i) {
                                return (CHECK ? min(max(c0 + i, a_lo), a_hi - 1) : c0 + i) * qs32;
                            };
                            const bool ld = !CHECK || any;
                            const float2 z2 = make_float2(0.0f, 0.0f);
                            if (!full) {  // fixed-point running sums: an exact difference
                                const long long *__restrict__ pf_hi = pf + ntap;
#pragma unroll
                                for (int h = 0; h < CH; h += 4) {  // loads of 4 values, then their use
                                    long long lo[4], hi[4];
#pragma unroll
                                    for (int j = 0; j < 4; j++) {
                                        const int o = off(h + j);
                                        lo[j] = ld ? pf[o] : 0;
                                        hi[j] = ld ? pf_hi[o] : 0;
                                    }
#pragma unroll
                                    for (int j = 0; j < 4; j++)
                                        var_value(h + j, x[h + j], window_energy(lo[j], hi[j], unit));
                                }
                            } else {  // centred windows: double-float FP32 arithmetic
#pragma unroll
                                for (int h = 0; h < CH; h += 2) {
                                    long long lo2[2], hi2[2];
                                    float2 lo1[2], hi1[2];
#pragma unroll
                                    for (int j = 0; j < 2; j++) {
                                        const int o = off(h + j);
                                        lo2[j] = ld ? pf[o] : 0;
                                        hi2[j] = ld ? pf[o + ntap] : 0;
                                        lo1[j] = ld ? pg[o] : z2;
                                        hi1[j] = ld ? pg[o + ntap] : z2;
                                    }
#pragma unroll
                                    for (int j = 0; j < 2; j++) {
                                        float v, mean;
                                        window_centred(lo2[j], hi2[j], unit, lo1[j], hi1[j], nf, inv_n, v,
                                                       mean);
                                        var_value(h + j, fmaf(-mean, ts, x[h + j]), v);
                                    }
                                }
                            }
                        };
                        if (interior)
                            var_chunk(std::false_type{});
                        else
                            var_chunk(std::true_type{});
                    } else if (nsum && interior) {
                        // every output of the warp is valid: no per-value range test
                        if (first) {
#pragma unroll
                            for (int i = 0; i < CH; i++) {
                                const float num = full ? fmaf(-mm[i], ts, x[i]) : x[i];
                                const float den = sst * e[i];
                                const float cc = den > kThreshold ? num * rsqrtf(den) : 0.0f;
                                sv[i] = fmaf(cc, wc, 0.0f);
                            }
                        } else {
#pragma unroll
                            for (int i = 0; i < CH; i++) {
                                const float num = full ? fmaf(-mm[i], ts, x[i]) : x[i];
                                const float den = sst * e[i];
                                const float cc = den > kThreshold ? num * rsqrtf(den) : 0.0f;
                                sv[i] = fmaf(cc, wc, sv[i]);
                            }
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < CH; i++) {
                            const int a = c0 + i;
                            const float num = full ? fmaf(-mm[i], ts, x[i]) : x[i];
                            const float den = sst * e[i];
                            float cc = den > kThreshold ? num * rsqrtf(den) : 0.0f;
                            if (!(a >= a_lo && a < a_hi))
                                cc = 0.0f;
                            if (nsum)
                                sv[i] = fmaf(cc, wc, first ? 0.0f : sv[i]);
                            else if (a >= a_lo && a < a_hi)
                                oc[(size_t)a * TC_Q * SC] = cc;
                        }
                    }
                    if (nsum)
                        tmem_stc<CH>(s_cols + c0, sv);
                }
                if (nsum)
                    tmem_wait_st();
                first = false;
                c++;
            }
            if (nsum) {
                // a channel part writes its partial sums to its own plane of part_out
                float *o = (PARTS ? pr.part_out + (size_t)part * pr.P.T * n_corr : outp) +
                           (size_t)t * n_corr + kb + (long long)TC_Q * a0;
                const long long lim = n_corr - kb - (long long)TC_Q * a0;
#pragma unroll 1
                for (int c0 = 0; c0 < NC; c0 += CH) {
                    float sv[CH];
                    if (!first) {
                        tmem_ldc<CH>(s_cols + c0, sv);
                        tmem_wait_ld();
                    }
                    if constexpr (VAR && !PARTS) {  // the Fisher-z transform of every output, fused
                        const float zn = pr.P.vp_norm[t], zb = pr.P.vp_bias[t], zs = pr.P.vp_scale[t];
#pragma unroll
                        for (int i = 0; i < CH; i++) {
                            const int a = c0 + i;
                            const float x = (!first && a >= a_lo && a < a_hi) ? sv[i] : 0.0f;
                            if ((long long)a * TC_Q < lim)
                                o[(size_t)a * TC_Q] = (tanhf(x / zn) + zb) * zs;
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < CH; i++) {
                            const int a = c0 + i;
                            if ((long long)a * TC_Q < lim)
                                o[(size_t)a * TC_Q] = (!first && a >= a_lo && a < a_hi) ? sv[i] : 0.0f;
                        }
                    }
                }
            }
        }
    epilogue_done:;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

// Self-test of the bounded waits: one CTA waits on an mbarrier that nothing
// ever arrives on; the wait must give up after `limit_ns`, raise code 128 in
// the error word and return, leaving the context usable.
__global__ void wait_selftest_kernel(unsigned *err, unsigned long long limit_ns)
{
    __shared__ __align__(8) unsigned long long bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0)
        mbar_wait(smem_u32(&bar), 0, &abort_flag, err, 128u, limit_ns);
    __syncthreads();
}

int launch_wait_selftest(unsigned *err, unsigned ms, cudaStream_t s)
{
    wait_selftest_kernel<<<1, 32, 0, s>>>(err, (unsigned long long)ms * 1000000ull);
    count_launch();
    return check_launch("wait_selftest_kernel");
}

// ------------------------------------------------------------------ host side
struct TcShape {
    int k_span, R, NW;
    size_t stage;
};

static TcShape tc_shape(int L, int step, int split, int nb)
{
    TcShape g;
    const int lphi = (L + step - 1) / step;
    g.k_span = ((2 * TC_Q - 2 + lphi) + 15) & ~15;
    g.R = nb + (g.k_span - 1) / TC_Q + 1;
    g.NW = g.k_span / 8 + 16;
    g.stage = (size_t)(split ? 2 : 1) * ((size_t)TC_CB * g.R * 16 + (size_t)g.NW * 128);
    g.stage = (g.stage + 1023) & ~(size_t)1023;
    return g;
}

constexpr size_t TC_BAR_BYTES = 256;

// Largest tile (lag blocks per CTA tile) whose two pipeline stages fit in shared memory.
int tc_choose_nb(int L, int step, int split, int forced)
{
    const int cands[3] = {128, 64, 32};
    for (int i = 0; i < 3; i++) {
        if (forced && cands[i] != forced)
            continue;
        if (2 * tc_shape(L, step, split, cands[i]).stage + TC_BAR_BYTES <= 227 * 1024)
            return cands[i];
    }
    return 0;
}

// Preprocessing of one search for the tensor-core kernel: bf16 hi/lo data
// streams and template blocks, in scratch owned by `ws`.  Fills `out`.
int tc_prepare(const Problem &P, const float *data_for_tc, int split, int nb, int tg, Scratch &ws,
               cudaStream_t s, TcProb *out)
{
    int rc;
    const int step = P.step, L = P.L;
    const TcShape g = tc_shape(L, step, split, nb);
    TcProb pr;
    pr.P = P;
    pr.R = g.R;
    pr.NW = g.NW;
    pr.n_tiles = (int)((P.n_corr + (long long)TC_Q * nb - 1) / ((long long)TC_Q * nb));
    pr.tg = tg > 0 ? tg : TC_TG;
    pr.nb = nb;
    // Stream rows a tile can touch.  An item is processed only when its tile
    // holds a valid output k of its template, i.e. k*step + mo >= 0 and
    // k*step + mo + L <= N for every channel; hence its first row
    // r0 = (I0 + mu - s)/Q lies in [-(NB + 2), (N/step + 1)/Q + 1] whatever the
    // moveouts are, and rows [r0, r0 + R) stay inside the padded stream.
    pr.row_front = nb + 3;
    pr.rows_total = pr.row_front + (int)(((long long)P.N / step + 2) / TC_Q) + 2 + g.R + 1;
    pr.item_begin = 0;
    pr.parts = 1;
    pr.part_out = nullptr;

    const size_t g_elems = (size_t)P.SC * step * TC_CB * pr.rows_total * 8;
    const size_t w_elems = (size_t)P.T * P.SC * step * g.NW * 64;
    const size_t n_meta = (size_t)P.T * P.SC * step;
    uint16_t *g_hi = nullptr, *g_lo = nullptr, *w_hi = nullptr, *w_lo = nullptr;
    int *mu = nullptr, *psi = nullptr;
    if ((rc = ws.get(&g_hi, g_elems, "bf16 data streams")) ||
        (split && (rc = ws.get(&g_lo, g_elems, "bf16 data streams (lo)"))) ||
        (rc = ws.get(&w_hi, w_elems, "bf16 template blocks")) ||
        (split && (rc = ws.get(&w_lo, w_elems, "bf16 template blocks (lo)"))) ||
        (rc = ws.get(&mu, n_meta, "phase moveouts")) || (rc = ws.get(&psi, n_meta, "phase streams")))
        return rc;
    const long long n = (long long)P.SC * step * TC_CB * pr.rows_total;
    tc_data_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data_for_tc, P.N, P.SC, step, pr.rows_total,
                                                               pr.row_front, g_hi, g_lo);
    const long long m = (long long)P.T * P.SC * step * g.NW * 8;
    tc_template_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(P.tpl, P.mo, P.T, P.SC, L, step, g.NW,
                                                                   w_hi, w_lo, mu, psi);
    count_launch(2);
    if ((rc = check_launch("tensor-core preprocessing")))
        return rc;
    pr.g_hi = g_hi;
    pr.g_lo = g_lo;
    pr.w_hi = w_hi;
    pr.w_lo = w_lo;
    pr.mu = mu;
    pr.psi = psi;
    *out = pr;
    return FMF_OK;
}

static int n_sms()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        n = 148;
    cudaGetLastError();
    return n;
}

// out[i] = sum over parts j = 0..k-1 of part[j][i], in that order; with
// per-channel lengths (norm set) the Fisher-z transform of that sum,
// (tanh(v / norm[t]) + bias[t]) * scale[t] for row t = i / n_corr.
__global__ void tc_parts_sum_kernel(const float *__restrict__ part, int k, long long m, int n_corr,
                                    const float *__restrict__ norm, const float *__restrict__ bias,
                                    const float *__restrict__ scale, float *__restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    float v = part[i];
    for (int j = 1; j < k; j++)
        v += part[(size_t)j * m + i];
    if (norm) {
        const int t = (int)(i / n_corr);
        v = (tanhf(v / norm[t]) + bias[t]) * scale[t];
    }
    out[i] = v;
}

// Channel parts k (1..8, at most SC) for a search of `items` (tile, template)
// items: the k that minimises the busiest SM's work, ceil(k items / SMs)
// rounds of (1/k + 0.05) item each (0.05: an item's fixed pipeline fill and
// output write); FMF_TC_PARTS=k forces a value.
static int tc_choose_parts(long long items, int SC)
{
    const int sms = n_sms(), kmax = SC < 8 ? SC : 8;
    if (const char *env = getenv("FMF_TC_PARTS")) {
        const int k = atoi(env);
        if (k >= 1)
            return k < kmax ? k : kmax;
    }
    int best = 1;
    double best_cost = 1e300;
    for (int k = 1; k <= kmax; k++) {
        const long long rounds = (k * items + sms - 1) / sms;
        const double cost = (double)rounds * (1.0 / k + 0.05);
        if (cost < best_cost - 1e-9) {
            best_cost = cost;
            best = k;
        }
    }
    return best;
}

// One persistent launch over the tile queue of `n` prepared searches (n <= TC_MAX_PROBS).
// `queue` is a device counter that this call zeroes on `s` before the launch.
int tc_run(const TcProb *probs, int n, int split, unsigned long long *queue, unsigned *err, cudaStream_t s)
{
    if (n < 1 || n > TC_MAX_PROBS)
        return set_error(FMF_ERR_ARG, "a persistent launch takes 1..%d searches", TC_MAX_PROBS);
    static thread_local TcBatch Bh;  // large; built on the host for the launch only
    TcBatch &B = Bh;
    long long items = 0;
    size_t stage = 0;
    // A lone search with fewer (tile, template) items than SMs runs each item as k
    // channel parts (network sum only; with per-channel lengths the parts add raw
    // Fisher-z sums and the transform follows the addition), k chosen to shorten the
    // busiest SM's queue.  FMF_TC_PARTS=k overrides the choice where parts are allowed.
    const Problem &P0 = probs[0].P;
    const bool can_split = n == 1 && P0.network_sum && P0.SC >= 2;
    const int parts = can_split ? tc_choose_parts((long long)probs[0].n_tiles * P0.T, P0.SC) : 1;
    Scratch pws(s);
    float *part_out = nullptr;
    if (parts > 1) {
        int rc = pws.get(&part_out, (size_t)parts * P0.T * P0.n_corr, "channel-part sums");
        if (rc)
            return rc;
    }
    for (int i = 0; i < n; i++) {
        B.prob[i] = probs[i];
        B.prob[i].item_begin = items;
        B.prob[i].parts = parts;
        B.prob[i].part_out = part_out;
        items += (long long)probs[i].n_tiles * probs[i].P.T * parts;
        const size_t st = tc_shape(probs[i].P.L, probs[i].P.step, split, probs[i].nb).stage;
        stage = st > stage ? st : stage;
    }
    B.n_probs = n;
    B.split = split;
    B.stage_bytes = (int)stage;
    B.total_items = items;
    B.queue = queue;
    B.err = err;
    // more than half of the SM's shared memory: one CTA per SM, so that the
    // CTA's 512-column TMEM allocation never waits for another CTA
    size_t smem = 2 * stage + TC_BAR_BYTES;
    if (smem < 120 * 1024)
        smem = 120 * 1024;
    if (smem > 227 * 1024)
        return set_error(FMF_ERR_SMEM, "tensor-core stages need %zu bytes of shared memory", smem);
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "clearing the tile queue: %s", cudaGetErrorString(e));
    const unsigned grid = (unsigned)(items < n_sms() ? (items > 0 ? items : 1) : n_sms());
    int n_var = 0;
    for (int i = 0; i < n; i++)
        n_var += probs[i].P.ntap != nullptr;
    if (n_var != 0 && n_var != n)
        return set_error(FMF_ERR_ARG, "a persistent launch mixes per-channel and fixed template lengths");
    int n_full = 0;
    for (int i = 0; i < n; i++)
        n_full += probs[i].P.normalize != 0;
    const int norm = n_full == 0 ? 0 : (n_full == n ? 1 : -1);
    void (*kern)(const TcBatch);
    if (n_var && norm >= 0)  // per-channel lengths: always one search, one normalisation
        kern = parts > 1 ? (norm == 0 ? tc_persistent<true, true, 0> : tc_persistent<true, true, 1>)
                         : (norm == 0 ? tc_persistent<true, false, 0> : tc_persistent<true, false, 1>);
    else if (n_var)
        kern = parts > 1 ? tc_persistent<true, true, -1> : tc_persistent<true, false, -1>;
    else if (parts > 1)
        kern = norm == 0 ? tc_persistent<false, true, 0>
                         : (norm == 1 ? tc_persistent<false, true, 1> : tc_persistent<false, true, -1>);
    else
        kern = norm == 0 ? tc_persistent<false, false, 0>
                         : (norm == 1 ? tc_persistent<false, false, 1> : tc_persistent<false, false, -1>);
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynamicSmem);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "tc_persistent shared memory (%zu bytes): %s", smem,
                         cudaGetErrorString(e));
    kern<<<grid, tc_threads(n_var != 0), smem, s>>>(B);
    count_launch();
    int rc = check_launch("tc_persistent");
    if (rc || parts == 1)
        return rc;
    const long long m = (long long)P0.T * P0.n_corr;
    tc_parts_sum_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(part_out, parts, m, P0.n_corr,
                                                                     P0.ntap ? P0.vp_norm : nullptr,
                                                                     P0.vp_bias, P0.vp_scale, P0.out);
    count_launch();
    return check_launch("tc_parts_sum_kernel");
}

size_t tc_prob_size() { return sizeof(TcProb); }

// Templates [t0, t0 + nt) of a prepared search, as a search of its own
// (every template-indexed pointer offset; data streams shared).
void tc_subset(const TcProb *full, int t0, int nt, TcProb *out)
{
    TcProb q = *full;
    const size_t SC = q.P.SC, step = q.P.step;
    const size_t o = (size_t)t0 * SC;
    q.P.tpl += o * q.P.L;
    q.P.sst += o;
    if (q.P.tsum)
        q.P.tsum += o;
    q.P.mo += o;
    q.P.w += o;
    q.P.k_lo += t0;
    q.P.k_hi += t0;
    if (q.P.ntap)
        q.P.ntap += o;
    if (q.P.zweight)
        q.P.zweight += o;
    if (q.P.vp_norm) {
        q.P.vp_norm += t0;
        q.P.vp_bias += t0;
        q.P.vp_scale += t0;
    }
    q.P.out += (size_t)t0 * q.P.n_corr * (q.P.network_sum ? 1 : SC);
    q.P.T = nt;
    q.w_hi += o * step * q.NW * 64;
    if (q.w_lo)
        q.w_lo += o * step * q.NW * 64;
    q.mu += o * step;
    q.psi += o * step;
    *out = q;
}

// Single search: preprocessing + one persistent launch.
int launch_tc(const Problem &P, const float *data_for_tc, int precision, unsigned *err, Scratch &ws,
              cudaStream_t s, int forced_nb, int template_group)
{
    int rc;
    const int split = precision == FMF_PREC_SPLIT_BF16;
    const int nb = tc_choose_nb(P.L, P.step, split, forced_nb);
    if (nb == 0)
        return set_error(FMF_ERR_SMEM, "template length %d, step %d: tensor-core tile does not fit shared memory",
                         P.L, P.step);
    TcProb pr;
    if ((rc = tc_prepare(P, data_for_tc, split, nb, template_group, ws, s, &pr)))
        return rc;
    unsigned long long *queue = nullptr;
    if ((rc = ws.get(&queue, 1, "tile queue")))
        return rc;
    return tc_run(&pr, 1, split, queue, err, s);
}

}  // namespace fmf
