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
// CTA = one template x NB*Q consecutive outputs, all channels:
//   warp 0      producer: cp.async.bulk (TMA bulk copies) of the data rows and
//               the template blocks of one (channel, phase) stage, two stages
//               in flight, mbarrier complete_tx;
//   warp 1      allocates TMEM (two NB-column FP32 accumulators) and one
//               thread issues tcgen05.mma, tcgen05.commit to the barriers;
//   warps 4-11  epilogue: tcgen05.ld of the accumulator, normalisation by the
//               FP64 window statistics, threshold, weighted network sum in
//               registers (channel order, fused multiply-add), outputs.
// Every wait is bounded (globaltimer); on timeout the CTA raises an error
// word, stops issuing, waits for its own copies/MMAs (bounded) and frees TMEM.
#include <cuda_bf16.h>

#include "fmf_common.cuh"

namespace fmf {

constexpr int TC_Q = 128;
constexpr int TC_CB = TC_Q / 8;
constexpr int TC_THREADS = 384;
constexpr int TC_TG = 16;  // templates interleaved per group of CTAs (L2 reuse of data rows)
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // 2 s per wait

struct TcGeom {
    int NB;           // lag blocks per tile (MMA N)
    int R;            // data rows per stage
    int NW;           // 128-byte template blocks per (template, channel, phase)
    int k_span;       // largest K extent (multiple of 16)
    int rows_total;   // rows per (channel, stream) in G
    int row_front;    // rows of zero padding before sample 0
    int stage_bytes;  // bytes of one pipeline stage
    int split;        // 1: hi/lo, three products; 0: single bf16 product
    int n_tiles;
    size_t smem;
};

struct TcArgs {
    Problem P;
    const uint16_t *g_hi, *g_lo;  // bf16 bits, [SC][step][CB][rows_total][8]
    const uint16_t *w_hi, *w_lo;  // bf16 bits, [T][SC][step][NW][64]
    const int *mu;                // [T][SC][step] moveout of each phase in its stream
    const int *psi;               // [T][SC][step] stream of each phase
    unsigned *err;                // device error word
    TcGeom g;
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
// when this wait gave up (then it raises the error word and the abort flag).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                          unsigned *err, unsigned code)
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
            if (gtimer() - t0 > TC_WAIT_NS) {
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

// ------------------------------------------------------------------ main kernel
template <int NB>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_kernel(const TcArgs A)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const TcGeom &g = A.g;
    const Problem &P = A.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // tile and template of this CTA (templates interleaved in groups of TC_TG)
    const int per_group = g.n_tiles * TC_TG;
    const int grp = blockIdx.x / per_group;
    const int rem = blockIdx.x - grp * per_group;
    const int tg0 = grp * TC_TG;
    const int tgn = min(TC_TG, P.T - tg0);
    const int tile = rem / tgn;
    const int t = tg0 + rem % tgn;
    const long long I0 = (long long)tile * TC_Q * NB;
    const int klo = P.k_lo[t], khi = P.k_hi[t];
    const int SC = P.SC, step = P.step;
    const float *w = P.w + (size_t)t * SC;
    const int *mo = P.mo + (size_t)t * SC;

    if (!(I0 < khi && I0 + (long long)TC_Q * NB > klo)) {
        // no valid output in this tile: zeros (network sum); per-channel output is pre-cleared
        if (P.network_sum)
            for (int x = threadIdx.x; x < TC_Q * NB; x += TC_THREADS)
                if (I0 + x < P.n_corr)
                    P.out[(size_t)t * P.n_corr + I0 + x] = 0.0f;
        return;
    }

    uint8_t *bar_base = smem + 2 * g.stage_bytes;
    const uint32_t full0 = smem_u32(bar_base), empty0 = full0 + 16, dfull0 = full0 + 32,
                   dempty0 = full0 + 48, fin = full0 + 64;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bar_base + 80);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bar_base + 84);

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; i++) {
            mbar_init(full0 + 8 * i, 1);
            mbar_init(empty0 + 8 * i, 1);
            mbar_init(dfull0 + 8 * i, 1);
            mbar_init(dempty0 + 8 * i, 8);
        }
        mbar_init(fin, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    constexpr uint32_t TMEM_COLS = NB * 2 <= 32 ? 32 : (NB * 2 <= 64 ? 64 : (NB * 2 <= 128 ? 128 : 256));
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

    const int R = g.R, NW = g.NW;
    // stage layout: [data hi][data lo, split only][template hi][template lo, split only]
    const uint32_t data_bytes = (uint32_t)TC_CB * R * 16;  // one of hi/lo
    const uint32_t wbytes = (uint32_t)NW * 128;
    const uint32_t w_off = (g.split ? 2u : 1u) * data_bytes;

    if (warp == 0) {
        // ---------------------------------------------------------- producer
        int j = 0;
        for (int ch = 0; ch < SC; ch++) {
            if (w[ch] == 0.0f)
                continue;
            for (int phi = 0; phi < step; phi++, j++) {
                const int s = j & 1;
                if (j >= 2 &&
                    !mbar_wait_warp(empty0 + 8 * s, ((j >> 1) - 1) & 1, abort_flag, A.err, 2u))
                    goto producer_done;
                const long long meta = ((long long)t * SC + ch) * step + phi;
                const int mu = A.mu[meta], psi = A.psi[meta];
                const int sres = ((mu % TC_Q) + TC_Q) % TC_Q;
                const long long r0 = (I0 + mu - sres) / TC_Q + g.row_front;
                const uint32_t st = smem_u32(smem + (size_t)s * g.stage_bytes);
                if (lane == 0)
                    mbar_expect_tx(full0 + 8 * s, (g.split ? 2u : 1u) * (data_bytes + wbytes));
                __syncwarp();
                const int cb = lane & 15, hl = lane >> 4;
                if (hl == 0 || g.split) {
                    const uint16_t *src = (hl ? A.g_lo : A.g_hi) +
                                          ((((long long)ch * step + psi) * TC_CB + cb) * g.rows_total + r0) * 8;
                    bulk_g2s(st + hl * data_bytes + cb * (uint32_t)R * 16, src, (uint32_t)R * 16,
                             full0 + 8 * s);
                }
                if (lane < (g.split ? 2 : 1)) {
                    const uint16_t *src = (lane ? A.w_lo : A.w_hi) + meta * NW * 64;
                    bulk_g2s(st + w_off + lane * wbytes, src, wbytes, full0 + 8 * s);
                }
            }
        }
    producer_done:
        // wait (bounded) until the copies this warp issued have landed
        if (lane == 0)
            for (int k = max(0, j - 2); k < j; k++)
                mbar_wait(full0 + 8 * (k & 1), (k >> 1) & 1, abort_flag, A.err, 0u);
        __syncwarp();
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NB >> 3) << 17) |
                                   ((uint32_t)(TC_Q >> 4) << 24);
            const uint32_t lbo_b = (uint32_t)R * 16;
            int j = 0, c = 0;
            for (int ch = 0; ch < SC; ch++) {
                if (w[ch] == 0.0f)
                    continue;
                const int d = c & 1;
                if (c >= 2 && !mbar_wait(dempty0 + 8 * d, ((c >> 1) - 1) & 1, abort_flag, A.err, 4u))
                    goto mma_done;
                tc_fence_after();
                const uint32_t dt = tmem + (uint32_t)(d * NB);
                uint32_t acc = 0;
                for (int phi = 0; phi < step; phi++, j++) {
                    const int s = j & 1;
                    if (!mbar_wait(full0 + 8 * s, (j >> 1) & 1, abort_flag, A.err, 8u))
                        goto mma_done;
                    tc_fence_after();
                    const long long meta = ((long long)t * SC + ch) * step + phi;
                    const int mu = A.mu[meta];
                    const int sres = ((mu % TC_Q) + TC_Q) % TC_Q;
                    const int lphi = (P.L - phi + step - 1) / step;
                    const int k_first = sres & ~15;
                    const int k_end = (sres + lphi + TC_Q - 1 + 15) & ~15;
                    const uint32_t zhi = smem_u32(smem + (size_t)s * g.stage_bytes);
                    const uint32_t zlo = zhi + data_bytes, whi = zhi + w_off, wlo = whi + wbytes;
                    for (int k = k_first; k < k_end; k += 16) {
                        const uint32_t wo = (uint32_t)(k >> 3) * 128u;
                        const uint32_t bo = (uint32_t)((k & (TC_Q - 1)) >> 3) * lbo_b +
                                            (uint32_t)(k / TC_Q) * 16u;
                        const uint64_t ah = sdesc(whi + wo, 128, 128);
                        const uint64_t bh = sdesc(zhi + bo, lbo_b, 128);
                        mma_bf16(dt, ah, bh, idesc, acc);
                        acc = 1;
                        if (g.split) {
                            mma_bf16(dt, ah, sdesc(zlo + bo, lbo_b, 128), idesc, 1);
                            mma_bf16(dt, sdesc(wlo + wo, 128, 128), bh, idesc, 1);
                        }
                    }
                    mma_commit(empty0 + 8 * s);
                }
                mma_commit(dfull0 + 8 * d);
                c++;
            }
        mma_done:
            // all MMAs issued by this thread complete before TMEM is released
            mma_commit(fin);
            mbar_wait(fin, 0, abort_flag, A.err, 0u);
        }
        __syncwarp();
    } else if (warp >= 4) {
        // ---------------------------------------------------------- epilogue
        constexpr int NC = NB / 2;
        const int quarter = warp & 3;
        const int half = (warp - 4) >> 2;
        const int m = 32 * quarter + lane;  // accumulator row
        const int b = TC_Q - 1 - m;         // phase of that row
        const int a0 = half * NC;           // first lag block of this thread
        // valid lag blocks: klo <= I0 + Q*a + b < khi
        const long long kb = I0 + b;
        const int a_lo = (int)max(0LL, (klo - kb + TC_Q - 1) / TC_Q) - a0;
        const int a_hi = (int)min((long long)NB, (khi - kb + TC_Q - 1) / TC_Q) - a0;
        const long long qs = (long long)TC_Q * step;
        float S[NC];
#pragma unroll
        for (int i = 0; i < NC; i++)
            S[i] = 0.0f;
        int c = 0;
        for (int ch = 0; ch < SC; ch++) {
            const float wc = w[ch];
            if (wc == 0.0f)
                continue;
            const int d = c & 1;
            if (!mbar_wait_warp(dfull0 + 8 * d, (c >> 1) & 1, abort_flag, A.err, 16u))
                break;
            tc_fence_after();
            const size_t row = (size_t)t * SC + ch;
            const float sst = P.sst[row];
            const float ts = P.normalize ? P.tsum[row] : 0.0f;
            // statistics of the window of lag block a0 (advanced by qs per block)
            const long long u0 = (kb + (long long)TC_Q * a0) * step + mo[ch];
            const float *se = P.stat_e + (size_t)ch * P.N + u0;
            const float *sm = P.normalize ? P.stat_m + (size_t)ch * P.N + u0 : se;
            float *oc = P.out + ((size_t)t * P.n_corr + kb + (long long)TC_Q * a0) * SC + ch;
            const uint32_t tbase = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(d * NB + a0);
#pragma unroll
            for (int c0 = 0; c0 < NC; c0 += 16) {
                float x[16];
                tmem_ld16(tbase + c0, x);
                tmem_wait_ld();
                if (c0 + 16 >= NC) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0)
                        mbar_arrive(dempty0 + 8 * d);
                }
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int a = c0 + i;
                    if (a >= a_lo && a < a_hi) {
                        float num = x[i];
                        if (P.normalize)
                            num = fmaf(-sm[a * qs], ts, num);
                        const float den = sst * se[a * qs];
                        const float cc = den > kThreshold ? num / sqrtf(den) : 0.0f;
                        if (P.network_sum)
                            S[a] = fmaf(cc, wc, S[a]);
                        else
                            oc[(size_t)a * TC_Q * SC] = cc;
                    }
                }
            }
            c++;
        }
        if (P.network_sum) {
            float *o = P.out + (size_t)t * P.n_corr + kb + (long long)TC_Q * a0;
            const long long lim = P.n_corr - kb - (long long)TC_Q * a0;
#pragma unroll
            for (int a = 0; a < NC; a++)
                if ((long long)a * TC_Q < lim)
                    o[(size_t)a * TC_Q] = (a >= a_lo && a < a_hi) ? S[a] : 0.0f;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

// ------------------------------------------------------------------ host side
static int choose_nb(int L, int step, int split, int forced)
{
    const int cands[3] = {128, 64, 32};
    for (int i = 0; i < 3; i++) {
        int nb = cands[i];
        if (forced && nb != forced)
            continue;
        int lphi = (L + step - 1) / step;
        int k_span = ((2 * TC_Q - 2 + lphi) + 15) & ~15;
        int R = nb + (k_span - 1) / TC_Q + 1;
        int NW = k_span / 8 + 16;
        size_t stage = (size_t)(split ? 2 : 1) * ((size_t)TC_CB * R * 16 + (size_t)NW * 128);
        if (2 * stage + 128 <= 227 * 1024)
            return nb;
    }
    return 0;
}

int launch_tc(const Problem &P, const float *data_for_tc, int precision, unsigned *err, Scratch &ws,
              cudaStream_t s, int forced_nb)
{
    int rc;
    const int split = precision == FMF_PREC_SPLIT_BF16;
    const int step = P.step, L = P.L;
    const int NB = choose_nb(L, step, split, forced_nb);
    if (NB == 0)
        return set_error(FMF_ERR_SMEM, "template length %d, step %d: tensor-core tile does not fit shared memory",
                         L, step);
    TcGeom g;
    g.NB = NB;
    g.split = split;
    const int lphi = (L + step - 1) / step;
    g.k_span = ((2 * TC_Q - 2 + lphi) + 15) & ~15;
    g.R = NB + (g.k_span - 1) / TC_Q + 1;
    g.NW = g.k_span / 8 + 16;
    g.stage_bytes = (int)((size_t)(split ? 2 : 1) * ((size_t)TC_CB * g.R * 16 + (size_t)g.NW * 128));
    g.stage_bytes = (g.stage_bytes + 1023) & ~1023;
    g.smem = 2 * (size_t)g.stage_bytes + 128;
    g.n_tiles = (int)((P.n_corr + (long long)TC_Q * NB - 1) / ((long long)TC_Q * NB));
    // Stream rows a tile can touch.  A CTA runs only when its tile holds a
    // valid output k of its template, i.e. k*step + mo >= 0 and
    // k*step + mo + L <= N for every channel; hence its first row
    // r0 = (I0 + mu - s)/Q lies in [-(NB + 2), (N/step + 1)/Q + 1] whatever the
    // moveouts are, and rows [r0, r0 + R) stay inside the padded stream.
    g.row_front = NB + 3;
    g.rows_total = g.row_front + (int)(((long long)P.N / step + 2) / TC_Q) + 2 + g.R + 1;
    const size_t g_elems = (size_t)P.SC * step * TC_CB * g.rows_total * 8;
    const size_t w_elems = (size_t)P.T * P.SC * step * g.NW * 64;
    const size_t n_meta = (size_t)P.T * P.SC * step;
    uint16_t *g_hi, *g_lo = nullptr, *w_hi, *w_lo = nullptr;
    int *mu, *psi;
    if ((rc = ws.get(&g_hi, g_elems, "bf16 data streams")) ||
        (split && (rc = ws.get(&g_lo, g_elems, "bf16 data streams (lo)"))) ||
        (rc = ws.get(&w_hi, w_elems, "bf16 template blocks")) ||
        (split && (rc = ws.get(&w_lo, w_elems, "bf16 template blocks (lo)"))) ||
        (rc = ws.get(&mu, n_meta, "phase moveouts")) || (rc = ws.get(&psi, n_meta, "phase streams")))
        return rc;

    {
        long long n = (long long)P.SC * step * TC_CB * g.rows_total;
        tc_data_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(data_for_tc, P.N, P.SC, step,
                                                                   g.rows_total, g.row_front, g_hi, g_lo);
        long long m = (long long)P.T * P.SC * step * g.NW * 8;
        tc_template_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(P.tpl, P.mo, P.T, P.SC, L, step,
                                                                       g.NW, w_hi, w_lo, mu, psi);
        count_launch(2);
        if ((rc = check_launch("tensor-core preprocessing")))
            return rc;
    }

    TcArgs A;
    A.P = P;
    A.g_hi = g_hi;
    A.g_lo = g_lo;
    A.w_hi = w_hi;
    A.w_lo = w_lo;
    A.mu = mu;
    A.psi = psi;
    A.err = err;
    A.g = g;
    const long long ctas = (long long)g.n_tiles * P.T;
    if (ctas > 0x7fffffffLL)
        return set_error(FMF_ERR_ARG, "too many tiles for one launch");
    cudaError_t e;
    switch (NB) {
    case 128:
        e = cudaFuncSetAttribute(tc_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
        if (e == cudaSuccess)
            tc_kernel<128><<<(unsigned)ctas, TC_THREADS, g.smem, s>>>(A);
        break;
    case 64:
        e = cudaFuncSetAttribute(tc_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
        if (e == cudaSuccess)
            tc_kernel<64><<<(unsigned)ctas, TC_THREADS, g.smem, s>>>(A);
        break;
    default:
        e = cudaFuncSetAttribute(tc_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
        if (e == cudaSuccess)
            tc_kernel<32><<<(unsigned)ctas, TC_THREADS, g.smem, s>>>(A);
        break;
    }
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "tc_kernel shared memory (%zu bytes): %s", g.smem,
                         cudaGetErrorString(e));
    count_launch();
    return check_launch("tc_kernel");
}

}  // namespace fmf
