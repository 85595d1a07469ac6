// fmf_plain.cu -- plain FP32 CUDA-core matched filter (drop-in form).
//
// Replaces the reference kernels network_corr + sum_cc
// (matched_filter.cu:42-168) and the per-lag loop of the CPU library
// (matched_filter.c:78-92, 416-455, 611-657).
//
// One CTA = one template x one tile of 4096 consecutive output indices (CTAs
// ordered template-fastest); it
// walks the template's channels in station-major / component-minor order,
// skipping channels of weight 0, and keeps the weighted network sum of its
// 4096 outputs on chip for the whole walk.  Each thread owns 16 consecutive
// outputs.
//
// step > 1 is handled polyphase: taps j = step*q + phi see the data stream
// d[step*(k + q) + mo + phi], so every phase phi is a unit-step correlation of
// ceil((L - phi)/step) taps against a decimated data window.  Per (channel,
// phase) one *stage* is staged in shared memory with cp.async (zero-filled
// outside [0, N)): the decimated data window (4096 + taps samples, stored with
// 4 padding floats every 16: the 16-byte load of lane l then falls in bank
// group 5*l mod 8 whatever the tap offset, so the 8 lanes of each quarter-warp
// access hit distinct banks) and the phase's template taps.
// Two stage buffers are in flight.
//
// Inner loop: a 20-register sliding window of data per thread; per 4 taps one
// 16-byte data load, one 16-byte broadcast template load and 64 FMAs.  Taps
// run in blocks of 80 (a multiple of the 16-float padding period), so every
// shared-memory offset inside a block is a compile-time constant and the loop
// issues almost nothing but loads and FMAs.
//
// Epilogue per channel (fused): numerator of "full" minus m*sum(t'),
// den = sst * E (E and m from the double-float window statistics), threshold 1e-6 on
// den, cc = num / sqrt(den), network sum acc = fma(cc, w, acc) in channel
// order (the reference's accumulation, matched_filter.c:450).  Outputs
// outside [k_lo, k_hi) are written as 0.
#include <cfloat>

#include "fmf_common.cuh"

namespace fmf {

constexpr int PL_THREADS = 256;
constexpr int PL_R = 16;                       // outputs per thread
constexpr int PL_TILE = PL_THREADS * PL_R;     // outputs per CTA
constexpr int PL_U = 20;                       // taps per unrolled iteration

__host__ __device__ __forceinline__ int padx(int x) { return x + ((x >> 4) << 2); }

struct PlainGeom {
    int lq_pad;       // taps per phase, padded to a multiple of PL_U
    int dw;           // data window length (logical floats)
    int data_floats;  // padded data floats
    int stat_off;     // offset of the staged window energies ('short', fixed lengths), else 0
    int stage_floats; // data + template (+ energies) floats, multiple of 4
    size_t smem;      // dynamic shared memory bytes
};

// stage_energies: 'short' with fixed template lengths also stages the tile's
// window energies (padded like the data, so that 16-byte reads of threads 16
// outputs apart hit distinct banks)
inline PlainGeom plain_geom(int L, int step, bool stage_energies)
{
    PlainGeom g;
    int lq = (L + step - 1) / step;
    g.lq_pad = (lq + PL_U - 1) / PL_U * PL_U;
    g.dw = PL_TILE + g.lq_pad;
    g.data_floats = padx(g.dw) + 4;
    g.stat_off = 0;
    g.stage_floats = (g.data_floats + g.lq_pad + 3) & ~3;
    g.smem = (size_t)(2 * g.stage_floats + PL_R * PL_THREADS) * sizeof(float);
    // only while two CTAs still share an SM (228 KB, 1 KB reserved per CTA)
    const int staged = g.stage_floats + ((padx(PL_TILE) + 3) & ~3);
    const size_t smem_staged = (size_t)(2 * staged + PL_R * PL_THREADS) * sizeof(float);
    if (stage_energies && 2 * (smem_staged + 1024) <= 228 * 1024) {
        g.stat_off = g.stage_floats;
        g.stage_floats = staged;
        g.smem = smem_staged;
    }
    return g;
}

__device__ __forceinline__ void cp_async4(float *smem, const float *gmem, bool valid)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    int n = valid ? 4 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(n)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

__device__ __forceinline__ int next_active(const float *w, int ch, int SC)
{
    while (ch < SC && w[ch] == 0.0f)
        ch++;
    return ch;
}

__device__ __forceinline__ void load_stage(float *buf, const Problem &P, const PlainGeom &g,
                                           int t, int ch, int phi, long long k0, int mo)
{
    const float *dch = P.data + (size_t)ch * P.N;
    const long long base = (long long)P.step * k0 + mo + phi;
    for (int x = threadIdx.x; x < g.dw; x += PL_THREADS) {
        long long src = base + (long long)P.step * x;
        bool ok = src >= 0 && src < P.N;
        cp_async4(buf + padx(x), ok ? dch + src : dch, ok);
    }
    float *tb = buf + g.data_floats;
    const float *tc = P.tpl + ((size_t)t * P.SC + ch) * P.L;
    for (int q = threadIdx.x; q < g.lq_pad; q += PL_THREADS) {
        int j = P.step * q + phi;
        bool ok = j < P.L;
        cp_async4(tb + q, ok ? tc + j : tc, ok);
    }
    if (g.stat_off && phi == P.step - 1) {
        // the window energies of the tile's valid outputs (its epilogue follows this
        // phase); the others are zero-filled and never used
        float *sb = buf + g.stat_off;
        const float *se = P.stat_e + (size_t)ch * P.N;
        const int klo = P.k_lo[t], khi = P.k_hi[t];
        for (int x = threadIdx.x; x < PL_TILE; x += PL_THREADS) {
            const long long k = k0 + x;
            const bool ok = k >= klo && k < khi;
            cp_async4(sb + padx(x), ok ? se + (k * P.step + mo) : se, ok);
        }
    }
}

// PL_U taps of one thread: data window advanced in place (ring of PL_U
// registers), template taps broadcast.  `d` points at data offset q of the
// thread's window, `tq` at template tap q; PADY(y) is the padded offset of
// data index q + y (q a multiple of 16, so it is a compile-time constant).
#define PL_TAPS_BODY(d, tq, PADY)                                                              \
    _Pragma("unroll") for (int s = 0; s < 5; s++)                                              \
    {                                                                                          \
        float4 v = *reinterpret_cast<const float4 *>((d) + PADY(16 + 4 * s));                  \
        win[(16 + 4 * s + 0) % PL_U] = v.x;                                                    \
        win[(16 + 4 * s + 1) % PL_U] = v.y;                                                    \
        win[(16 + 4 * s + 2) % PL_U] = v.z;                                                    \
        win[(16 + 4 * s + 3) % PL_U] = v.w;                                                    \
        float4 tv4 = *reinterpret_cast<const float4 *>((tq) + 4 * s);                          \
        float tv[4] = {tv4.x, tv4.y, tv4.z, tv4.w};                                            \
        _Pragma("unroll") for (int jj = 0; jj < 4; jj++)                                       \
            _Pragma("unroll") for (int r = 0; r < PL_R; r++)                                   \
                acc[r] = fmaf(tv[jj], win[(4 * s + r + jj) % PL_U], acc[r]);                   \
    }

// Taps [0, taps) of one phase (taps a multiple of PL_U, at most g.lq_pad).
__device__ __forceinline__ void compute_phase(const float *buf, const PlainGeom &g, int taps,
                                              float acc[PL_R])
{
    const float *tb = buf + g.data_floats;
    const int x0 = threadIdx.x * PL_R;  // a multiple of 16: padx(x0 + y) = padx(x0) + padx(y)
    const float *db = buf + padx(x0);
    float win[PL_U];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float4 v = *reinterpret_cast<const float4 *>(db + padx(4 * i));
        win[4 * i + 0] = v.x;
        win[4 * i + 1] = v.y;
        win[4 * i + 2] = v.z;
        win[4 * i + 3] = v.w;
    }
    int q = 0;
    // blocks of 80 taps (a multiple of 16 and of PL_U): every padded offset is a constant
    for (; q + 4 * PL_U <= taps; q += 4 * PL_U) {
        const float *d = db + padx(q);
        const float *tq = tb + q;
#pragma unroll
        for (int it = 0; it < 4; it++) {
#define PL_PADY(y) padx(it * PL_U + (y))
            PL_TAPS_BODY(d, tq + it * PL_U, PL_PADY)
#undef PL_PADY
        }
    }
    // the remaining taps, PL_U at a time
    for (; q < taps; q += PL_U) {
#define PL_PADQ(y) (padx(q + (y)) - padx(q))
        const float *d = db + padx(q);
        PL_TAPS_BODY(d, tb + q, PL_PADQ)
#undef PL_PADQ
    }
}

// FULL: 'full' normalisation; VAR: per-channel template lengths (Problem::ntap)
// -- one instantiation per mode, so that each keeps only its own epilogue code.
template <bool FULL, bool VAR>
__global__ void __launch_bounds__(PL_THREADS, 2)
plain_kernel(const Problem P, const PlainGeom g)
{
    extern __shared__ __align__(16) float smem[];
    float *net = smem + 2 * g.stage_floats;  // [PL_R][PL_THREADS]

    // templates fastest: the CTAs running at any time share a few tiles, so
    // their data windows and window statistics are read from L2
    const int t = (int)(blockIdx.x % (unsigned)P.T);
    const int k0 = (int)(blockIdx.x / (unsigned)P.T) * PL_TILE;  // < n_corr <= INT_MAX
    const int klo = P.k_lo[t], khi = P.k_hi[t];
    const int tid = threadIdx.x;
    const float *w = P.w + (size_t)t * P.SC;
    const int *mo = P.mo + (size_t)t * P.SC;

#pragma unroll
    for (int r = 0; r < PL_R; r++)
        net[r * PL_THREADS + tid] = 0.0f;

    const bool busy = k0 < khi && k0 + PL_TILE > klo;
    if (busy) {
        float acc[PL_R];
#pragma unroll
        for (int r = 0; r < PL_R; r++)
            acc[r] = 0.0f;
        int ch = next_active(w, 0, P.SC), phi = 0, b = 0;
        if (ch < P.SC)
            load_stage(smem, P, g, t, ch, 0, k0, mo[ch]);
        cp_async_commit();
        while (ch < P.SC) {
            int nch = ch, nphi = phi + 1;
            if (nphi == P.step) {
                nphi = 0;
                nch = next_active(w, ch + 1, P.SC);
            }
            if (nch < P.SC)
                load_stage(smem + (b ^ 1) * g.stage_floats, P, g, t, nch, nphi, k0, mo[nch]);
            cp_async_commit();
            cp_async_wait1();
            __syncthreads();
            // per-channel template lengths: the taps past the channel's own length are
            // zeros, so the phase stops after its own taps (rounded up to PL_U)
            int taps = g.lq_pad;
            if constexpr (VAR) {
                const int n = P.ntap[(size_t)t * P.SC + ch];
                const int own = n > phi ? (n - phi + P.step - 1) / P.step : 0;
                taps = min(g.lq_pad, (own + PL_U - 1) / PL_U * PL_U);
            }
            compute_phase(smem + b * g.stage_floats, g, taps, acc);
            if (VAR && phi == P.step - 1) {
                // per-channel template length: window sums of that length from the
                // running sums (d^2 in exact fixed point, d as float pairs),
                // the 'precise' threshold (on the square root, matched_filter.c:650-652)
                // and a Fisher-z network sum (matched_filter.c:596-601)
                const size_t row = (size_t)t * P.SC + ch;
                const float sst = P.sst[row], zw = P.zweight[row];
                const float ts = FULL ? P.tsum[row] : 0.0f;
                const int n = P.ntap[row];
                const float nf = (float)n, inv_n = 1.0f / nf;
                const long long *p2 = P.pre2q + (size_t)ch * (P.N + 1);
                const float unit = P.unit2[ch];
                const float2 *p1 = FULL ? P.pre1f + (size_t)ch * (P.N + 1) : nullptr;
#pragma unroll
                for (int r = 0; r < PL_R; r++) {
                    const int k = k0 + tid * PL_R + r;
                    if (k >= klo && k < khi) {
                        const int u = k * P.step + mo[ch];  // a window inside [0, N - n]
                        float num = acc[r], ssd;
                        if (FULL) {
                            float mean;
                            window_centred(p2[u], p2[u + n], unit, p1[u], p1[u + n], nf, inv_n, ssd,
                                           mean);
                            num = fmaf(-mean, ts, num);
                        } else {
                            ssd = window_energy(p2[u], p2[u + n], unit);
                        }
                        const float den = sqrtf(sst * ssd);
                        const float cc = den > kThreshold ? num / den : 0.0f;
                        net[r * PL_THREADS + tid] =
                            fmaf(atanhf(cc - 10.0f * FLT_EPSILON), zw, net[r * PL_THREADS + tid]);
                    }
                    acc[r] = 0.0f;
                }
            } else if (phi == P.step - 1) {
                // fused epilogue of channel ch
                const size_t row = (size_t)t * P.SC + ch;
                const float sst = P.sst[row], wc = w[ch];
                const float ts = FULL ? P.tsum[row] : 0.0f;
                const float *se = P.stat_e + (size_t)ch * P.N;
                const float2 *sem = reinterpret_cast<const float2 *>(P.stat_e) + (size_t)ch * P.N;
                float staged[PL_R];  // 'short': this thread's energies from the stage, if staged
                if (!FULL && g.stat_off) {
                    const float *sb = smem + b * g.stage_floats + g.stat_off + padx(tid * PL_R);
#pragma unroll
                    for (int i = 0; i < PL_R; i += 4) {
                        const float4 v = *reinterpret_cast<const float4 *>(sb + i);
                        staged[i] = v.x;
                        staged[i + 1] = v.y;
                        staged[i + 2] = v.z;
                        staged[i + 3] = v.w;
                    }
                }
#pragma unroll
                for (int r = 0; r < PL_R; r++) {
                    const int k = k0 + tid * PL_R + r;
                    if (k >= klo && k < khi) {
                        const int u = k * P.step + mo[ch];  // a window inside [0, N - L]
                        float num = acc[r], energy;
                        if (FULL) {  // (centred energy, mean) pairs
                            const float2 em = sem[u];
                            num = fmaf(-em.y, ts, num);
                            energy = em.x;
                        } else {
                            energy = g.stat_off ? staged[r] : se[u];
                        }
                        float den = sst * energy;
                        float cc = den > kThreshold ? num * rsqrtf(den) : 0.0f;
                        if (P.network_sum)
                            net[r * PL_THREADS + tid] = fmaf(cc, wc, net[r * PL_THREADS + tid]);
                        else
                            P.out[((size_t)t * P.n_corr + k) * P.SC + ch] = cc;
                    }
                    acc[r] = 0.0f;
                }
            }
            __syncthreads();
            b ^= 1;
            ch = nch;
            phi = nphi;
        }
    }
    if (P.network_sum) {
        float *o = P.out + (size_t)t * P.n_corr;
#pragma unroll
        for (int r = 0; r < PL_R; r++) {
            const int k = k0 + tid * PL_R + r;
            if (k < P.n_corr)
                o[k] = net[r * PL_THREADS + tid];
        }
    }
}

// Host launcher.  Returns FMF status.
int launch_plain(const Problem &P, cudaStream_t stream)
{
    PlainGeom g = plain_geom(P.L, P.step, !P.ntap && !P.normalize);
    if (g.smem > 227 * 1024)
        return set_error(FMF_ERR_SMEM,
                         "template length %d with step %d needs %zu bytes of shared memory (max 232448)",
                         P.L, P.step, g.smem);
    void (*kern)(const Problem, const PlainGeom) =
        P.ntap ? (P.normalize ? plain_kernel<true, true> : plain_kernel<false, true>)
               : (P.normalize ? plain_kernel<true, false> : plain_kernel<false, false>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynamicSmem);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "plain kernel shared memory (%zu bytes): %s", g.smem,
                         cudaGetErrorString(e));
    const long long n_tiles = (P.n_corr + PL_TILE - 1) / PL_TILE;
    if (n_tiles * P.T > 0x7fffffffLL)
        return set_error(FMF_ERR_ARG, "too many (template, tile) pairs for one launch");
    kern<<<(unsigned)(n_tiles * P.T), PL_THREADS, g.smem, stream>>>(P, g);
    count_launch();
    return check_launch("plain_kernel");
}

}  // namespace fmf
