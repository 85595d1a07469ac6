// fmf_auto.cu -- the numerator precision FMF_PREC_AUTO chooses for a search.
//
// The split-bf16 tensor-core form (x = hi + lo, three bf16 products, FP32
// accumulation) is ~8x faster than the plain FP32 form, but each of its
// products t*d carries a relative error of 4.4e-6 RMS (2.7e-5 at most): a
// coefficient over L taps errs by about 4.4e-6 / sqrt(L) (measured on random
// operands, FP64 reference), and a template copied into the data at a
// power-of-two scale adds a bias of up to 2.8e-6 * |cc| (the dropped lo*lo
// products then all have one sign).  AUTO runs the split form when this
// model puts the largest error of the whole search at or below 1e-5 (relative
// to max(1, sum |w|) for network sums), and the plain FP32 form otherwise:
//
//   per channel   s_ch = 4.4e-6 * sqrt(D_ch / L_eff)
//   network sum   est  = 2.8e-6 * sum|w| + k * sqrt(sum_ch w^2 s_ch^2)
//   per channel   est  = 2.8e-6 + k * s_ch            (network_sum = 0)
//   k = sqrt(2 ln M) + 3 for M outputs (the Gaussian maximum, plus a margin
//   for the heavier tails of short sums: 8.4 standard deviations seen at L = 8)
//
// L_eff = (sum t^2)^2 / sum t^4 is the template channel's effective number of
// taps (its own length for per-channel lengths): at a match the error sums
// over the taps that carry the energy.  D_ch = 1 for 'short'; for 'full' the
// products are of the centred data d - c, whose window mean m adds to every
// product's size: D_ch = 1 + max over windows of L m^2 / V (V the window's
// centred energy), sampled every kAutoStride windows.
//
// Per-channel lengths sum atanh(cc_ch) * z_ch (z_ch = sqrt(n - 3) w_ch) and
// map the sum through tanh (matched_filter.c:596-601, 405-408): an error in
// cc_ch grows by 1 / (1 - cc_ch^2) there, so each channel's s_ch is scaled by
//   A_ch = max(M^(2 / (n - 1)), 1 / (1 - 0.9^2))
// -- the first the amplification at the largest |cc| that n-tap windows of
// noise reach among M channel windows (P(|cc| > c) ~ (1 - c^2)^((n-1)/2)),
// the second at a detection of |cc| = 0.9 -- and the estimate is
//   est = k * sqrt(sum_ch (z_ch A_ch s_ch)^2) / sum_ch |z_ch|
// (the tanh has slope at most 1; the output scale is the weight sum).
// Channels of 4 taps or fewer always run in FP32.  The bound holds while
// every channel's |cc| stays at or below max(0.9, the noise maximum).
#include <cmath>
#include <cstring>

#include "fmf_common.cuh"

namespace fmf {

constexpr float kSplitRms = 4.4e-6f;   // RMS relative error of one split-bf16 product
constexpr float kSplitBias = 2.8e-6f;  // bias per unit |cc| at a power-of-two copy
constexpr float kAutoTol = 1e-5f;
constexpr int kAutoStride = 7;
constexpr float kFisherAmp = 1.0f / (1.0f - 0.9f * 0.9f);  // 1 / (1 - cc^2) at |cc| = 0.9

// grid = SC, 256 threads: D_ch - 1 of 'full' from the (centred energy, mean)
// window statistics of the fixed-length path.
__global__ void auto_dc_stats_kernel(const float2 *__restrict__ stat, int N, int nwin, int L,
                                     float *__restrict__ dc)
{
    __shared__ float red[8];
    const float2 *row = stat + (size_t)blockIdx.x * N;
    float mx = 0.0f;
    for (int u = threadIdx.x * kAutoStride; u < nwin; u += blockDim.x * kAutoStride) {
        const float2 vm = row[u];
        if (vm.x > 0.0f)
            mx = fmaxf(mx, (float)L * vm.y * vm.y / vm.x);
    }
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++)
            mx = fmaxf(mx, red[i]);
        dc[blockIdx.x] = mx;
    }
}

// The same from the running sums of the per-channel-length path, for windows
// of the longest length L.
__global__ void auto_dc_prefix_kernel(const long long *__restrict__ pre2q,
                                      const float *__restrict__ unit2,
                                      const float2 *__restrict__ pre1f, int N, int L,
                                      float *__restrict__ dc)
{
    __shared__ float red[8];
    const int ch = blockIdx.x;
    const long long *p2 = pre2q + (size_t)ch * (N + 1);
    const float2 *p1 = pre1f + (size_t)ch * (N + 1);
    const float q = unit2[ch], nf = (float)L, inv_n = 1.0f / nf;
    float mx = 0.0f;
    for (int u = threadIdx.x * kAutoStride; u + L <= N; u += blockDim.x * kAutoStride) {
        float v, mean;
        window_centred(p2[u], p2[u + L], q, p1[u], p1[u + L], nf, inv_n, v, mean);
        if (v > 0.0f)
            mx = fmaxf(mx, nf * mean * mean / v);
    }
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++)
            mx = fmaxf(mx, red[i]);
        dc[ch] = mx;
    }
}

// grid = T, 256 threads (8 warps, one channel per warp at a time): the
// estimate of template t divided by its bar, as float bits into *worst
// (atomicMax: the ratios are non-negative).  ntap non-null: the Fisher-z
// network sum of per-channel lengths, ln_m = ln(channel windows).
__global__ void auto_template_kernel(const float *__restrict__ tpl, const float *__restrict__ w,
                                     const int *__restrict__ ntap, int SC, int L,
                                     const float *__restrict__ dc, int network_sum, float k,
                                     float ln_m, unsigned *__restrict__ worst)
{
    __shared__ float sw[8], sv[8], smax[8];
    const int t = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float sum_w = 0.0f, var = 0.0f, ch_max = 0.0f;
    for (int ch = warp; ch < SC; ch += 8) {
        const size_t row = (size_t)t * SC + ch;
        const float wc = w[row];
        if (wc == 0.0f)
            continue;
        const int n = ntap ? ntap[row] : L;
        const float *x = tpl + row * L;
        float s2 = 0.0f, s4 = 0.0f;
        for (int j = lane; j < n; j += 32) {
            const float v = x[j] * x[j];
            s2 += v;
            s4 += v * v;
        }
        for (int o = 16; o > 0; o >>= 1) {
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            s4 += __shfl_xor_sync(0xffffffffu, s4, o);
        }
        if (lane == 0 && ntap && n <= 4) {
            ch_max = INFINITY;  // Fisher z of a few taps: FP32
        } else if (lane == 0 && s4 > 0.0f) {
            const float leff = s2 * s2 / s4;
            const float d = 1.0f + (dc ? dc[ch] : 0.0f);
            const float s = kSplitRms * sqrtf(d / leff);  // per-channel standard deviation
            if (ntap) {  // Fisher z: weight z = sqrt(n - 3) w, amplification A
                const float z = sqrtf((float)(n - 3)) * wc;
                const float amp = fmaxf(expf(2.0f * ln_m / (float)(n - 1)), kFisherAmp);
                sum_w += fabsf(z);
                var += (z * amp * s) * (z * amp * s);
            } else {
                sum_w += fabsf(wc);
                var += wc * wc * s * s;
                ch_max = fmaxf(ch_max, (kSplitBias + k * s) / kAutoTol);
            }
        }
    }
    if (lane == 0) {
        sw[warp] = sum_w;
        sv[warp] = var;
        smax[warp] = ch_max;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float W = 0.0f, V = 0.0f, M = 0.0f;
        for (int i = 0; i < 8; i++) {
            W += sw[i];
            V += sv[i];
            M = fmaxf(M, smax[i]);
        }
        float ratio = M;
        if (ntap)
            ratio = M > 0.0f ? M : (W > 0.0f ? k * sqrtf(V) / (kAutoTol * W) : 0.0f);
        else if (network_sum)
            ratio = (kSplitBias * W + k * sqrtf(V)) / (kAutoTol * fmaxf(1.0f, W));
        atomicMax(worst, __float_as_uint(ratio));
    }
}

int choose_auto_precision(const Problem &P, Scratch &ws, cudaStream_t s, int *precision)
{
    int rc;
    unsigned *worst = nullptr;
    float *dc = nullptr;
    if ((rc = ws.get(&worst, 1, "precision estimate")))
        return rc;
    cudaError_t e = cudaMemsetAsync(worst, 0, sizeof(unsigned), s);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "precision estimate: %s", cudaGetErrorString(e));
    if (P.normalize == 1) {
        if ((rc = ws.get(&dc, (size_t)P.SC, "precision estimate")))
            return rc;
        if (P.pre2q)
            auto_dc_prefix_kernel<<<P.SC, 256, 0, s>>>(P.pre2q, P.unit2, P.pre1f, P.N, P.L, dc);
        else
            auto_dc_stats_kernel<<<P.SC, 256, 0, s>>>(reinterpret_cast<const float2 *>(P.stat_e), P.N,
                                                      P.N - P.L + 1, P.L, dc);
        count_launch();
    }
    const double outputs = (double)P.T * P.n_corr * (P.network_sum ? 1 : P.SC);
    const float k = (float)(std::sqrt(2.0 * std::log(outputs > 2.0 ? outputs : 2.0)) + 3.0);
    const double windows = (double)P.T * P.n_corr * P.SC;
    const float ln_m = (float)std::log(windows > 2.0 ? windows : 2.0);
    for (int t0 = 0; t0 < P.T; t0 += 65535) {
        const int nt = P.T - t0 < 65535 ? P.T - t0 : 65535;
        const size_t o = (size_t)t0 * P.SC;
        auto_template_kernel<<<nt, 256, 0, s>>>(P.tpl + o * P.L, P.w + o, P.ntap ? P.ntap + o : nullptr,
                                                P.SC, P.L, dc, P.network_sum, k, ln_m, worst);
        count_launch();
    }
    unsigned bits = 0;
    if ((rc = check_launch("precision estimate")))
        return rc;
    if ((e = cudaMemcpyAsync(&bits, worst, sizeof(bits), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "precision estimate: %s", cudaGetErrorString(e));
    float ratio;
    memcpy(&ratio, &bits, sizeof(ratio));
    *precision = ratio <= 1.0f ? FMF_PREC_SPLIT_BF16 : FMF_PREC_FP32;
    return FMF_OK;
}

}  // namespace fmf
