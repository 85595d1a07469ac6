// fmf_noalloc.cu -- the allocation-free entry point fmf_matched_filter_noalloc.
//
// Who needs it: callers that must not allocate device memory once they are
// running.  A real-time detection loop that reserved its memory at start-up
// cannot afford cudaMalloc/cudaFree in its processing path (both can
// synchronise the device and take unbounded time), and a host application
// that owns the GPU's memory budget -- it reserves nearly all device memory
// up front for its own pool, or runs under a fixed per-process memory cap --
// would see this library's own allocations fail or fragment its pool.  The
// regular entry points allocate their working arrays per call from the
// device's stream-ordered pool; this one does not allocate at all.
//
// What it does: the plain FP32 form (the same kernels as fmf_matched_filter),
// with every working array (per-template lag ranges, window statistics, the
// template energies when the caller passes none, and for 'full' the centred
// data and templates) carved out of ONE file-scope device array of
// FMF_NOALLOC_SCRATCH_BYTES bytes.  That array belongs to the
// module, so every GPU that loads this library holds it until the process
// exits.  Inputs and outputs are the caller's device pointers.
//
// Rules the caller must know:
//  * The array's device address is looked up once per device, with that
//    device current, by the first call on that device (cudaGetSymbolAddress);
//    make that first call before any stream capture.
//  * Every call uses the same array.  Calls that overlap on the GPU (on two
//    streams, or from two threads, without ordering between them) race on it
//    and corrupt each other's results: serialise them.  Nothing read from the
//    array is assumed to start at zero -- each call writes every element it
//    later reads -- so the previous call's leftovers do no harm.
//  * Searches that need more scratch than the array holds, and device arrays
//    that are not 4-byte aligned, are rejected with FMF_ERR_ARG before any
//    work is queued.
#include <cstdio>
#include <mutex>

#include "fmf_common.cuh"

namespace fmf {

__global__ void template_range_kernel(const int *, int, int, int, int, int, int, int *, int *);
__global__ void template_energy_kernel(const float *, int, int, float *);
__global__ void template_center_kernel(const float *, int, float *, float *);
__global__ void channel_centre_kernel(const float *, int, float *);

// The only working memory of fmf_matched_filter_noalloc.  In host code this
// name is a host-side stand-in, not a device address: host code uses the
// address returned by cudaGetSymbolAddress (scratch_base below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[FMF_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kNoallocDevices = 64;
unsigned char *g_scratch_base[kNoallocDevices];
std::mutex g_scratch_mutex;

// Device address of g_noalloc_scratch on the current device, looked up once.
int scratch_base(unsigned char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "noalloc: no current device: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoallocDevices)
        return set_error(FMF_ERR_UNSUPPORTED, "noalloc: device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_base[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return set_error(FMF_ERR_CUDA, "noalloc: cudaGetSymbolAddress failed: %s",
                             cudaGetErrorString(e));
        g_scratch_base[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_base[dev];
    return FMF_OK;
}

// Sequential 256-byte-aligned carving of the scratch array.
struct Carve {
    unsigned char *base;
    size_t used = 0;
    template <class T>
    T *take(size_t count)
    {
        T *p = reinterpret_cast<T *>(base + used);
        used += (count * sizeof(T) + 255) & ~size_t(255);
        return p;
    }
};

// Bytes of the carve of fmf_matched_filter_noalloc, or SIZE_MAX when the
// search cannot fit (so that no product below can wrap): lag ranges, window
// statistics ('full': (energy, mean) pairs), the template energies when the
// caller passes none, then for 'full' the centred data, channel centres,
// centred templates and their sums.
size_t scratch_bytes(size_t T, size_t SC, size_t L, size_t N, bool full, bool energies)
{
    const size_t cap = FMF_NOALLOC_SCRATCH_BYTES;
    // every factor pair below is bounded before it is multiplied: each part
    // must fit the array on its own
    if (T > cap / 8 || SC > cap / 4 || N > cap / 4 || L > cap / 4 || SC > cap / 4 / N ||
        T > cap / 4 / SC || T * SC > cap / 4 / (L + 1))
        return SIZE_MAX;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t b = al(2 * T * sizeof(int)) + al(SC * N * sizeof(float) * (full ? 2 : 1));
    if (energies)
        b += al(T * SC * sizeof(float));
    if (full)
        b += al(SC * N * sizeof(float)) + al(SC * sizeof(float)) + al(T * SC * L * sizeof(float)) +
             al(T * SC * sizeof(float));
    return b;
}

}  // namespace
}  // namespace fmf

extern "C" int fmf_matched_filter_noalloc(const float *templates, const float *sum_square_templates,
                                          const int *moveouts, const float *data,
                                          const float *weights, size_t step,
                                          size_t n_samples_template, size_t n_samples_data,
                                          size_t n_templates, size_t n_stations,
                                          size_t n_components, size_t n_corr, float *cc_out,
                                          int normalize, int sum_cc_mode, void *stream)
{
    using namespace fmf;
    set_error(FMF_OK, "");
    reset_launch_count();
    if (!templates || !moveouts || !data || !weights || !cc_out)
        return set_error(FMF_ERR_ARG, "noalloc: null array argument");
    {  // the kernels load these in place as 4-byte elements
        const void *ptrs[6] = {templates, sum_square_templates, moveouts, data, weights, cc_out};
        for (const void *p : ptrs)
            if ((uintptr_t)p & 3)
                return set_error(FMF_ERR_ARG, "noalloc: device array %p is not 4-byte aligned", p);
    }
    if (step < 1 || n_samples_template < 1 || n_templates < 1 || n_stations < 1 ||
        n_components < 1 || n_corr < 1 || n_samples_data < n_samples_template)
        return set_error(FMF_ERR_ARG, "noalloc: invalid sizes");
    if (normalize != 0 && normalize != 1)
        return set_error(FMF_ERR_ARG, "noalloc: normalize must be 0 or 1");
    if (n_stations > (size_t)INT_MAX || n_components > (size_t)INT_MAX)
        return set_error(FMF_ERR_ARG, "noalloc: sizes out of range");
    const size_t SCz = n_stations * n_components;
    if (n_samples_data > (size_t)INT_MAX / 2 || n_corr > (size_t)INT_MAX || SCz > (size_t)INT_MAX ||
        n_templates > (size_t)INT_MAX || step > (size_t)INT_MAX / 2 ||
        n_corr > (n_samples_data - n_samples_template) / step + 1)
        return set_error(FMF_ERR_ARG, "noalloc: sizes out of range");
    const bool full = normalize == 1;
    const bool energies = sum_square_templates == nullptr;
    const size_t need =
        scratch_bytes(n_templates, SCz, n_samples_template, n_samples_data, full, energies);
    if (need > (size_t)FMF_NOALLOC_SCRATCH_BYTES) {
        if (need == SIZE_MAX)
            return set_error(FMF_ERR_ARG,
                             "noalloc: this search needs more scratch than the %zu bytes the "
                             "allocation-free entry point has (use fmf_matched_filter_ex)",
                             (size_t)FMF_NOALLOC_SCRATCH_BYTES);
        return set_error(FMF_ERR_ARG,
                         "noalloc: this search needs %zu bytes of scratch; the allocation-free entry "
                         "point has %zu (use fmf_matched_filter_ex)",
                         need, (size_t)FMF_NOALLOC_SCRATCH_BYTES);
    }
    const int T = (int)n_templates, SC = (int)SCz, L = (int)n_samples_template,
              N = (int)n_samples_data;
    if (window_stats_smem(L, full) > 227 * 1024)
        return set_error(FMF_ERR_SMEM, "noalloc: template length %d too long", L);

    unsigned char *base = nullptr;
    int rc = scratch_base(&base);
    if (rc)
        return rc;
    cudaStream_t s = (cudaStream_t)stream;
    Carve cv{base};
    int *k_lo = cv.take<int>(2 * (size_t)T);
    int *k_hi = k_lo + T;
    float *stat_e = cv.take<float>((size_t)SC * N * (full ? 2 : 1));
    float *sst = energies ? cv.take<float>((size_t)T * SC) : nullptr;
    float *dcen = nullptr, *mu = nullptr, *tcen = nullptr, *tsum = nullptr;
    if (full) {
        dcen = cv.take<float>((size_t)SC * N);
        mu = cv.take<float>((size_t)SC);
        tcen = cv.take<float>((size_t)T * SC * L);
        tsum = cv.take<float>((size_t)T * SC);
    }

    cudaGetLastError();
    template_range_kernel<<<(T + 127) / 128, 128, 0, s>>>(moveouts, T, SC, L, N, (int)step, (int)n_corr,
                                                            k_lo, k_hi);
    count_launch();
    if (energies) {  // as numpy sums float32 templates**2: bit-identical energies
        template_energy_kernel<<<(T * SC + 127) / 128, 128, 0, s>>>(templates, T * SC, L, sst);
        count_launch();
    }
    if (full) {
        template_center_kernel<<<(unsigned)((size_t)T * SC), 128, 0, s>>>(templates, L, tcen, tsum);
        channel_centre_kernel<<<SC, 1024, 0, s>>>(data, N, mu);
        count_launch(2);
    }
    if ((rc = launch_window_stats(data, N, L, SC, mu, dcen, stat_e, s)))
        return rc;
    cudaError_t e;
    if ((e = cudaGetLastError()) != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "noalloc: preprocessing launch: %s", cudaGetErrorString(e));
    if (!sum_cc_mode) {
        e = cudaMemsetAsync(cc_out, 0, (size_t)T * n_corr * SC * sizeof(float), s);
        if (e != cudaSuccess)
            return set_error(FMF_ERR_CUDA, "noalloc: clearing the output: %s", cudaGetErrorString(e));
    }

    Problem P;
    P.tpl = full ? tcen : templates;
    P.sst = energies ? sst : sum_square_templates;
    P.tsum = tsum;
    P.mo = moveouts;
    P.w = weights;
    P.data = full ? dcen : data;
    P.stat_e = stat_e;
    P.k_lo = k_lo;
    P.k_hi = k_hi;
    P.out = cc_out;
    P.T = T;
    P.SC = SC;
    P.L = L;
    P.N = N;
    P.step = (int)step;
    P.n_corr = (int)n_corr;
    P.normalize = normalize;
    P.network_sum = sum_cc_mode != 0;
    P.ntap = nullptr;
    P.pre2q = nullptr;
    P.unit2 = nullptr;
    P.pre1f = nullptr;
    P.zweight = nullptr;
    P.vp_norm = P.vp_bias = P.vp_scale = nullptr;
    if ((rc = launch_plain_all(P, s)))
        return rc;
    return FMF_OK;
}
