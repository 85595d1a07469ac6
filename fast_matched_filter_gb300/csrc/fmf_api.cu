// fmf_api.cu -- C ABI and host driver of the GB300 matched-filter library.
//
// Replaces the reference GPU host driver (matched_filter.cu:171-399): one
// process drives its current device; inputs are copied (or used in place
// when the caller passes device pointers), the per-call preprocessing kernels
// run once, and one kernel launch covers every template and every output
// index -- no lag chunks, no per-chunk memset/sync/copy round trips.
// Errors are returned as FMF_* status codes with a message for
// fmf_last_error(); nothing here terminates the process.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <climits>
#include <mutex>
#include <thread>
#include <vector>

#if defined(__linux__)
#include <sys/mman.h>
#include <unistd.h>
#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23  /* Linux 5.14 */
#endif
#endif

#include "fmf_common.cuh"

#define FMF_VERSION_STRING "fmf_gb300 0.1.0 sm_103a"

namespace fmf {

// ---------------------------------------------------------------- errors
static thread_local int g_status = FMF_OK;
static thread_local char g_msg[512] = "";
static thread_local int g_launches = 0;

int set_error(int status, const char *fmt, ...)
{
    g_status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    return status;
}

static int clear_error()
{
    g_status = FMF_OK;
    g_msg[0] = '\0';
    return FMF_OK;
}

void count_launch(int n) { g_launches += n; }
static thread_local int g_last_precision = -1;
void set_last_precision(int precision) { g_last_precision = precision; }
void reset_launch_count() { g_launches = 0; }

// ---------------------------------------------------------------- event timing
// Opt-in (fmf_timing_begin/end): every call records CUDA events on its stream
// around the preprocessing kernels and around the correlation kernel, and
// host-pointer calls around their copies.
enum SpanKind {
    kSpanPrep = 0,     // preprocessing kernels
    kSpanKernel = 1,   // correlation kernels (with their operand repacking)
    kSpanInput = 2,    // host-to-device copies of the inputs
    kSpanOutput = 3,   // device-to-host copies of the result, first to last
    kSpanTail = 4,     // the part of those copies after the last correlation kernel
    kSpanKinds = 5
};
struct TimedSpan {
    cudaEvent_t a, b;
    int kind;
};
static thread_local bool g_timing = false;
static thread_local TimedSpan g_spans[4096];
static thread_local int g_nspans = 0;

static cudaEvent_t mark(cudaStream_t s)
{
    cudaEvent_t e = nullptr;
    if (!g_timing)
        return nullptr;
    if (cudaEventCreate(&e) != cudaSuccess)
        return nullptr;
    cudaEventRecord(e, s);
    return e;
}

static void span(cudaEvent_t a, cudaEvent_t b, int kind)
{
    if (!a || !b)
        return;
    if (g_nspans < 4096)
        g_spans[g_nspans++] = TimedSpan{a, b, kind};
    else {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
}

// Maps the host pages of [p, p + bytes) for writing, on several threads, so
// that the device-to-host copy of a result into them does not fault every page
// in on its way: a fresh output array -- the reference's front-end allocates
// one per call, fast_matched_filter.py:269-274 -- is untouched memory, and a
// copy into it ran at 29 GB/s against 190 GB/s into mapped pages (8.6 GB for
// the full-day search).  Mapped pages cost a page-table walk; where the
// kernel refuses the advice (older kernels, page-locked mappings) nothing
// is done.
void populate_host(void *p, size_t bytes)
{
#if defined(__linux__)
    const long page = sysconf(_SC_PAGESIZE);
    if (!p || bytes == 0 || page <= 0)
        return;
    const uintptr_t a = (uintptr_t)p & ~(uintptr_t)(page - 1);
    const uintptr_t b = ((uintptr_t)p + bytes + page - 1) & ~(uintptr_t)(page - 1);
    const size_t pages = (b - a) / page;
    const size_t min_part = ((size_t)32 << 20) / page;  // at least 32 MB per thread
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt == 0 ? 1 : (nt > 16 ? 16 : nt);
    if (pages / min_part < nt)
        nt = (unsigned)(pages / min_part > 0 ? pages / min_part : 1);
    auto part = [&](unsigned i) {
        const size_t p0 = pages * i / nt, p1 = pages * (i + 1) / nt;
        if (p1 > p0)
            madvise((void *)(a + p0 * page), (p1 - p0) * page, MADV_POPULATE_WRITE);
    };
    if (nt == 1) {
        part(0);
        return;
    }
    std::vector<std::thread> pool;
    for (unsigned i = 1; i < nt; i++)
        pool.emplace_back(part, i);
    part(0);
    for (auto &t : pool)
        t.join();
#else
    (void)p;
    (void)bytes;
#endif
}

// Page-locked (or registered) host memory is mapped already: populate_host
// would only walk its page tables.
bool host_is_pinned(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

int check_launch(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return FMF_OK;
}

static int cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return FMF_OK;
    if (e == cudaErrorMemoryAllocation)
        return set_error(FMF_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
    return set_error(FMF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ---------------------------------------------------------------- kernels
__global__ void template_range_kernel(const int *, int, int, int, int, int, int, int *, int *);
__global__ void template_center_kernel(const float *, int, float *, float *);
__global__ void template_energy_kernel(const float *, int, int, float *);
__global__ void channel_centre_kernel(const float *, int, float *);
__global__ void zero_count_kernel(const float *, long long, long long, long long, unsigned long long *);
int launch_tc(const Problem &P, const float *data_for_tc, int precision, unsigned *err, Scratch &ws,
              cudaStream_t s, int forced_nb, int template_group);
int launch_wait_selftest(unsigned *err, unsigned ms, cudaStream_t s);
int launch_fisher_atanh(const float *y, float *out, long long n, cudaStream_t s);

// ---------------------------------------------------------------- device error word
// Kernels with bounded waits OR a code into this word when a wait gives up.
constexpr int kMaxDevices = 64;
static unsigned *g_err_word[kMaxDevices];

int device_error_word(unsigned **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return set_error(FMF_ERR_CUDA, "no usable current device");
    static std::mutex m;  // first calls from several host threads allocate once
    std::lock_guard<std::mutex> lock(m);
    if (!g_err_word[dev]) {
        void *p = nullptr;
        if ((e = cudaMalloc(&p, 64)) != cudaSuccess || (e = cudaMemset(p, 0, 64)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(FMF_ERR_CUDA, "allocating the error word: %s", cudaGetErrorString(e));
        }
        g_err_word[dev] = static_cast<unsigned *>(p);
    }
    *out = g_err_word[dev];
    return FMF_OK;
}

// Reads and clears the error word after the device has finished the work.
int collect_device_errors()
{
    unsigned *w = nullptr;
    int rc = device_error_word(&w);
    if (rc)
        return rc;
    unsigned v = 0;
    cudaError_t e = cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && v)
        e = cudaMemset(w, 0, sizeof(v));
    if (e != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "reading the error word: %s", cudaGetErrorString(e));
    if (v)
        return set_error(FMF_ERR_TIMEOUT, "a device-side wait gave up (code 0x%x)", v);
    return FMF_OK;
}

// The device's default pool keeps the memory that calls free (release threshold
// at its maximum), so that the next call reuses it instead of mapping it again.
void keep_pool_cached()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long thr = ULLONG_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
}

// ---------------------------------------------------------------- validation
int validate_args(const Args &a)
{
    if (!a.tpl || !a.mo || !a.data || !a.w || !a.out)
        return set_error(FMF_ERR_ARG, "null array argument");  // sst may be null: computed here
    if (a.step < 1 || a.L < 1 || a.T < 1 || a.S < 1 || a.C < 1 || a.n_corr < 1)
        return set_error(FMF_ERR_ARG,
                         "sizes must be positive (step=%zu L=%zu T=%zu S=%zu C=%zu n_corr=%zu)",
                         a.step, a.L, a.T, a.S, a.C, a.n_corr);
    if (a.N < a.L)
        return set_error(FMF_ERR_ARG, "data length %zu is shorter than the template length %zu", a.N,
                         a.L);
    if (a.N > (size_t)INT_MAX / 2 || a.n_corr > (size_t)INT_MAX || a.S * a.C > (size_t)INT_MAX ||
        a.T > (size_t)INT_MAX || a.step > (size_t)INT_MAX / 2)
        return set_error(FMF_ERR_ARG, "sizes exceed the 32-bit index range of this build");
    if (a.n_corr > (a.N - a.L) / a.step + 1)
        return set_error(FMF_ERR_ARG, "n_corr=%zu exceeds (N-L)/step+1=%zu", a.n_corr,
                         (a.N - a.L) / a.step + 1);
    if (a.normalize != 0 && a.normalize != 1)
        return set_error(FMF_ERR_ARG, "normalize must be 0 (short) or 1 (full), got %d", a.normalize);
    if (a.precision < FMF_PREC_FP32 || a.precision > FMF_PREC_AUTO)
        return set_error(FMF_ERR_ARG, "unknown precision %d", a.precision);
    if (a.flags & FMF_FLAG_DEVICE_POINTERS) {  // the kernels load these in place: 4-byte elements
        const void *ptrs[6] = {a.tpl, a.sst, a.mo, a.data, a.w, a.out};
        for (const void *p : ptrs)
            if ((uintptr_t)p & 3)
                return set_error(FMF_ERR_ARG, "device array %p is not 4-byte aligned", p);
    }
    return FMF_OK;
}

// ---------------------------------------------------------------- core (device pointers)
int prepare_problem(const Args &a, Scratch &ws, cudaStream_t s, Problem *Pout, const float **data_for_tc)
{
    int rc;
    const int T = (int)a.T, SC = (int)(a.S * a.C), L = (int)a.L, N = (int)a.N;
    const bool full = a.normalize == 1;
    if (window_stats_smem(L, full) > 227 * 1024)
        return set_error(FMF_ERR_SMEM, "template length %d too long for the window-statistics kernel", L);

    int *k_lo = nullptr, *k_hi = nullptr;
    float *stat_e = nullptr, *mu = nullptr, *dcen = nullptr, *tcen = nullptr, *tsum = nullptr;
    if ((rc = ws.get(&k_lo, 2 * (size_t)T, "template ranges")))
        return rc;
    k_hi = k_lo + T;
    if ((rc = ws.get(&stat_e, (size_t)SC * N * (full ? 2 : 1), "window statistics")))
        return rc;
    if (full) {
        if ((rc = ws.get(&mu, (size_t)SC, "channel centres")) ||
            (rc = ws.get(&dcen, (size_t)SC * N, "centred data")) ||
            (rc = ws.get(&tcen, (size_t)T * SC * L, "centred templates")) ||
            (rc = ws.get(&tsum, (size_t)T * SC, "template sums")))
            return rc;
    }

    template_range_kernel<<<(T + 127) / 128, 128, 0, s>>>(a.mo, T, SC, L, N, (int)a.step,
                                                            (int)a.n_corr, k_lo, k_hi);
    count_launch();
    const float *sst = a.sst;
    if (!sst) {  // template energies as numpy computes them for float32 templates
        float *e = nullptr;
        if ((rc = ws.get(&e, (size_t)T * SC, "template energies")))
            return rc;
        const int rows = T * SC;
        template_energy_kernel<<<(rows + 127) / 128, 128, 0, s>>>(a.tpl, rows, L, e);
        count_launch();
        sst = e;
    }
    if (full) {
        template_center_kernel<<<(unsigned)((size_t)T * SC), 128, 0, s>>>(a.tpl, L, tcen, tsum);
        channel_centre_kernel<<<SC, 1024, 0, s>>>(a.data, N, mu);
        count_launch(2);
    }
    if ((rc = launch_window_stats(a.data, N, L, SC, mu, dcen, stat_e, s)))
        return rc;
    if ((rc = check_launch("preprocessing kernels")))
        return rc;

    Problem P;
    P.tpl = full ? tcen : a.tpl;
    P.sst = sst;
    P.tsum = tsum;
    P.mo = a.mo;
    P.w = a.w;
    P.data = full ? dcen : a.data;
    P.stat_e = stat_e;
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
    P.network_sum = a.sum_mode != 0;
    P.ntap = nullptr;
    P.pre2q = nullptr;
    P.unit2 = nullptr;
    P.pre1f = nullptr;
    P.zweight = nullptr;
    P.vp_norm = P.vp_bias = P.vp_scale = nullptr;

    if (!P.network_sum) {
        size_t bytes = (size_t)T * a.n_corr * SC * sizeof(float);
        if ((rc = cuda_status(cudaMemsetAsync(a.out, 0, bytes, s), "clearing the output")))
            return rc;
    }
    *Pout = P;
    *data_for_tc = full ? dcen : a.data;
    return FMF_OK;
}

// check_zeros count of templates [t0, t0 + nt) of a search's output into
// counts[t0 ..] (device), on stream s.
static int launch_zero_count(const Args &a, const float *out, int t0, int nt,
                             unsigned long long *counts, cudaStream_t s)
{
    const long long row = (long long)a.n_corr * (a.sum_mode ? 1 : (long long)(a.S * a.C));
    const long long last = a.sum_mode ? (long long)a.n_corr : (long long)a.C;
    long long stop = a.zero_stop < 0 ? 0 : (a.zero_stop > last ? last : a.zero_stop);
    const long long span = last == row ? stop : row;
    long long blocks = (span + 256 * 8 - 1) / (256 * 8);
    blocks = blocks < 1 ? 1 : (blocks > 1024 ? 1024 : blocks);
    for (int c0 = 0; c0 < nt; c0 += 65535) {
        const int cn = nt - c0 < 65535 ? nt - c0 : 65535;
        zero_count_kernel<<<dim3((unsigned)blocks, (unsigned)cn), 256, 0, s>>>(
            out + (size_t)(t0 + c0) * row, row, last, stop, counts + t0 + c0);
        count_launch();
    }
    return check_launch("zero count");
}

// Plain FP32 form over all templates, in launches of at most 65535 templates.
int launch_plain_all(const Problem &P, cudaStream_t s)
{
    int rc;
    for (int t0 = 0; t0 < P.T; t0 += 65535) {
        Problem Q = P;
        int nt = P.T - t0 < 65535 ? P.T - t0 : 65535;
        size_t o = (size_t)t0 * P.SC;
        Q.tpl += o * P.L;
        Q.sst += o;
        if (Q.tsum)
            Q.tsum += o;
        Q.mo += o;
        Q.w += o;
        Q.k_lo += t0;
        Q.k_hi += t0;
        Q.out += (size_t)t0 * P.n_corr * (P.network_sum ? 1 : P.SC);
        Q.T = nt;
        if ((rc = launch_plain(Q, s)))
            return rc;
    }
    return FMF_OK;
}

// Search on device pointers with its working arrays in `ws` (they stay
// allocated, and *Pout valid, until ws goes out of scope).
static int run_device_ws(const Args &a, cudaStream_t s, Scratch &ws, Problem *Pout)
{
    int rc;
    Problem &P = *Pout;
    const float *data_for_tc = nullptr;
    cudaEvent_t ev_prep0 = mark(s);
    if ((rc = prepare_problem(a, ws, s, &P, &data_for_tc)))
        return rc;
    cudaEvent_t ev_prep1 = mark(s);
    span(ev_prep0, ev_prep1, kSpanPrep);
    int precision = a.precision;
    if (precision == FMF_PREC_AUTO && (rc = choose_auto_precision(P, ws, s, &precision)))
        return rc;
    set_last_precision(precision);
    if (precision != FMF_PREC_FP32) {
        unsigned *err = nullptr;
        if ((rc = device_error_word(&err)))
            return rc;
        const char *nb_env = getenv("FMF_TC_NB");
        int forced = nb_env ? atoi(nb_env) : 0;
        if (a.flags & 0xff00)
            forced = ((a.flags >> 8) & 0xff) * 16;
        const int group = (a.flags >> 16) & 0xff;
        if (forced != 0 && forced != 32 && forced != 64 && forced != 128)
            return set_error(FMF_ERR_ARG, "tensor-core tile of %d lag blocks (32, 64 or 128)", forced);
        cudaEvent_t ev0 = mark(s);
        rc = launch_tc(P, data_for_tc, precision, err, ws, s, forced, group);
        span(ev0, mark(s), kSpanKernel);
        return rc;
    }
    cudaEvent_t ev_main0 = mark(s);
    rc = launch_plain_all(P, s);
    span(ev_main0, mark(s), kSpanKernel);
    return rc;
}

static int run_device(const Args &a, cudaStream_t s)
{
    Scratch ws(s);
    Problem P;
    int rc = run_device_ws(a, s, ws, &P);
    if (rc || !a.zero_counts)
        return rc;
    if ((rc = cuda_status(cudaMemsetAsync(a.zero_counts, 0, a.T * sizeof(unsigned long long), s),
                          "clearing the zero counts")))
        return rc;
    return launch_zero_count(a, a.out, 0, (int)a.T, a.zero_counts, s);
}

// ---------------------------------------------------------------- host-pointer path
// Templates [t0, t0 + nt) of a prepared problem.
static Problem problem_subset(const Problem &P, int t0, int nt)
{
    Problem Q = P;
    const size_t o = (size_t)t0 * P.SC;
    Q.tpl += o * P.L;
    Q.sst += o;
    if (Q.tsum)
        Q.tsum += o;
    Q.mo += o;
    Q.w += o;
    Q.k_lo += t0;
    Q.k_hi += t0;
    Q.out += (size_t)t0 * P.n_corr * (P.network_sum ? 1 : P.SC);
    Q.T = nt;
    return Q;
}

// Device-resident search whose result is copied to `host_out` in template
// chunks on a second stream, each chunk's copy overlapping the next chunk's
// kernel.  Preprocessing is done once for all templates.
static int run_streamed(const Args &d, float *host_out, cudaStream_t s)
{
    int rc;
    Scratch ws(s);
    Problem P;
    const float *data_for_tc = nullptr;
    cudaEvent_t ev_prep0 = mark(s);
    if ((rc = prepare_problem(d, ws, s, &P, &data_for_tc)))
        return rc;
    cudaEvent_t ev_kern0 = mark(s);
    span(ev_prep0, ev_kern0, kSpanPrep);
    const size_t row = (size_t)P.n_corr * (P.network_sum ? 1 : P.SC);  // floats per template
    const size_t out_bytes = (size_t)P.T * row * sizeof(float);
    const int n_chunks = out_bytes < ((size_t)64 << 20) ? 1 : (P.T < 8 ? P.T : 8);
    // Template chunks of tapering size (weights 8,8,8,8,4,2,1,1 of 40 when there
    // are enough templates): each chunk's copy overlaps the next chunk's kernel,
    // and the last copy, which nothing overlaps, is small.
    int bounds[9];
    {
        static const int wts[8] = {8, 8, 8, 8, 4, 2, 1, 1};
        const bool taper = n_chunks == 8 && P.T >= 40;
        int acc = 0;
        bounds[0] = 0;
        for (int c = 0; c < n_chunks; c++) {
            acc += taper ? wts[c] : 1;
            const int total = taper ? 40 : n_chunks;
            bounds[c + 1] = (int)(((long long)P.T * acc) / total);
        }
        bounds[n_chunks] = P.T;
    }
    unsigned *err = nullptr;
    std::vector<unsigned char> tcfull;
    int split = 0;
    int precision = d.precision;
    if (precision == FMF_PREC_AUTO && (rc = choose_auto_precision(P, ws, s, &precision)))
        return rc;
    set_last_precision(precision);
    if (precision != FMF_PREC_FP32) {
        if ((rc = device_error_word(&err)))
            return rc;
        split = precision == FMF_PREC_SPLIT_BF16;
        const char *nb_env = getenv("FMF_TC_NB");
        int forced = nb_env ? atoi(nb_env) : 0;
        if (d.flags & 0xff00)
            forced = ((d.flags >> 8) & 0xff) * 16;
        const int nb = tc_choose_nb(P.L, P.step, split, forced);
        if (nb == 0)
            return set_error(FMF_ERR_SMEM, "template length %d, step %d: tensor-core tile does not fit "
                                           "shared memory", P.L, P.step);
        tcfull.resize(tc_prob_size());
        if ((rc = tc_prepare(P, data_for_tc, split, nb, (d.flags >> 16) & 0xff, ws, s,
                             reinterpret_cast<TcProb *>(tcfull.data()))))
            return rc;
    }
    unsigned long long *zc = nullptr;  // device zero counts, copied to d.zero_counts (host)
    if (d.zero_counts) {
        if ((rc = ws.get(&zc, (size_t)P.T, "zero counts")) ||
            (rc = cuda_status(cudaMemsetAsync(zc, 0, (size_t)P.T * sizeof(unsigned long long), s),
                              "clearing the zero counts")))
            return rc;
    }
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev[9] = {};
    cudaError_t e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
    for (int i = 0; i <= n_chunks && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
    if (e == cudaSuccess) {
        // every chunk's kernels first, then the copies: a copy into pageable host memory
        // returns only when it is done, and the kernels of the later chunks are queued by then
        int launched = 0;
        for (int c = 0; c < n_chunks && rc == FMF_OK && e == cudaSuccess; c++, launched++) {
            const int t0 = bounds[c], nt = bounds[c + 1] - bounds[c];
            if (nt > 0) {
                if (!tcfull.empty()) {
                    std::vector<unsigned char> sub(tc_prob_size());
                    unsigned long long *queue = nullptr;
                    tc_subset(reinterpret_cast<const TcProb *>(tcfull.data()), t0, nt,
                              reinterpret_cast<TcProb *>(sub.data()));
                    if (!(rc = ws.get(&queue, 1, "tile queue")))
                        rc = tc_run(reinterpret_cast<const TcProb *>(sub.data()), 1, split, queue, err, s);
                } else {
                    rc = launch_plain_all(problem_subset(P, t0, nt), s);
                }
                if (!rc && zc)
                    rc = launch_zero_count(d, P.out, t0, nt, zc, s);
            }
            if (!rc)
                e = cudaEventRecord(ev[c], s);
        }
        // end of the last correlation kernel (twice: each span owns its events)
        cudaEvent_t ev_kern1 = mark(s), ev_kern1b = mark(s), ev_out0 = nullptr;
        span(ev_kern0, ev_kern1, kSpanKernel);
        const bool pinned = host_is_pinned(host_out);
        for (int c = 0; c < launched && rc == FMF_OK && e == cudaSuccess; c++) {
            const int t0 = bounds[c], nt = bounds[c + 1] - bounds[c];
            if (nt <= 0)
                continue;
            const size_t off = (size_t)t0 * row, n = (size_t)nt * row * sizeof(float);
            if ((e = cudaStreamWaitEvent(s2, ev[c], 0)) != cudaSuccess)
                break;
            if (!ev_out0)
                ev_out0 = mark(s2);
            if (!pinned)
                populate_host(host_out + off, n);  // while the kernels run
            if ((e = cudaMemcpyAsync(host_out + off, P.out + off, n, cudaMemcpyDeviceToHost, s2)) !=
                cudaSuccess)
                break;
        }
        // the copy-out window, and its part after the last correlation kernel
        cudaEvent_t ev_out1 = ev_out0 ? mark(s2) : nullptr, ev_out1b = ev_out0 ? mark(s2) : nullptr;
        span(ev_out0, ev_out1, kSpanOutput);
        span(ev_kern1b, ev_out1b, kSpanTail);
        if (!ev_out1b && ev_kern1b)
            cudaEventDestroy(ev_kern1b);
        if (e == cudaSuccess && rc == FMF_OK && zc)
            e = cudaMemcpyAsync(d.zero_counts, zc, (size_t)P.T * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, s);
        // scratch is freed on s: let s wait for the last copy
        if (e == cudaSuccess && (e = cudaEventRecord(ev[n_chunks], s2)) == cudaSuccess)
            e = cudaStreamWaitEvent(s, ev[n_chunks], 0);
    }
    if (e != cudaSuccess && rc == FMF_OK)
        rc = cuda_status(e, "streaming the result to the host");
    if (s2) {
        cudaStreamSynchronize(s2);
        cudaStreamDestroy(s2);
    }
    for (int i = 0; i <= n_chunks; i++)
        if (ev[i])
            cudaEventDestroy(ev[i]);
    return rc;
}

// Device copies of the five input arrays of a host-pointer call (in `io`);
// *d = a with its input pointers replaced.
static int copy_inputs(const Args &a, Scratch &io, cudaStream_t s, Args *d)
{
    int rc;
    const size_t SC = a.S * a.C;
    const size_t n_tsc = a.T * SC;
    const size_t n[5] = {n_tsc * a.L, n_tsc, n_tsc, SC * a.N, n_tsc};
    const void *src[5] = {a.tpl, a.sst, a.mo, a.data, a.w};
    float *buf[5];
    for (int i = 0; i < 5; i++) {
        if (!src[i]) {  // template energies left to the library
            buf[i] = nullptr;
            continue;
        }
        if ((rc = io.get(&buf[i], n[i], "input copies")))
            return rc;
        if ((rc = cuda_status(cudaMemcpyAsync(buf[i], src[i], n[i] * 4, cudaMemcpyHostToDevice, s),
                              "copying inputs to the device")))
            return rc;
    }
    *d = a;
    d->tpl = buf[0];
    d->sst = buf[1];
    d->mo = reinterpret_cast<const int *>(buf[2]);
    d->data = buf[3];
    d->w = buf[4];
    return FMF_OK;
}

static int run_host(const Args &a, cudaStream_t s)
{
    int rc;
    const size_t out_n = a.T * a.n_corr * (a.sum_mode ? 1 : a.S * a.C);
    {
        Scratch io(s);  // device copies of the arguments, freed in stream order
        Args d;
        float *out = nullptr;
        cudaEvent_t ev_in0 = mark(s);
        if ((rc = copy_inputs(a, io, s, &d)) || (rc = io.get(&out, out_n, "output copy")))
            return rc;
        span(ev_in0, mark(s), kSpanInput);
        d.out = out;
        if ((rc = run_streamed(d, a.out, s)))
            return rc;
    }
    if ((rc = cuda_status(cudaStreamSynchronize(s), "matched filter")))
        return rc;
    return g_last_precision != FMF_PREC_FP32 ? collect_device_errors() : FMF_OK;
}

static int entry(const Args &a, void *stream)
{
    clear_error();
    g_launches = 0;
    int rc = validate_args(a);
    if (rc)
        return rc;
    keep_pool_cached();
    cudaGetLastError();  // this library's runtime state only: start from a clean slate
    cudaStream_t s = (cudaStream_t)stream;
    if (a.flags & FMF_FLAG_DEVICE_POINTERS)
        return run_device(a, s);
    return run_host(a, s);
}

// ---------------------------------------------------------------- detection
struct DetectOut {
    float n_mad;
    size_t min_sep, max_det;
    float *med, *mad, *thr;
    int *count, *lag;
    float *val;
};

// Device buffers standing in for host outputs (host-pointer calls).
struct DetectDev {
    float *med = nullptr, *mad = nullptr, *thr = nullptr, *val = nullptr;
    int *count = nullptr, *lag = nullptr;
};

static int detect_outputs(const DetectOut &o, size_t T, bool device, Scratch &ws, DetectDev *d)
{
    int rc;
    if (device) {
        d->med = o.med;
        d->mad = o.mad;
        d->thr = o.thr;
        d->count = o.count;
        d->lag = o.lag;
        d->val = o.val;
        return FMF_OK;
    }
    const size_t nd = T * o.max_det;
    if ((rc = ws.get(&d->med, T, "detection outputs")) || (rc = ws.get(&d->mad, T, "detection outputs")) ||
        (rc = ws.get(&d->thr, T, "detection outputs")) || (rc = ws.get(&d->count, T, "detection outputs")) ||
        (rc = ws.get(&d->lag, nd > 0 ? nd : 1, "detection outputs")) ||
        (rc = ws.get(&d->val, nd > 0 ? nd : 1, "detection outputs")))
        return rc;
    return FMF_OK;
}

static int detect_copy_back(const DetectOut &o, size_t T, const DetectDev &d, cudaStream_t s)
{
    int rc;
    const size_t nd = T * o.max_det;
    struct {
        void *dst;
        const void *src;
        size_t bytes;
    } cp[6] = {{o.med, d.med, T * 4}, {o.mad, d.mad, T * 4}, {o.thr, d.thr, T * 4},
               {o.count, d.count, T * 4}, {o.lag, d.lag, nd * 4}, {o.val, d.val, nd * 4}};
    for (auto &c : cp)
        if (c.dst && c.bytes &&
            (rc = cuda_status(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, s),
                              "copying detections to the host")))
            return rc;
    if ((rc = cuda_status(cudaStreamSynchronize(s), "detection")))
        return rc;
    return detect_finish_host(o.count, T);
}

static int detect_entry(const float *cc, size_t T, size_t n_corr, const int *begin, const int *end,
                        const DetectOut &o, int flags, cudaStream_t s)
{
    int rc;
    if ((rc = validate_detect(T, n_corr, o.n_mad, o.min_sep, o.max_det, o.count, o.lag, o.val)))
        return rc;
    if (!cc)
        return set_error(FMF_ERR_ARG, "detection: null cc");
    if ((begin == nullptr) != (end == nullptr))
        return set_error(FMF_ERR_ARG, "detection: give both lag_begin and lag_end, or neither");
    const bool device = flags & FMF_FLAG_DEVICE_POINTERS;
    if (!device && begin)
        for (size_t t = 0; t < T; t++)
            if (begin[t] < 0 || end[t] < begin[t] || (size_t)end[t] > n_corr)
                return set_error(FMF_ERR_ARG, "detection: lag window [%d, %d) of template %zu is not "
                                              "inside [0, %zu)", begin[t], end[t], t, n_corr);
    keep_pool_cached();
    cudaGetLastError();
    Scratch ws(s);
    DetectDev d;
    if ((rc = detect_outputs(o, T, device, ws, &d)))
        return rc;
    if (device)
        return detect_device(cc, (int)T, (int)n_corr, n_corr, begin, end, o.n_mad, (int)o.min_sep,
                             (int)o.max_det, d.med, d.mad, d.thr, d.count, d.lag, d.val, ws, s);
    int *range = nullptr;
    if (begin) {
        if ((rc = ws.get(&range, 2 * T, "lag windows")) ||
            (rc = cuda_status(cudaMemcpyAsync(range, begin, T * 4, cudaMemcpyHostToDevice, s),
                              "copying lag windows")) ||
            (rc = cuda_status(cudaMemcpyAsync(range + T, end, T * 4, cudaMemcpyHostToDevice, s),
                              "copying lag windows")))
            return rc;
    }
    // rows in chunks of at most 1 GiB of device memory
    size_t per = ((size_t)1 << 30) / (n_corr * sizeof(float));
    per = per < 1 ? 1 : (per > T ? T : per);
    float *rows = nullptr;
    if ((rc = ws.get(&rows, per * n_corr, "cc rows")))
        return rc;
    for (size_t t0 = 0; t0 < T; t0 += per) {
        const size_t nt = T - t0 < per ? T - t0 : per;
        if ((rc = cuda_status(cudaMemcpyAsync(rows, cc + t0 * n_corr, nt * n_corr * 4,
                                              cudaMemcpyHostToDevice, s),
                              "copying cc rows to the device")))
            return rc;
        const size_t od = t0 * o.max_det;
        if ((rc = detect_device(rows, (int)nt, (int)n_corr, n_corr, range ? range + t0 : nullptr,
                                range ? range + T + t0 : nullptr, o.n_mad, (int)o.min_sep,
                                (int)o.max_det, d.med + t0, d.mad + t0, d.thr + t0, d.count + t0,
                                d.lag + od, d.val + od, ws, s)))
            return rc;
    }
    return detect_copy_back(o, T, d, s);
}

// Search (network sum) into a device buffer, then detection over each
// template's valid lag range; only the detections leave the device.
static int search_detect_entry(const Args &a0, const DetectOut &o, cudaStream_t s)
{
    int rc;
    Args a = a0;
    a.sum_mode = 1;
    a.out = reinterpret_cast<float *>(o.count);  // placeholder for the argument check
    if ((rc = validate_args(a)) ||
        (rc = validate_detect(a.T, a.n_corr, o.n_mad, o.min_sep, o.max_det, o.count, o.lag, o.val)))
        return rc;
    keep_pool_cached();
    cudaGetLastError();
    const bool device = a.flags & FMF_FLAG_DEVICE_POINTERS;
    Scratch ws(s);
    Args d = a;
    if (!device && (rc = copy_inputs(a, ws, s, &d)))
        return rc;
    DetectDev dd;
    if ((rc = detect_outputs(o, a.T, device, ws, &dd)))
        return rc;
    // templates in chunks whose cc rows take at most 16 GiB of device memory
    // (FMF_SEARCH_DETECT_CHUNK_BYTES overrides the limit)
    const size_t SC = a.S * a.C;
    size_t chunk_bytes = (size_t)16 << 30;
    if (const char *env = getenv("FMF_SEARCH_DETECT_CHUNK_BYTES"))
        chunk_bytes = (size_t)strtoull(env, nullptr, 10);
    size_t per = chunk_bytes / (a.n_corr * sizeof(float));
    per = per < 1 ? 1 : (per > a.T ? a.T : per);
    for (size_t t0 = 0; t0 < a.T; t0 += per) {
        const size_t nt = a.T - t0 < per ? a.T - t0 : per;
        Scratch wc(s);  // this chunk's working arrays, freed in stream order
        Args dc = d;
        dc.T = nt;
        dc.tpl = d.tpl + t0 * SC * a.L;
        dc.sst = d.sst ? d.sst + t0 * SC : nullptr;
        dc.mo = d.mo + t0 * SC;
        dc.w = d.w + t0 * SC;
        float *cc = nullptr;
        if ((rc = wc.get(&cc, nt * a.n_corr, "cc sums")))
            return rc;
        dc.out = cc;
        Problem P;
        const size_t od = t0 * o.max_det;
        if ((rc = run_device_ws(dc, s, wc, &P)) ||
            (rc = detect_device(cc, (int)nt, (int)a.n_corr, a.n_corr, P.k_lo, P.k_hi, o.n_mad,
                                (int)o.min_sep, (int)o.max_det, dd.med ? dd.med + t0 : nullptr,
                                dd.mad ? dd.mad + t0 : nullptr, dd.thr ? dd.thr + t0 : nullptr,
                                dd.count + t0, dd.lag ? dd.lag + od : nullptr,
                                dd.val ? dd.val + od : nullptr, wc, s)))
            return rc;
    }
    if (device)
        return FMF_OK;
    if ((rc = detect_copy_back(o, a.T, dd, s)))
        return rc;
    return g_last_precision != FMF_PREC_FP32 ? collect_device_errors() : FMF_OK;
}

}  // namespace fmf

// ---------------------------------------------------------------- C ABI
extern "C" {

int fmf_matched_filter_ex(const float *templates, const float *sum_square_templates,
                          const int *moveouts, const float *data, const float *weights,
                          size_t step, size_t n_samples_template, size_t n_samples_data,
                          size_t n_templates, size_t n_stations, size_t n_components,
                          size_t n_corr, float *cc_out, int normalize, int sum_cc_mode,
                          int precision, int flags, void *stream)
{
    fmf::Args a;
    a.tpl = templates;
    a.sst = sum_square_templates;
    a.mo = moveouts;
    a.data = data;
    a.w = weights;
    a.out = cc_out;
    a.step = step;
    a.L = n_samples_template;
    a.N = n_samples_data;
    a.T = n_templates;
    a.S = n_stations;
    a.C = n_components;
    a.n_corr = n_corr;
    a.normalize = normalize;
    a.sum_mode = sum_cc_mode;
    a.precision = precision;
    a.flags = flags;
    return fmf::entry(a, stream);
}

int fmf_matched_filter_check_zeros(const float *templates, const float *sum_square_templates,
                                   const int *moveouts, const float *data, const float *weights,
                                   size_t step, size_t n_samples_template, size_t n_samples_data,
                                   size_t n_templates, size_t n_stations, size_t n_components,
                                   size_t n_corr, float *cc_out, int normalize, int sum_cc_mode,
                                   int precision, int flags, void *stream, long long zero_stop,
                                   unsigned long long *zero_counts)
{
    if (!zero_counts) {
        fmf::clear_error();
        return fmf::set_error(FMF_ERR_ARG, "null zero_counts");
    }
    fmf::Args a;
    a.tpl = templates;
    a.sst = sum_square_templates;
    a.mo = moveouts;
    a.data = data;
    a.w = weights;
    a.out = cc_out;
    a.step = step;
    a.L = n_samples_template;
    a.N = n_samples_data;
    a.T = n_templates;
    a.S = n_stations;
    a.C = n_components;
    a.n_corr = n_corr;
    a.normalize = normalize;
    a.sum_mode = sum_cc_mode;
    a.precision = precision;
    a.flags = flags;
    a.zero_stop = zero_stop;
    a.zero_counts = zero_counts;
    return fmf::entry(a, stream);
}

int fmf_matched_filter(const float *templates, const float *sum_square_templates,
                       const int *moveouts, const float *data, const float *weights,
                       size_t step, size_t n_samples_template, size_t n_samples_data,
                       size_t n_templates, size_t n_stations, size_t n_components,
                       size_t n_corr, float *cc_out, int normalize, int sum_cc_mode)
{
    return fmf_matched_filter_ex(templates, sum_square_templates, moveouts, data, weights, step,
                                 n_samples_template, n_samples_data, n_templates, n_stations,
                                 n_components, n_corr, cc_out, normalize, sum_cc_mode,
                                 FMF_PREC_FP32, 0, nullptr);
}

int matched_filter(const float *templates, const float *sum_square_templates, const int *moveouts,
                   const float *data, const float *weights, size_t step, size_t n_samples_template,
                   size_t n_samples_data, size_t n_templates, size_t n_stations,
                   size_t n_components, size_t n_corr, float *cc_out, int normalize,
                   int sum_cc_mode)
{
    int rc = fmf_matched_filter(templates, sum_square_templates, moveouts, data, weights, step,
                                n_samples_template, n_samples_data, n_templates, n_stations,
                                n_components, n_corr, cc_out, normalize, sum_cc_mode);
    if (rc != FMF_OK)
        fprintf(stderr, "fmf_gb300 matched_filter failed (status %d): %s\n", rc, fmf::g_msg);
    return rc;
}

int fmf_detect(const float *cc, size_t n_templates, size_t n_corr, const int *lag_begin,
               const int *lag_end, float n_mad, size_t min_separation, size_t max_detections,
               float *median_out, float *mad_out, float *threshold_out, int *count_out, int *lag_out,
               float *value_out, int flags, void *stream)
{
    fmf::clear_error();
    fmf::g_launches = 0;
    if (flags & FMF_FLAG_DEVICE_POINTERS) {  // read and written in place: 4-byte elements
        const void *ptrs[9] = {cc, lag_begin, lag_end, median_out, mad_out, threshold_out,
                               count_out, lag_out, value_out};
        for (const void *p : ptrs)
            if ((uintptr_t)p & 3)
                return fmf::set_error(FMF_ERR_ARG, "device array %p is not 4-byte aligned", p);
    }
    const fmf::DetectOut o{n_mad,      min_separation, max_detections, median_out, mad_out,
                           threshold_out, count_out,   lag_out,        value_out};
    return fmf::detect_entry(cc, n_templates, n_corr, lag_begin, lag_end, o, flags,
                             (cudaStream_t)stream);
}

int fmf_matched_filter_detect(const float *templates, const float *sum_square_templates,
                              const int *moveouts, const float *data, const float *weights,
                              size_t step, size_t n_samples_template, size_t n_samples_data,
                              size_t n_templates, size_t n_stations, size_t n_components,
                              size_t n_corr, int normalize, int precision, float n_mad,
                              size_t min_separation, size_t max_detections, float *median_out,
                              float *mad_out, float *threshold_out, int *count_out, int *lag_out,
                              float *value_out, int flags, void *stream)
{
    fmf::clear_error();
    fmf::g_launches = 0;
    fmf::Args a;
    a.tpl = templates;
    a.sst = sum_square_templates;
    a.mo = moveouts;
    a.data = data;
    a.w = weights;
    a.out = nullptr;
    a.step = step;
    a.L = n_samples_template;
    a.N = n_samples_data;
    a.T = n_templates;
    a.S = n_stations;
    a.C = n_components;
    a.n_corr = n_corr;
    a.normalize = normalize;
    a.sum_mode = 1;
    a.precision = precision;
    a.flags = flags;
    const fmf::DetectOut o{n_mad,      min_separation, max_detections, median_out, mad_out,
                           threshold_out, count_out,   lag_out,        value_out};
    return fmf::search_detect_entry(a, o, (cudaStream_t)stream);
}

int fmf_template_energies(const float *templates, size_t n_rows, size_t n_samples_template, float *out,
                          int flags, void *stream)
{
    using namespace fmf;
    clear_error();
    g_launches = 0;
    if (!templates || !out)
        return set_error(FMF_ERR_ARG, "energies: null array argument");
    if (n_rows < 1 || n_samples_template < 1 || n_rows > (size_t)INT_MAX ||
        n_samples_template > (size_t)INT_MAX)
        return set_error(FMF_ERR_ARG, "energies: sizes out of range (rows=%zu L=%zu)", n_rows,
                         n_samples_template);
    keep_pool_cached();
    cudaGetLastError();
    cudaStream_t s = (cudaStream_t)stream;
    const int rows = (int)n_rows, L = (int)n_samples_template;
    if (flags & FMF_FLAG_DEVICE_POINTERS) {
        template_energy_kernel<<<(rows + 127) / 128, 128, 0, s>>>(templates, rows, L, out);
        count_launch();
        return check_launch("template energies");
    }
    int rc;
    Scratch ws(s);
    float *dt = nullptr, *de = nullptr;
    if ((rc = ws.get(&dt, n_rows * n_samples_template, "templates")) ||
        (rc = ws.get(&de, n_rows, "energies")) ||
        (rc = cuda_status(cudaMemcpyAsync(dt, templates, n_rows * n_samples_template * 4,
                                          cudaMemcpyHostToDevice, s),
                          "copying templates")))
        return rc;
    template_energy_kernel<<<(rows + 127) / 128, 128, 0, s>>>(dt, rows, L, de);
    count_launch();
    if ((rc = check_launch("template energies")) ||
        (rc = cuda_status(cudaMemcpyAsync(out, de, n_rows * 4, cudaMemcpyDeviceToHost, s),
                          "copying energies")))
        return rc;
    return cuda_status(cudaStreamSynchronize(s), "template energies");
}

int fmf_last_error(char *buf, size_t len)
{
    if (buf && len) {
        strncpy(buf, fmf::g_msg, len - 1);
        buf[len - 1] = '\0';
    }
    return fmf::g_status;
}

const char *fmf_version(void) { return FMF_VERSION_STRING; }

int fmf_last_launch_count(void) { return fmf::g_launches; }

int fmf_selftest_wait_timeout(unsigned ms)
{
    fmf::clear_error();
    if (ms < 1 || ms > 5000)
        return fmf::set_error(FMF_ERR_ARG, "selftest wait limit must be 1..5000 ms");
    unsigned *err = nullptr;
    int rc = fmf::device_error_word(&err);
    if (rc)
        return rc;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return fmf::cuda_status(e, "fmf_selftest_wait_timeout");
    if ((rc = fmf::collect_device_errors()))  // start from a clear word
        return rc;
    if ((rc = fmf::launch_wait_selftest(err, ms, nullptr)))
        return rc;
    return fmf_device_errors();
}

namespace fmf {
// 16 independent multiply-add chains per thread: the FP32 FMA rate the SMs
// sustain on register operands, the denominator of the plain kernel's roofline.
__global__ void __launch_bounds__(256) fma_rate_kernel(float *sink, int iters, float a, float b)
{
    float x[16];
#pragma unroll
    for (int i = 0; i < 16; i++)
        x[i] = threadIdx.x * 1e-3f + (float)i;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 16; i++)
            x[i] = fmaf(x[i], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 16; i++)
        s += x[i];
    if (s == -1.0f)  // never: keeps the chains live
        sink[0] = s;
}
}  // namespace fmf

int fmf_measure_fp32_fma(double *tflops)
{
    fmf::clear_error();
    if (!tflops)
        return fmf::set_error(FMF_ERR_ARG, "null output");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *sink = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    if (e == cudaSuccess)
        e = cudaMalloc(&sink, sizeof(float));
    if (e == cudaSuccess)
        e = cudaEventCreate(&a);
    if (e == cudaSuccess)
        e = cudaEventCreate(&b);
    const int iters = 20000, grid = 4 * sms;
    float ms = 0.0f, best = 0.0f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; rep++) {  // the first run warms the clocks
        fmf::fma_rate_kernel<<<grid, 256>>>(sink, iters, 0.999f, 0.001f);
        cudaEventRecord(a);
        fmf::fma_rate_kernel<<<grid, 256>>>(sink, iters, 0.999f, 0.001f);
        cudaEventRecord(b);
        if ((e = cudaEventSynchronize(b)) == cudaSuccess && (e = cudaEventElapsedTime(&ms, a, b)) == cudaSuccess)
            best = (best == 0.0f || ms < best) ? ms : best;
    }
    if (a)
        cudaEventDestroy(a);
    if (b)
        cudaEventDestroy(b);
    if (sink)
        cudaFree(sink);
    if (e != cudaSuccess)
        return fmf::cuda_status(e, "fmf_measure_fp32_fma");
    const double fma = (double)grid * 256 * 16 * iters;
    *tflops = 2.0 * fma / (best * 1e-3) / 1e12;
    return FMF_OK;
}

int fmf_eval_atanh(const float *y, float *out, size_t n, void *stream)
{
    fmf::clear_error();
    fmf::reset_launch_count();
    if (n > 0 && (!y || !out))
        return fmf::set_error(FMF_ERR_ARG, "null array argument");
    if (n > ((size_t)1 << 40))
        return fmf::set_error(FMF_ERR_ARG, "n too large");
    return fmf::launch_fisher_atanh(y, out, (long long)n, (cudaStream_t)stream);
}

int fmf_device_errors(void)
{
    fmf::clear_error();
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
        return fmf::cuda_status(e, "fmf_device_errors");
    return fmf::collect_device_errors();
}

int fmf_timing_begin(void)
{
    for (int i = 0; i < fmf::g_nspans; i++) {
        cudaEventDestroy(fmf::g_spans[i].a);
        cudaEventDestroy(fmf::g_spans[i].b);
    }
    fmf::g_nspans = 0;
    fmf::g_timing = true;
    return FMF_OK;
}

int fmf_timing_end_ex(double *ms, int n_kinds, int *n_calls)
{
    double acc[fmf::kSpanKinds] = {};
    int calls = 0, rc = FMF_OK;
    for (int i = 0; i < fmf::g_nspans; i++) {
        fmf::TimedSpan &sp = fmf::g_spans[i];
        float t = 0.0f;
        cudaError_t e = cudaEventSynchronize(sp.b);
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&t, sp.a, sp.b);
        if (e != cudaSuccess)
            rc = fmf::cuda_status(e, "fmf_timing_end");
        acc[sp.kind] += t;
        calls += sp.kind == fmf::kSpanKernel;
        cudaEventDestroy(sp.a);
        if (i + 1 >= fmf::g_nspans || fmf::g_spans[i + 1].a != sp.b)
            cudaEventDestroy(sp.b);
    }
    fmf::g_nspans = 0;
    fmf::g_timing = false;
    for (int k = 0; ms && k < n_kinds; k++)
        ms[k] = k < fmf::kSpanKinds ? acc[k] : 0.0;
    if (n_calls)
        *n_calls = calls;
    return rc;
}

int fmf_timing_end(double *prep_ms, double *kernel_ms, int *n_calls)
{
    double ms[2];
    const int rc = fmf_timing_end_ex(ms, 2, n_calls);
    if (prep_ms)
        *prep_ms = ms[0];
    if (kernel_ms)
        *kernel_ms = ms[1];
    return rc;
}

int fmf_last_precision(void) { return fmf::g_last_precision; }

int fmf_release_cache(void)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fmf::cuda_status(e, "fmf_release_cache");
    cudaMemPool_t pool;
    e = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemPoolTrimTo(pool, 0);
    return fmf::cuda_status(e, "fmf_release_cache");
}

}  // extern "C"
