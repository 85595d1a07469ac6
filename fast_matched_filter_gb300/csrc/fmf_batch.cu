// fmf_batch.cu -- many independent searches of uneven sizes in one graph.
//
// The reference runs one search per call (matched_filter.cu:171-399).  A
// batch records any number of searches (device pointers, each with its own
// T, S, C, L, N, step, normalisation and output layout) and runs them as one
// CUDA graph: every search's preprocessing kernels, then, for the tensor-core
// precisions, one persistent launch per normalisation and 64 searches over a
// shared tile queue (fmf_tc.cu), or, for FP32, the plain kernel per search.  The graph is
// captured on the first run (on a stream the batch owns, joined to the
// caller's stream with events) and replayed afterwards; its scratch lives in
// graph memory nodes.  The searches' preprocessing (and the FP32 searches)
// are captured on kBatchBranches forked streams, so they become concurrent
// branches of the graph: each is small and would leave most of the GPU idle
// if they ran one after another.  Inputs are read when the graph runs, so a
// batch can be re-run after its input buffers were refilled.
#include <cstring>
#include <memory>
#include <vector>

#include "fmf_common.cuh"

namespace fmf {
constexpr int kBatchBranches = 8;  // concurrent graph branches for the per-search work
}

struct fmf_batch {
    int precision = FMF_PREC_SPLIT_BF16;
    int tile = 0;      // forced lag blocks per tensor-core tile (0 = largest that fits)
    int group = 0;     // templates interleaved per group of tile-queue items (0 = default)
    int device = -1;
    std::vector<fmf::Args> searches;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    // fork/join of the capture: branch streams and their events
    cudaStream_t branch[fmf::kBatchBranches] = {};
    cudaEvent_t ev_fork = nullptr, ev_main = nullptr;
    cudaEvent_t ev_join[fmf::kBatchBranches] = {}, ev_rejoin[fmf::kBatchBranches] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;  // kernel launches in one replay
};

namespace fmf {

static int batch_record(fmf_batch *b, cudaStream_t s)
{
    int rc;
    cudaError_t e;
    Scratch ws(s);  // freed last, on s
    // fork: the branch streams join the capture
    if ((e = cudaEventRecord(b->ev_fork, s)) != cudaSuccess)
        return set_error(FMF_ERR_CUDA, "forking the batch capture: %s", cudaGetErrorString(e));
    for (int k = 0; k < kBatchBranches; k++)
        if ((e = cudaStreamWaitEvent(b->branch[k], b->ev_fork, 0)) != cudaSuccess)
            return set_error(FMF_ERR_CUDA, "forking the batch capture: %s", cudaGetErrorString(e));
    int status = FMF_OK;
    {
        std::vector<std::unique_ptr<Scratch>> bws;  // per-branch scratch, freed on its branch
        for (int k = 0; k < kBatchBranches; k++)
            bws.emplace_back(new Scratch(b->branch[k]));
        const size_t n = b->searches.size();
        std::vector<Problem> P(n);
        std::vector<const float *> dtc(n);
        const int split = b->precision == FMF_PREC_SPLIT_BF16;
        const bool tc = b->precision != FMF_PREC_FP32;
        std::vector<int> nb(n);
        const size_t psz = tc_prob_size();
        std::vector<unsigned char> probs(psz * n);
        for (size_t i = 0; i < n && status == FMF_OK; i++) {
            const int k = (int)(i % kBatchBranches);
            cudaStream_t si = b->branch[k];
            if ((status = prepare_problem(b->searches[i], *bws[k], si, &P[i], &dtc[i])))
                break;
            if (!tc) {
                status = launch_plain_all(P[i], si);
                continue;
            }
            nb[i] = tc_choose_nb(P[i].L, P[i].step, split, b->tile);
            if (nb[i] == 0) {
                status = set_error(FMF_ERR_SMEM, "search %zu: template length %d with step %d does not "
                                                 "fit a tensor-core tile", i, P[i].L, P[i].step);
                break;
            }
            status = tc_prepare(P[i], dtc[i], split, nb[i], b->group, *bws[k], si,
                                reinterpret_cast<TcProb *>(probs.data() + psz * i));
        }
        // join the branches, then the persistent launches on s
        for (int k = 0; k < kBatchBranches; k++)
            if ((e = cudaEventRecord(b->ev_join[k], b->branch[k])) != cudaSuccess ||
                (e = cudaStreamWaitEvent(s, b->ev_join[k], 0)) != cudaSuccess)
                status = status ? status : set_error(FMF_ERR_CUDA, "joining the batch capture: %s",
                                                     cudaGetErrorString(e));
        if (status == FMF_OK && tc) {
            unsigned *err = nullptr;
            if ((status = device_error_word(&err)) == FMF_OK) {
                // one persistent launch per normalisation (each runs the epilogue
                // instantiation of its own mode: a mixed launch carries both modes' code),
                // 64 searches at most per launch
                for (int norm = 0; norm < 2 && status == FMF_OK; norm++) {
                    std::vector<unsigned char> grp;
                    for (size_t i = 0; i < n; i++)
                        if (P[i].normalize == norm)
                            grp.insert(grp.end(), probs.begin() + psz * i, probs.begin() + psz * (i + 1));
                    const size_t ng = grp.size() / psz;
                    for (size_t i0 = 0; i0 < ng && status == FMF_OK; i0 += TC_MAX_PROBS) {
                        unsigned long long *queue = nullptr;
                        if ((status = ws.get(&queue, 1, "tile queue")))
                            break;
                        const int m = (int)(ng - i0 < (size_t)TC_MAX_PROBS ? ng - i0 : TC_MAX_PROBS);
                        status = tc_run(reinterpret_cast<const TcProb *>(grp.data() + psz * i0), m, split,
                                        queue, err, s);
                    }
                }
            }
        }
        // the branch scratch is freed after the work on s that reads it
        if ((e = cudaEventRecord(b->ev_main, s)) == cudaSuccess)
            for (int k = 0; k < kBatchBranches && e == cudaSuccess; k++)
                e = cudaStreamWaitEvent(b->branch[k], b->ev_main, 0);
        if (e != cudaSuccess && status == FMF_OK)
            status = set_error(FMF_ERR_CUDA, "ordering the batch scratch: %s", cudaGetErrorString(e));
    }  // branch scratch freed here, on the branch streams
    // rejoin the branches before the capture ends
    for (int k = 0; k < kBatchBranches; k++)
        if ((e = cudaEventRecord(b->ev_rejoin[k], b->branch[k])) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s, b->ev_rejoin[k], 0)) != cudaSuccess)
            status = status ? status : set_error(FMF_ERR_CUDA, "joining the batch capture: %s",
                                                 cudaGetErrorString(e));
    rc = status;
    return rc;
}

static void batch_reset_graph(fmf_batch *b)
{
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

}  // namespace fmf

extern "C" {

int fmf_batch_create(fmf_batch **out, int precision)
{
    fmf::set_error(FMF_OK, "");
    if (!out)
        return fmf::set_error(FMF_ERR_ARG, "null batch pointer");
    *out = nullptr;
    if (precision < FMF_PREC_FP32 || precision > FMF_PREC_BF16)
        return fmf::set_error(FMF_ERR_ARG, "unknown precision %d", precision);
    fmf_batch *b = new fmf_batch();
    b->precision = precision;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&b->ev_main, cudaEventDisableTiming);
    for (int k = 0; k < fmf::kBatchBranches && e == cudaSuccess; k++) {
        e = cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&b->ev_rejoin[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        fmf_batch_destroy(b);
        return fmf::set_error(FMF_ERR_CUDA, "creating a batch: %s", cudaGetErrorString(e));
    }
    *out = b;
    return FMF_OK;
}

int fmf_batch_set_tiles(fmf_batch *b, int lag_blocks, int template_group)
{
    fmf::set_error(FMF_OK, "");
    if (!b)
        return fmf::set_error(FMF_ERR_ARG, "null batch");
    if (lag_blocks != 0 && lag_blocks != 32 && lag_blocks != 64 && lag_blocks != 128)
        return fmf::set_error(FMF_ERR_ARG, "lag_blocks must be 0, 32, 64 or 128");
    if (template_group < 0 || template_group > 1024)
        return fmf::set_error(FMF_ERR_ARG, "template_group must be in [0, 1024]");
    b->tile = lag_blocks;
    b->group = template_group;
    fmf::batch_reset_graph(b);
    return FMF_OK;
}

int fmf_batch_add(fmf_batch *b, const float *templates, const float *sum_square_templates,
                  const int *moveouts, const float *data, const float *weights, size_t step,
                  size_t n_samples_template, size_t n_samples_data, size_t n_templates,
                  size_t n_stations, size_t n_components, size_t n_corr, float *cc_out,
                  int normalize, int sum_cc_mode)
{
    fmf::set_error(FMF_OK, "");
    if (!b)
        return fmf::set_error(FMF_ERR_ARG, "null batch");
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
    a.precision = b->precision;
    a.flags = FMF_FLAG_DEVICE_POINTERS;
    int rc = fmf::validate_args(a);
    if (rc)
        return rc;
    b->searches.push_back(a);
    fmf::batch_reset_graph(b);
    return FMF_OK;
}

int fmf_batch_run(fmf_batch *b, void *stream)
{
    fmf::set_error(FMF_OK, "");
    if (!b)
        return fmf::set_error(FMF_ERR_ARG, "null batch");
    if (b->searches.empty())
        return fmf::set_error(FMF_ERR_ARG, "empty batch");
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != b->device)
        return fmf::set_error(FMF_ERR_ARG, "batch created on device %d, current device is %d", b->device,
                              dev);
    cudaGetLastError();
    cudaStream_t user = (cudaStream_t)stream;
    cudaError_t e;
    if (!b->exec) {
        unsigned *err = nullptr;  // allocated outside the capture
        int rc = fmf::device_error_word(&err);
        if (rc)
            return rc;
        e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess)
            return fmf::set_error(FMF_ERR_CUDA, "beginning graph capture: %s", cudaGetErrorString(e));
        const int before = fmf_last_launch_count();
        rc = fmf::batch_record(b, b->stream);
        b->launches = fmf_last_launch_count() - before;
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->stream, &g);
        if (rc) {
            if (g)
                cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess)
            return fmf::set_error(FMF_ERR_CUDA, "ending graph capture: %s", cudaGetErrorString(e));
        b->graph = g;
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) {
            fmf::batch_reset_graph(b);
            return fmf::set_error(FMF_ERR_CUDA, "instantiating the batch graph: %s", cudaGetErrorString(e));
        }
    }
    if ((e = cudaEventRecord(b->ev_in, user)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(b->stream, b->ev_in, 0)) != cudaSuccess ||
        (e = cudaGraphLaunch(b->exec, b->stream)) != cudaSuccess ||
        (e = cudaEventRecord(b->ev_out, b->stream)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(user, b->ev_out, 0)) != cudaSuccess)
        return fmf::set_error(FMF_ERR_CUDA, "launching the batch graph: %s", cudaGetErrorString(e));
    return FMF_OK;
}

int fmf_batch_launch_count(const fmf_batch *b) { return b ? b->launches : 0; }

int fmf_batch_destroy(fmf_batch *b)
{
    if (!b)
        return FMF_OK;
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    fmf::batch_reset_graph(b);
    if (b->ev_in)
        cudaEventDestroy(b->ev_in);
    if (b->ev_out)
        cudaEventDestroy(b->ev_out);
    if (b->ev_fork)
        cudaEventDestroy(b->ev_fork);
    if (b->ev_main)
        cudaEventDestroy(b->ev_main);
    for (int k = 0; k < fmf::kBatchBranches; k++) {
        if (b->ev_join[k])
            cudaEventDestroy(b->ev_join[k]);
        if (b->ev_rejoin[k])
            cudaEventDestroy(b->ev_rejoin[k]);
        if (b->branch[k])
            cudaStreamDestroy(b->branch[k]);
    }
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
    return FMF_OK;
}

}  // extern "C"
