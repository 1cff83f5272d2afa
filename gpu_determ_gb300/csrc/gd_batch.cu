// gd_batch.cu -- several velocity grids stepped together as one CUDA graph,
// and the per-context launch autotuner.
//
// A batch is a list of groups (context, cells).  One gd_batch_step runs
// gd_step for every group: groups on different contexts run concurrently on
// their own streams (forked from and joined back into the batch's stream);
// groups sharing a context run in order on one stream, since a context's
// scratch serves one launch at a time.  In the fused mode every group's gain
// is instead one persistent launch of the pair-product kernel over a device
// list of (grid, cell tile, s-chunk) units of all groups.  The first step runs
// eagerly (it sizes every buffer and uploads every launch table); with
// use_graph the second step captures the whole sequence into a CUDA graph and
// every later step is one cudaGraphLaunch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gd_internal.h"

struct gd_batch {
    struct Group {
        gd_ctx *ctx;
        float *f;
        int ncells, ld, mode;
        float param;
        double *m5;
        float *time_dev, *dt_dev;
        int slot;
    };
    std::vector<Group> groups;
    std::vector<gd_ctx *> slot_ctx;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> done;
    cudaStream_t main = nullptr;
    cudaEvent_t fork = nullptr, joined = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = 0;
    int64_t steps = 0;
    int mode = GD_BATCH_STREAMS;
};

namespace {

void drop_graph(gd_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// every group's step on its slot stream, forked from and joined into main
int enqueue_steps(gd_batch *b)
{
    GD_CUDA(cudaEventRecord(b->fork, b->main));
    for (size_t s = 0; s < b->streams.size(); s++) GD_CUDA(cudaStreamWaitEvent(b->streams[s], b->fork, 0));
    for (const gd_batch::Group &g : b->groups) {
        int rc = gd_step(g.ctx, g.f, g.ncells, g.ld, g.mode, g.param, nullptr, nullptr, nullptr, g.m5, g.time_dev,
                         g.dt_dev, (gd_stream)b->streams[g.slot]);
        if (rc) return rc;
    }
    for (size_t s = 0; s < b->streams.size(); s++) {
        GD_CUDA(cudaEventRecord(b->done[s], b->streams[s]));
        GD_CUDA(cudaStreamWaitEvent(b->main, b->done[s], 0));
    }
    return GD_OK;
}

// The fused modes: every group's loss, then ONE launch of the gain for all
// groups (GD_BATCH_FUSED_PAIR_TC: the persistent pair-product kernel with its
// contraction on the tensor cores; GD_BATCH_FUSED_CMATRIX: the collision-
// matrix kernel over every grid's nodes), then every group's projection and
// relaxation, all on the batch stream.  Each group's results equal gd_step on
// its context's gain path bit for bit (the same per-unit work: integer sums
// on the pair path, the same CTA pairs on the matrix path).
int enqueue_fused(gd_batch *b)
{
    using namespace gd;
    const size_t ng = b->groups.size();
    std::vector<float *> nu(ng), gain(ng);
    std::vector<double *> q(ng);
    std::vector<PtJob> jobs(ng);
    std::vector<CmJob> cjobs(ng);
    for (size_t k = 0; k < ng; k++) {
        const gd_batch::Group &g = b->groups[k];
        Context &c = g.ctx->c;
        nu[k] = gain[k] = nullptr;
        q[k] = nullptr;
        int rc = step_buffers(c, g.ld, b->main, &nu[k], &gain[k], &q[k]);
        if (!rc) rc = run_loss_path(c, g.f, g.ncells, g.ld, nu[k], b->main);
        if (rc) return rc;
        jobs[k] = PtJob{&c, g.f, g.ncells, g.ld, gain[k]};
        cjobs[k] = CmJob{c.cmatrix, g.f, g.ncells, g.ld, gain[k]};
    }
    int rc = b->mode == GD_BATCH_FUSED_CMATRIX ? launch_cmatrix(cjobs.data(), (int)ng, b->main)
                                               : launch_pair_tc(jobs.data(), (int)ng, b->main);
    if (rc) return rc;
    for (size_t k = 0; k < ng; k++) {
        const gd_batch::Group &g = b->groups[k];
        Context &c = g.ctx->c;
        rc = run_project(c, g.f, nu[k], gain[k], g.ncells, g.ld, nu[k], q[k], nullptr, 0, 0.f, nullptr, g.m5, b->main);
        if (!rc)
            rc = run_relax_q(c, g.f, nu[k], gain[k], q[k], g.ncells, g.ld, g.mode, g.param, g.time_dev, g.dt_dev,
                             b->main);
        if (rc) return rc;
    }
    return GD_OK;
}

int check_fused(const gd_batch *b, int mode)
{
    using namespace gd;
    if (b->groups.size() > 4) return set_error(GD_ERR_UNSUPPORTED, "fused batch: at most 4 groups");
    for (size_t k = 0; k < b->groups.size(); k++) {
        const Context &c = b->groups[k].ctx->c;
        if (mode == GD_BATCH_FUSED_PAIR_TC && (c.gain_path != GD_GAIN_PAIR_TC || !c.pair_tc))
            return set_error(GD_ERR_UNSUPPORTED, "fused batch: every group's context needs gain path GD_GAIN_PAIR_TC");
        if (mode == GD_BATCH_FUSED_CMATRIX &&
            (c.gain_path != b->groups[0].ctx->c.gain_path || !c.cmatrix ||
             (c.gain_path != GD_GAIN_CMATRIX_BF16 && c.gain_path != GD_GAIN_CMATRIX_BF16X3)))
            return set_error(GD_ERR_UNSUPPORTED,
                             "fused batch: every group's context needs the same collision-matrix gain path");
        for (size_t j = 0; j < k; j++)
            if (b->groups[j].ctx == b->groups[k].ctx)
                return set_error(GD_ERR_UNSUPPORTED, "fused batch: one group per context");
    }
    return GD_OK;
}

}  // namespace

extern "C" int gd_batch_set_mode(gd_batch *b, int mode)
{
    using namespace gd;
    if (!b) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (mode != GD_BATCH_STREAMS && mode != GD_BATCH_FUSED_PAIR_TC && mode != GD_BATCH_FUSED_CMATRIX)
        return set_error(GD_ERR_INVALID_ARG, "unknown batch mode");
    if (mode != GD_BATCH_STREAMS) {
        const int rc = check_fused(b, mode);
        if (rc) return rc;
    }
    b->mode = mode;
    drop_graph(b);
    return GD_OK;
}

extern "C" int gd_batch_create(gd_batch **out)
{
    using namespace gd;
    if (!out) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gd_batch *b = new gd_batch();
    cudaGetDevice(&b->device);
    if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->joined, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return set_error(GD_ERR_CUDA, "batch streams");
    }
    *out = b;
    return GD_OK;
}

extern "C" int gd_batch_destroy(gd_batch *b)
{
    if (!b) return GD_OK;
    gd::DeviceGuard ds(b->device);
    cudaStreamSynchronize(b->main);
    drop_graph(b);
    for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->done) cudaEventDestroy(e);
    cudaEventDestroy(b->fork);
    cudaEventDestroy(b->joined);
    cudaStreamDestroy(b->main);
    delete b;
    return GD_OK;
}

extern "C" int gd_batch_add(gd_batch *b, gd_ctx *ctx, float *f, int ncells, int ld, int mode, float param, double *m5,
                            float *time_dev, float *dt_dev)
{
    using namespace gd;
    if (!b || !ctx || !f) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ncells < 1 || ld < ncells) return set_error(GD_ERR_INVALID_ARG, "need 1 <= ncells <= ld");
    if (mode != GD_DT_COURANT && mode != GD_DT_FIXED) return set_error(GD_ERR_INVALID_ARG, "unknown dt mode");
    if (!(param > 0.f) || !std::isfinite(param)) return set_error(GD_ERR_INVALID_ARG, "dt parameter must be > 0");
    if (ctx->c.device != b->device) return set_error(GD_ERR_INVALID_ARG, "context on another device");
    gd::DeviceGuard ds(b->device);
    int slot = -1;
    for (size_t s = 0; s < b->slot_ctx.size(); s++)
        if (b->slot_ctx[s] == ctx) slot = (int)s;
    if (slot < 0) {
        cudaStream_t st;
        cudaEvent_t ev;
        GD_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaStreamDestroy(st);
            return set_error(GD_ERR_CUDA, "batch event");
        }
        slot = (int)b->streams.size();
        b->streams.push_back(st);
        b->done.push_back(ev);
        b->slot_ctx.push_back(ctx);
    }
    b->groups.push_back({ctx, f, ncells, ld, mode, param, m5, time_dev, dt_dev, slot});
    drop_graph(b);
    return (int)GD_OK;
}

extern "C" int gd_batch_step(gd_batch *b, int use_graph, gd_stream stream)
{
    using namespace gd;
    if (!b) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (b->groups.empty()) return set_error(GD_ERR_INVALID_ARG, "empty batch");
    gd::DeviceGuard ds(b->device);
    cudaStream_t user = (cudaStream_t)stream;
    // order after the caller's stream, and the caller's stream after the step
    GD_CUDA(cudaEventRecord(b->joined, user));
    GD_CUDA(cudaStreamWaitEvent(b->main, b->joined, 0));
    int rc = GD_OK;
    if (b->mode != GD_BATCH_STREAMS && (rc = check_fused(b, b->mode))) return rc;
    auto enqueue = [&]() { return b->mode != GD_BATCH_STREAMS ? enqueue_fused(b) : enqueue_steps(b); };
    if (!use_graph || b->steps == 0) {
        rc = enqueue();
    } else {
        if (!b->exec) {
            GD_CUDA(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeRelaxed));
            rc = enqueue();
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(b->main, &g);
            if (!rc && e != cudaSuccess) rc = cuda_error(e, "batch graph capture");
            if (rc) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return rc;
            }
            b->graph = g;
            e = cudaGraphInstantiate(&b->exec, b->graph, 0);
            if (e != cudaSuccess) {
                drop_graph(b);
                return cuda_error(e, "batch graph instantiation");
            }
        }
        GD_CUDA(cudaGraphLaunch(b->exec, b->main));
    }
    if (rc) return rc;
    GD_CUDA(cudaEventRecord(b->joined, b->main));
    GD_CUDA(cudaStreamWaitEvent(user, b->joined, 0));
    b->steps++;
    return GD_OK;
}

extern "C" int gd_batch_check(gd_batch *b)
{
    using namespace gd;
    if (!b) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    gd::DeviceGuard ds(b->device);
    GD_CUDA(cudaStreamSynchronize(b->main));
    // every context's records (projection status, tensor-core time-outs),
    // each read and cleared by gd_ctx_check
    int first = GD_OK;
    for (gd_ctx *c : b->slot_ctx) {
        const int rc = gd_ctx_check(c, nullptr);
        if (rc && first == GD_OK) first = rc;
    }
    return first;
}

extern "C" int gd_batch_info(const gd_batch *b, int *groups, int *streams, int *graph_nodes, int64_t *steps)
{
    using namespace gd;
    if (!b) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (groups) *groups = (int)b->groups.size();
    if (streams) *streams = (int)b->streams.size();
    if (graph_nodes) {
        size_t n = 0;
        if (b->graph) GD_CUDA(cudaGraphGetNodes(b->graph, nullptr, &n));
        *graph_nodes = (int)n;
    }
    if (steps) *steps = b->steps;
    return GD_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: times the gain launch candidates of one context on the caller's
// cells and keeps the fastest.  Candidates: the FP32 pair kernel with 1, 2 or
// 4 CTAs per SM as the minimum s-chunk fill (trading partial-sum traffic for
// parallelism), the pair formulation with its contraction on the tensor cores
// (when its per-class-box weight table fits the memory budget), and the
// tensor-core collision matrices in BF16x3 and BF16 mode, each with 1 or 2
// CTAs per MMA (2: CTA-pair MMA, M = 256 cells), when the caller's mask admits
// them and their stored triangle tiles (bounded by every tile of the block
// upper triangle) fit the memory budget.  Each candidate: one untimed run,
// then the median of three runs timed with CUDA events on the stream.

extern "C" int gd_ctx_autotune(gd_ctx *ctx, const float *f, int ncells, int ld, int path_mask, double mem_budget,
                               gd_autotune_result *res, gd_stream stream)
{
    using namespace gd;
    if (!ctx || !f || !res) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ncells < 1 || ld < ncells) return set_error(GD_ERR_INVALID_ARG, "need 1 <= ncells <= ld");
    if (!(path_mask & 15)) return set_error(GD_ERR_INVALID_ARG, "path_mask admits no gain path");
    Context &c = ctx->c;
    gd::DeviceGuard ds(c.device);
    cudaStream_t st = (cudaStream_t)stream;
    std::memset(res, 0, sizeof(*res));
    struct Cand {
        int path, waves, cluster;
    };
    std::vector<Cand> cands;
    if (path_mask & (1 << GD_GAIN_PAIR))
        for (int w : {1, 2, 4}) cands.push_back({GD_GAIN_PAIR, w, 1});
    if ((path_mask & (1 << GD_GAIN_PAIR_TC)) && pair_tc_bytes(c) <= mem_budget)
        cands.push_back({GD_GAIN_PAIR_TC, 0, 1});
    if ((path_mask & (1 << GD_GAIN_CMATRIX_BF16X3)) && cmatrix_bytes_bound(c, GD_CMATRIX_BF16X3) <= mem_budget)
        for (int cl : {1, 2}) cands.push_back({GD_GAIN_CMATRIX_BF16X3, 0, cl});
    if ((path_mask & (1 << GD_GAIN_CMATRIX_BF16)) && cmatrix_bytes_bound(c, GD_CMATRIX_BF16) <= mem_budget)
        for (int cl : {1, 2}) cands.push_back({GD_GAIN_CMATRIX_BF16, 0, cl});
    if (cands.empty()) return set_error(GD_ERR_UNSUPPORTED, "no gain path fits the memory budget");
    if (cands.size() > GD_AUTOTUNE_MAX) cands.resize(GD_AUTOTUNE_MAX);
    float *gain = nullptr;
    GD_CUDA(cudaMalloc(&gain, sizeof(float) * (size_t)c.d.n_pnt * ld));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int saved_path = c.gain_path, saved_waves = c.gain_waves;
    int rc = GD_OK;
    float best = INFINITY;
    int best_i = -1;
    for (size_t i = 0; i < cands.size() && !rc; i++) {
        res->cand_path[i] = cands[i].path;
        res->cand_waves[i] = cands[i].waves;
        res->cand_cluster[i] = cands[i].cluster;
        res->cand_ms[i] = -1.f;
        int r = gd_ctx_set_gain_path(ctx, cands[i].path);
        if (r == GD_ERR_OUT_OF_MEMORY) {  // this candidate does not fit: skip it
            cudaGetLastError();
            continue;
        }
        if (r) {
            rc = r;
            break;
        }
        if (cands[i].waves) c.gain_waves = cands[i].waves;
        if (c.cmatrix && (r = gd_cmatrix_set_cluster(c.cmatrix, cands[i].cluster))) {
            rc = r;
            break;
        }
        float t[3];
        for (int k = -1; k < 3 && !rc; k++) {
            cudaEventRecord(e0, st);
            rc = run_gain_path(c, f, ncells, ld, gain, st);
            cudaEventRecord(e1, st);
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(GD_ERR_CUDA, "autotune timing");
            if (!rc && k >= 0) cudaEventElapsedTime(&t[k], e0, e1);
        }
        if (rc) break;
        std::sort(t, t + 3);
        res->cand_ms[i] = t[1];
        if (t[1] < best) {
            best = t[1];
            best_i = (int)i;
        }
    }
    res->n_candidates = (int)cands.size();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(gain);
    if (rc || best_i < 0) {
        c.gain_waves = saved_waves;
        gd_ctx_set_gain_path(ctx, saved_path);
        return rc ? rc : set_error(GD_ERR_UNSUPPORTED, "no gain candidate could run");
    }
    if ((rc = gd_ctx_set_gain_path(ctx, cands[best_i].path))) return rc;
    if (c.cmatrix && (rc = gd_cmatrix_set_cluster(c.cmatrix, cands[best_i].cluster))) return rc;
    c.gain_waves = cands[best_i].waves ? cands[best_i].waves : saved_waves;
    res->path = cands[best_i].path;
    res->waves = c.gain_waves;
    res->cluster = cands[best_i].cluster;
    res->best_ms = best;
    return GD_OK;
}
