// gd_surrogate.cu -- collision gain from the learned surrogate with the plain
// method as fallback.
//
// Per call: the loss frequency nu is computed exactly (loss kernel); an error
// network predicts log10 of each cell's relative L2 error; cells whose
// estimate exceeds log10(tol) (or is not finite) are compacted in ascending
// order.  When every cell falls back, the context's plain gain runs in place
// and the network is not evaluated.  Otherwise the network predicts Q for
// every cell, giving the gain I = Q + nu f, and the fallback cells' f is
// gathered into a dense block, their gain recomputed by the context's plain
// gain path and scattered back.  The caller then applies the
// FP64 conservation projection (gd_project) as for the plain method, so every
// cell's Q conserves mass, momentum and energy whichever path produced it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "gd_internal.h"

namespace gd {
namespace {

// gain[i][c] += nu[i][c] * f[i][c]
__global__ void add_loss_kernel(float *__restrict__ gain, const float *__restrict__ nu, const float *__restrict__ f,
                                int n, int ncells, int ld)
{
    const int64_t total = (int64_t)n * ncells;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / ncells), c = (int)(t % ncells);
        const size_t o = (size_t)i * ld + c;
        gain[o] = gain[o] + nu[o] * f[o];
    }
}

// One block of 1024 threads: idx[0..count) = cells with !(est <= thr) in
// ascending order (all cells when est is null and thr is -inf, none when est
// is null otherwise); *count written last.
__global__ void select_kernel(const float *__restrict__ est, int ncells, float thr, int all,
                              int *__restrict__ idx, int *__restrict__ count)
{
    __shared__ int warp_sum[32];
    __shared__ int base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int c0 = 0; c0 < ncells; c0 += blockDim.x) {
        const int c = c0 + threadIdx.x;
        int flag = 0;
        if (c < ncells) flag = all ? 1 : (est ? !(est[c] <= thr) : 0);
        const unsigned bal = __ballot_sync(0xffffffffu, flag);
        const int in_warp = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_sum[warp] = __popc(bal);
        __syncthreads();
        if (warp == 0) {
            int v = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0;
            // inclusive scan over the warps' counts
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            warp_sum[lane] = v;
        }
        __syncthreads();
        const int before = (warp ? warp_sum[warp - 1] : 0);
        if (flag) idx[base + before + in_warp] = c;
        __syncthreads();
        if (threadIdx.x == 0) base += warp_sum[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = base;
}

// dst[i][k] = src[i][idx[k]], k < count (dst stride ldd)
__global__ void gather_cells_kernel(const float *__restrict__ src, int ld, const int *__restrict__ idx, int count,
                                    int n, float *__restrict__ dst, int ldd)
{
    const int64_t total = (int64_t)n * count;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / count), k = (int)(t % count);
        dst[(size_t)i * ldd + k] = src[(size_t)i * ld + idx[k]];
    }
}

// dst[i][idx[k]] = src[i][k]
__global__ void scatter_cells_kernel(const float *__restrict__ src, int lds, const int *__restrict__ idx, int count,
                                     int n, float *__restrict__ dst, int ld)
{
    const int64_t total = (int64_t)n * count;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / count), k = (int)(t % count);
        dst[(size_t)i * ld + idx[k]] = src[(size_t)i * lds + k];
    }
}

// out[c] = ||a[:, c] - b[:, c]|| / ||b[:, c]|| in FP64, thread per cell
// (coalesced over cells), nodes summed in order.
__global__ void cell_rel_l2_kernel(const double *__restrict__ a, int lda, const double *__restrict__ b, int ldb, int n,
                                   int ncells, double *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n; i++) {
        const double bv = b[(size_t)i * ldb + c], d = a[(size_t)i * lda + c] - bv;
        num += d * d;
        den += bv * bv;
    }
    out[c] = den > 0.0 ? sqrt(num / den) : (num > 0.0 ? INFINITY : 0.0);
}

int grid_for(int64_t total) { return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 16)); }

}  // namespace
}  // namespace gd

struct gd_surrogate {
    gd_ctx *ctx = nullptr;
    gd_mlp *net = nullptr, *est = nullptr;
    int device = 0, n = 0, cap = 0;
    float *est_buf = nullptr, *fs = nullptr, *gs = nullptr;
    int *idx = nullptr, *d_count = nullptr, *h_count = nullptr;
};

namespace {

void free_surrogate(gd_surrogate *s)
{
    gd::DeviceGuard ds(s->device);
    cudaFree(s->est_buf);
    cudaFree(s->fs);
    cudaFree(s->gs);
    cudaFree(s->idx);
    cudaFree(s->d_count);
    if (s->h_count) cudaFreeHost(s->h_count);
    delete s;
}

}  // namespace

extern "C" int gd_surrogate_create(gd_ctx *ctx, gd_mlp *net, gd_mlp *est, int max_cells, gd_surrogate **out)
{
    using namespace gd;
    if (!ctx || !net || !out) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    gd_info ci;
    int rc = gd_ctx_info(ctx, &ci);
    if (rc) return rc;
    gd_mlp_info_t ni, ei;
    if ((rc = gd_mlp_info(net, &ni))) return rc;
    if (ni.n_in != ci.n_pnt || ni.n_out != ci.n_pnt)
        return set_error(GD_ERR_INVALID_ARG, "the network must map n_pnt inputs to n_pnt outputs");
    if (max_cells < 1 || max_cells > ni.batch_cap)
        return set_error(GD_ERR_INVALID_ARG, "max_cells must be in [1, network batch_cap]");
    if (est) {
        if ((rc = gd_mlp_info(est, &ei))) return rc;
        if (ei.n_in != ci.n_pnt || ei.n_out != 1 || max_cells > ei.batch_cap)
            return set_error(GD_ERR_INVALID_ARG, "the error network must map n_pnt inputs to 1 output, cap >= max_cells");
    }
    gd_surrogate *s = new gd_surrogate();
    s->ctx = ctx;
    s->net = net;
    s->est = est;
    s->n = ci.n_pnt;
    s->cap = max_cells;
    s->device = ctx->c.device;
    gd::DeviceGuard dg(s->device);
    const size_t blk = (size_t)s->n * max_cells * sizeof(float);
    if (cudaMalloc(&s->est_buf, (size_t)max_cells * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&s->idx, (size_t)max_cells * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&s->d_count, sizeof(int)) != cudaSuccess || cudaMalloc(&s->fs, blk) != cudaSuccess ||
        cudaMalloc(&s->gs, blk) != cudaSuccess || cudaMallocHost(&s->h_count, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        free_surrogate(s);
        return set_error(GD_ERR_OUT_OF_MEMORY, "surrogate buffers");
    }
    *out = s;
    return GD_OK;
}

extern "C" int gd_surrogate_destroy(gd_surrogate *s)
{
    if (s) free_surrogate(s);
    return GD_OK;
}

extern "C" int gd_surrogate_gain(gd_surrogate *s, const float *f, int ncells, int ld, float tol, float *nu,
                                 float *gain, float *est_out, int *n_fallback, gd_stream stream)
{
    using namespace gd;
    if (!s || !f || !nu || !gain) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ncells < 1 || ncells > s->cap || ld < ncells)
        return set_error(GD_ERR_INVALID_ARG, "need 1 <= ncells <= max_cells and ld >= ncells");
    if (std::isnan(tol)) return set_error(GD_ERR_INVALID_ARG, "tolerance is NaN");
    gd::DeviceGuard ds(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc;
    if (tol <= 0.f) {  // the plain method for every cell
        if ((rc = gd_collision(s->ctx, f, ncells, ld, nu, gain, stream))) return rc;
        if (n_fallback) *n_fallback = ncells;
        return GD_OK;
    }
    // the exact loss, then the error estimate decides which cells take the
    // plain gain; the network runs only when some cell keeps its output
    if ((rc = gd_collision(s->ctx, f, ncells, ld, nu, nullptr, stream))) return rc;
    if (s->est && (rc = gd_mlp_forward(s->est, f, ld, ncells, s->est_buf, ncells, stream))) return rc;
    select_kernel<<<1, 1024, 0, st>>>(s->est ? s->est_buf : nullptr, ncells, std::log10(tol), 0, s->idx, s->d_count);
    GD_CUDA(cudaGetLastError());
    GD_CUDA(cudaMemcpyAsync(s->h_count, s->d_count, sizeof(int), cudaMemcpyDeviceToHost, st));
    GD_CUDA(cudaStreamSynchronize(st));
    if (s->est && (rc = gd_mlp_check(s->est, stream))) return rc;
    const int count = *s->h_count;
    if (count == ncells) {
        // every cell falls back: the plain gain straight into place (the same
        // launch as gathering all cells in order would make)
        if ((rc = gd_collision(s->ctx, f, ncells, ld, nullptr, gain, stream))) return rc;
    } else {
        if ((rc = gd_mlp_forward(s->net, f, ld, ncells, gain, ld, stream))) return rc;
        add_loss_kernel<<<grid_for((int64_t)s->n * ncells), 256, 0, st>>>(gain, nu, f, s->n, ncells, ld);
        GD_CUDA(cudaGetLastError());
        if (count > 0) {
            const int64_t tot = (int64_t)s->n * count;
            gather_cells_kernel<<<grid_for(tot), 256, 0, st>>>(f, ld, s->idx, count, s->n, s->fs, count);
            GD_CUDA(cudaGetLastError());
            if ((rc = gd_collision(s->ctx, s->fs, count, count, nullptr, s->gs, stream))) return rc;
            scatter_cells_kernel<<<grid_for(tot), 256, 0, st>>>(s->gs, count, s->idx, count, s->n, gain, ld);
            GD_CUDA(cudaGetLastError());
        }
        if ((rc = gd_mlp_check(s->net, stream))) return rc;  // synchronises the stream
    }
    if (est_out) {
        if (s->est)
            GD_CUDA(cudaMemcpyAsync(est_out, s->est_buf, (size_t)ncells * sizeof(float), cudaMemcpyDeviceToDevice, st));
        else
            GD_CUDA(cudaMemsetAsync(est_out, 0, (size_t)ncells * sizeof(float), st));
    }
    if (n_fallback) *n_fallback = count;
    return GD_OK;
}

extern "C" int gd_cell_rel_l2(const double *a, int lda, const double *b, int ldb, int n, int ncells, double *out,
                              gd_stream stream)
{
    using namespace gd;
    if (!a || !b || !out || n < 1 || ncells < 1 || lda < ncells || ldb < ncells)
        return set_error(GD_ERR_INVALID_ARG, "bad relative-L2 arguments");
    cell_rel_l2_kernel<<<(ncells + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a, lda, b, ldb, n, ncells, out);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}
