// gd_internal.h -- shared declarations of the GB300 collision-integral library.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <map>
#include <vector>

#include "gpu_determ.h"

namespace gd {

struct PairTc;

// Lattice sizes derived from a grid spec.  The "class box" of a parity
// class is the set of offsets v with 0 <= v_a < n_a and v_a of one parity per
// axis; it has hx*hy*hz members, indexed (x2*hy + y2)*hz + z2 with v_a = 2*v2_a +
// parity_a.
struct Dims {
    int nx, ny, nz, nyz, nxyz;
    int hx, hy, hz, nclass;  // half sizes and class-box size
    int sx, sy, sz;          // extents of the pair sums s = i + i1: 2n - 1
    int64_t ns;              // sx*sy*sz
    int n_pnt;
    float du, dv, dw, d3v;
};

// One nonzero post-collision weight of the row |g|: off is the byte offset
// of n's pair product in the gain kernel's shared P_s array (class index of
// n times the kernel's cell block times 4), w the FP32 weight.
struct WEntry {
    uint32_t off;
    float w;
};
static_assert(sizeof(WEntry) == 8, "WEntry must be 8 bytes");

// Half components (x2, y2, z2) in 6-bit fields whose bit 5 is a guard bit:
// "x2 <= Dx2 and y2 <= Dy2 and z2 <= Dz2" is
// ((half_bound(Dx2, Dy2, Dz2) - half_pack(x2, y2, z2)) & kHalfGuard) == kHalfGuard.
constexpr uint32_t kHalfGuard = (1u << 5) | (1u << 11) | (1u << 17);
__host__ __device__ inline uint32_t half_pack(int x2, int y2, int z2)
{
    return (uint32_t)x2 | ((uint32_t)y2 << 6) | ((uint32_t)z2 << 12);
}
__host__ __device__ inline uint32_t half_bound(int dx2, int dy2, int dz2)
{
    return half_pack(dx2, dy2, dz2) | kHalfGuard;
}

struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// Floats of a context's reduction buffer (block maxima of nu', then dt).
constexpr int kReduceFloats = 2048;

struct Context {
    gd_grid_spec spec{};
    Dims d{};
    int device = 0;
    // host copies of the grid
    std::vector<float> u, v, w;
    std::vector<int> ui, vi, wi;
    std::vector<int> cmap;  // box index -> compact index or -1
    // device tables
    int16_t *d_cmap = nullptr;    // [nxyz] box -> compact, -1 outside the sphere
    uint32_t *d_nodes = nullptr;  // [n_pnt] packed box coords x | y << 10 | z << 20
    float *d_b = nullptr;         // [nxyz] loss kernel by |g|
    double *d_phi = nullptr;      // [5][n_pnt] basis 1, xi_x, xi_y, xi_z, xi^2 (FP64)
    int *d_list_off = nullptr;    // [nxyz + 1] weight-row offsets by |g| box index
    WEntry *d_list = nullptr;     // nonzero weights, rows in box order of |g|
    int64_t n_entries = 0;
    // Rows that are bitwise identical (same parity class, same |g|) form one
    // group; the gain kernel contracts a group once and scatters the result to
    // every member g.  Groups are ordered by parity class.
    int n_groups = 0;
    int class_grp_off[9] = {};      // group range of each parity class
    int *d_grp_row_off = nullptr;   // [n_groups + 1] into d_grp_rows
    WEntry *d_grp_rows = nullptr;   // one row per group
    int *d_grp_mem_off = nullptr;   // [n_groups + 1] into d_grp_members
    uint32_t *d_grp_members = nullptr;  // member g as guarded half components x2 | y2 << 6 | z2 << 12
    int64_t n_grp_entries = 0;
    // Work items per D = (Dx, Dy, Dz) (box-indexed like g): the row groups with
    // a member in B(D), each with the list of its members that lie in B(D).
    int *d_D_item_off = nullptr;   // [nxyz + 1] into d_D_items
    int4 *d_D_items = nullptr;     // {group, member begin, member end, 0}
    uint32_t *d_D_members = nullptr;  // member g as half_pack(x2, y2, z2)
    std::vector<int> h_grp_row_off, h_grp_mem_off;
    std::vector<uint32_t> h_grp_members;
    std::vector<WEntry> h_grp_rows;
    // pair-sum schedule for the gain kernel: work-balanced chunk boundaries
    std::vector<int64_t> s_work_prefix;  // [ns + 1] cumulative work in linear s order
    // counts reported by gd_ctx_info
    int64_t pair_products = 0, contraction_terms = 0, scatter_terms = 0;
    int gain_path = GD_GAIN_PAIR;    // gain algorithm for gd_collision / gd_step
    gd_cmatrix *cmatrix = nullptr;   // collision matrices when gain_path is a GD_GAIN_CMATRIX_*
    PairTc *pair_tc = nullptr;       // per-D weight table when gain_path is GD_GAIN_PAIR_TC
    int gain_cb = 32;                // cells per lane row of the gain kernel (fixed per grid)
    bool gain_cmap_smem = true;      // its box -> compact map in shared memory (else through L1)
    size_t gain_smem = 0;            // its dynamic shared memory
    // scratch owned by the context (grown on demand)
    Scratch scratch;
    Scratch step_buf;  // gd_step's nu, gain (FP32) and Q (FP64) when the caller passes none
    // chunk boundaries on the device per chunk count, uploaded once (a
    // replayed CUDA graph reads them without any host copy)
    std::map<int, int *> s_bounds_dev;
    // work-unit lists of pair tensor-core launches led by this context, per
    // launch shape (device array, count), uploaded once
    std::map<std::string, std::pair<int4 *, int>> pt_units_dev;
    int gain_waves = 2;         // gain launch: at least this many CTAs per SM (autotuned)
    float *d_reduce = nullptr;  // [kReduceFloats]: block maxima of nu', then dt
    unsigned int *d_status = nullptr;  // numeric status of projections: flags, first failing cell
    int sm_count = 0;
};

// Makes an object's device current for the duration of a call and restores
// the caller's device afterwards.
struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Limit on the large device allocations of one object (collision matrices,
// surrogate network), 0 = only the free device memory (gd_set_memory_limit).
size_t memory_limit();

// error state -------------------------------------------------------------
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);
#define GD_CUDA(call)                                        \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return gd::cuda_error(e_, #call); \
    } while (0)

// grid (host, gd_grid.cpp) -------------------------------------------------
int grid_count(const gd_grid_spec &s);
int grid_fill(const gd_grid_spec &s, float *u, float *v, float *w, int *ui, int *vi, int *wi,
              float *steps);

// device table builders (gd_weights.cu) ------------------------------------
// Dense reference-layout tables: b[nxyz] and/or a[(nx/2)*nx*(ny/2)*(nz/2)*ny*nz].
int launch_dense_tables(const Dims &d, float *b, float *a, cudaStream_t st);
// Compact the dense table a into per-|g| rows (device), returns entries.
int build_weight_rows(Context &c, const float *a_dense, cudaStream_t st);

// kernels -------------------------------------------------------------------
int run_loss(Context &c, const float *f, int ncells, int ld, float *nu, cudaStream_t st);
int run_gain(Context &c, const float *f, int ncells, int ld, float *gain, cudaStream_t st);
// gain by the context's selected path
int run_gain_path(Context &c, const float *f, int ncells, int ld, float *gain, cudaStream_t st);
int run_project(Context &c, const float *f, const float *nu, const float *gain, int ncells,
                int ld, float *nu_corr, double *q, double *x, int fixed_dt_mode, float dt,
                float *f_out, double *m5, cudaStream_t st);
int run_relax(Context &c, float *f, const float *nu_corr, const float *gain, int ncells, int ld,
              int mode, float param, float *time_dev, float *dt_dev, cudaStream_t st);
int run_relax_q(Context &c, float *f, const float *nu_corr, const float *gain, const double *q,
                int ncells, int ld, int mode, float param, float *time_dev, float *dt_dev,
                cudaStream_t st);
int run_moments(Context &c, const float *f, int ncells, int ld, double *m5, cudaStream_t st);
int run_basis(Context &c, float *basis, cudaStream_t st);

// group identical weight rows (gd_capi.cu)
int build_row_groups(Context &c);

// gain kernel shape for this grid: cells per lane row and shared memory (gd_gain.cu)
int gain_plan_cells(Context &c);
// gain launch pieces for a caller-provided partial buffer (gd_gain.cu)
int gain_launch_shape(Context &c, int ncells, int *cb, size_t *smem, int *nblk, int *chunks);
void gain_chunk_bounds(const Context &c, int nchunks, int *bounds);
int launch_gain_pair(Context &c, const float *f, int ncells, int ld, float *gain, float *part,
                     int nchunks, const int *d_bounds, int cb, size_t smem, cudaStream_t st);

// device copy of the work-balanced s-chunk boundaries for nchunks chunks
// (built once per count, gd_gain.cu)
int gain_bounds_device(Context &c, int nchunks, const int **out);
// gain[node][c] = sum over chunks of part[chunk][node][c], in chunk order
int reduce_gain_partials(Context &c, const float *part, int nchunks, int cells_pad, int ncells, int ld,
                         float *gain, cudaStream_t st);

// pair-product gain with the contraction on the tensor cores (gd_pair_tc.cu)
int pair_tc_build(Context &c);
void pair_tc_free(Context &c);
double pair_tc_bytes(const Context &c);
int run_pair_tc(Context &c, const float *f, int ncells, int ld, float *gain, cudaStream_t st);
// several grids' pair tensor-core gains in one persistent launch (1-4 jobs on
// distinct contexts with built tables); results equal separate launches bit
// for bit
struct PtJob {
    Context *c;
    const float *f;
    int ncells, ld;
    float *gain;
};
int launch_pair_tc(const PtJob *jobs, int njobs, cudaStream_t st);
// the collision-matrix gain of 1-4 grids (one gd_cmatrix each, one mode) in
// one launch (gd_cmatrix.cu); results equal separate launches bit for bit
struct CmJob {
    gd_cmatrix *cm;
    const float *f;
    int ncells, ld;
    float *gain;
};
int launch_cmatrix(const CmJob *jobs, int njobs, cudaStream_t st);
// reads (synchronising st) and clears the pipeline time-out record of the
// pair tensor-core kernel; *timed_out receives whether it was set
int pair_tc_take_timeout(Context &c, cudaStream_t st, bool *timed_out);
// the same for a context's collision matrices (gd_cmatrix.cu)
int cmatrix_take_timeout(gd_cmatrix *cm, cudaStream_t st, bool *timed_out);

// BF16 tiled tensor map with 128-byte swizzle for the TMA loads of the
// tensor-core kernels (gd_cmatrix.cu)
int encode_bf16_sw128(CUtensorMap *m, void *ptr, int rank, const uint64_t *dims, const uint64_t *strides,
                      const uint32_t *box);

// scratch -------------------------------------------------------------------
int ensure_scratch(Context &c, size_t bytes);
// gd_step's nu / gain / Q buffers for the ones passed as NULL (gd_capi.cu)
int step_buffers(Context &c, int ld, cudaStream_t st, float **nu, float **gain, double **q);

// tensor-core GEMM (gd_mlp.cu), one launch: C[M][N] = A_hi B_hi^T + A_hi B_lo^T
// + A_lo B_hi^T, A [M][K] and B [N][K] K-major BF16 (K a multiple of 64), C
// FP32 with ldc % 4 == 0 and 16-byte aligned rows.  The tensor cores sum at
// most k_chunk (a multiple of 64) products per FP32 accumulation; the chunks
// are added in FP32, in chunk order.  stall_polls > 0 is the
// failure-detection test hook of gd_ctx_inject_timeout (every CTA's bounded
// wait on a barrier nothing arrives at runs out).
int gemm_bf16x3_nt_f32(const void *Ah, const void *Al, int M, const void *Bh, const void *Bl, int N, int K, float *C,
                       int ldc, int *err, cudaStream_t st, int stall_polls, int k_chunk);
// loss on the tensor cores when the context uses collision matrices
// (gd_cmatrix.cu); GD_ERR_UNSUPPORTED when the layout does not allow it.
int cmatrix_loss(gd_cmatrix *cm, const float *f, int ncells, int ld, float *nu, cudaStream_t st);
// the loss matrix alone, for contexts on the pair path with its contraction on
// the tensor cores (gd_cmatrix.cu)
int cmatrix_create_loss_only(gd_ctx *ctx, gd_cmatrix **out);
// loss for the context's gain path: tensor cores with collision matrices (when
// the layout allows), else the FP32 kernel
int run_loss_path(Context &c, const float *f, int ncells, int ld, float *nu, cudaStream_t st);
// stored tiles of a context's collision matrices (0 for NULL)
int64_t cmatrix_stored_tiles(const gd_cmatrix *cm);
int64_t cmatrix_issued_slices(const gd_cmatrix *cm);
int64_t cmatrix_node_tiles(const gd_cmatrix *cm);
// upper bound of the collision matrices' bytes (every triangle tile stored)
double cmatrix_bytes_bound(const Context &c, int mode);

}  // namespace gd

// the opaque handle of the C ABI
struct gd_ctx {
    gd::Context c;
};
