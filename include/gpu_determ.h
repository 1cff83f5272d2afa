/*
 * gpu_determ.h -- C ABI of the GB300 collision-integral library.
 *
 * Deterministic discrete-velocity evaluation of the hard-sphere Boltzmann
 * collision integral Q(f) = I(f) - f nu(f) on a uniform 3-D velocity lattice
 * truncated to a sphere, batched over spatial cells, on one GPU (sm_103a).
 *
 * Conventions
 *  - Every function returns GD_OK (0) or a GD_ERR_* code; the message of the
 *    last failure on the calling host thread is gd_last_error().
 *  - Distribution arrays are device pointers laid out [node][cell]: node is the
 *    compact index over the in-sphere lattice nodes (the order of the grid's
 *    u/v/w index lists), cell is fastest, `ld` is the stride between nodes
 *    (ld >= ncells).  With R large enough to keep every node this is exactly
 *    the reference layout f[(i*ny + j)*nz + k][cell] with npx = ld.
 *  - Streams are cudaStream_t passed as gd_stream (NULL = legacy stream).
 *  - Results are bitwise reproducible run to run: floating-point sums run in
 *    a fixed order, and the one path that adds with atomics adds integers.
 *
 * Reference interfaces (savthe/gpu_determ) each entry point replaces are cited
 * as file:line.
 */
#ifndef GPU_DETERM_H
#define GPU_DETERM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *gd_stream;
typedef struct gd_ctx gd_ctx;

enum {
    GD_OK = 0,
    GD_ERR_INVALID_ARG = 1,  /* bad size, pointer or option */
    GD_ERR_CUDA = 2,         /* a CUDA runtime call or launch failed */
    GD_ERR_OUT_OF_MEMORY = 3,
    GD_ERR_UNSUPPORTED = 4,  /* grid or batch outside what the kernels support */
    GD_ERR_SINGULAR = 5,     /* a 5x5 conservation system had no solution */
    GD_ERR_IO = 6,           /* file could not be opened or parsed */
};

/* Velocity grid: nodes u_i = vmin + d (2i+1)/2 per axis, kept when
 * u^2+v^2+w^2 < R^2 (R <= 0 keeps all).  nx, ny, nz even.
 * Replaces VelocityGrid::init (velocity_grid.hpp:39-43, velocity_grid.cu:73-126)
 * and check_if_point_is_in_domain (velocity_grid.cu:6-14). */
typedef struct {
    int nx, ny, nz;
    float vmin[3], vmax[3];
    float R;
} gd_grid_spec;

typedef struct {
    int nx, ny, nz, n_pnt;
    float du, dv, dw, d3v;
    int64_t nonzero_weights;   /* nonzero entries of the weight table a */
    int64_t table_a_elems;     /* (nx/2)*nx*(ny/2)*(nz/2)*ny*nz, reference layout */
    int64_t pair_products;     /* (s, n) pair products formed per cell-eval */
    int64_t contraction_terms; /* nonzero-weight x pair-product terms per cell-eval */
    int64_t scatter_terms;     /* (s, g, sign) output updates per cell-eval */
    int64_t cmatrix_tiles;     /* stored 256 x 64 tiles of the collision matrices (0 without) */
    int64_t cmatrix_slices;    /* 256 x 16 slices with a nonzero entry over every node's matrix: the MMA
                                  K steps one cell tile issues in GD_CMATRIX_BF16X3 mode */
    int64_t cmatrix_node_tiles; /* tiles over every node's matrix (a node uses the stored tiles of its
                                   orbit's representative): what one BF16 pass issues per cell tile */
} gd_info;

/* Library version (major*10000 + minor*100 + patch). */
int gd_version(void);
/* Message of the last failure on this host thread ("" when none). */
const char *gd_last_error(void);

/* ---- host-side grid (no GPU needed) ------------------------------------ */
/* Number of in-sphere nodes.  Replaces the counting loop of
 * VelocityGrid::init (velocity_grid.cu:80-84). */
int gd_grid_count(const gd_grid_spec *spec, int *n_pnt);
/* Node centres u[nx], v[ny], w[nz]; index lists ui/vi/wi[n_pnt];
 * steps[4] = {du, dv, dw, d3v}.  Replaces VelocityGrid::init
 * (velocity_grid.cu:73-126) and its VelocityGridBase fields
 * (velocity_grid.hpp:6-31). */
int gd_grid_fill(const gd_grid_spec *spec, float *u, float *v, float *w, int *ui, int *vi,
                 int *wi, float *steps);

/* ---- options file ------------------------------------------------------ */
/* "key = value" lines with '#' comments; keys nx, ny, nz, npx (others are
 * ignored); nyz and nxyz derived.  GD_ERR_IO when the file cannot be opened
 * ("Can't open <path>"), GD_ERR_INVALID_ARG when a value is not an integer.
 * Replaces load_options (options.hpp:16, options.cu:34-53). */
typedef struct {
    int nx, ny, nz, nyz, nxyz, npx;
} gd_options;
int gd_load_options(const char *path, gd_options *out);

/* Caps the large device allocations of one object (collision matrices,
 * surrogate network) at `bytes` (0, the default: only the free device memory
 * limits them); creation beyond the cap fails with GD_ERR_OUT_OF_MEMORY and
 * changes nothing.  Process-wide. */
int gd_set_memory_limit(size_t bytes);

/* ---- context ----------------------------------------------------------- */
/* Binds to `device`, uploads the grid and builds the weight tables on the GPU
 * (FP64 analytic builder, compacted to nonzero entries).  Replaces the
 * device half of VelocityGrid (VelocityGrid::device, DeviceVelocityGrid,
 * velocity_grid.cu:21-48) and init_matrices (compute_matrix.h:13,
 * compute_matrix.cu:564-600). */
int gd_ctx_create(const gd_grid_spec *spec, int device, gd_ctx **out);
int gd_ctx_destroy(gd_ctx *ctx);
int gd_ctx_info(const gd_ctx *ctx, gd_info *out);

/* Dense tables in the reference layout: b[nx*ny*nz] (loss kernel
 * 4 pi |g| d3v) and a[table_a_elems] (post-collision weights), device
 * buffers owned by the caller; either may be NULL.  Replaces the table
 * contents of init_matrices (compute_matrix.cu:505-562). */
int gd_export_tables(gd_ctx *ctx, float *b, float *a, gd_stream stream);
/* 14 moment-basis rows over the full box [14][nx*ny*nz] (xi_x, xi_y, xi_z,
 * xi^2, xi_x^2, xi_x xi_y, xi_x xi_z, xi_x xi^2, xi_y^2, xi_y xi_z,
 * xi_y xi^2, xi_z^2, xi_z xi^2, xi^2 xi^2).  Replaces init_correction_array
 * (velocity.h:41, velocity.cu:17-65). */
int gd_correction_basis(gd_ctx *ctx, float *basis, gd_stream stream);

/* ---- collision operator ------------------------------------------------ */
/* Loss frequency nu[i][c] = sum_j b(|i-j|) f[j][c] and gain I[i][c] over the
 * in-sphere nodes (either output may be NULL), on the context's gain path:
 * GD_GAIN_PAIR computes both in FP32 (SIMT kernels); the tensor-core paths
 * (collision matrices, GD_GAIN_PAIR_TC) compute the gain on the tensor cores
 * and, when ld is a multiple of 4, the loss as one BF16x3 GEMM (see
 * gd_ctx_set_gain_path).  Replaces the
 * loss and gain stages of evolve_colisions (collision_integral.h:11-17,
 * collision_integral.cu:32-188, 587-648). */
int gd_collision(gd_ctx *ctx, const float *f, int ncells, int ld, float *nu, float *gain,
                 gd_stream stream);
/* FP64 mass/momentum/energy projection per cell: solves A X = B with
 * A_kl = sum f nu phi_k phi_l, B_k = sum (I - f nu) phi_k, phi = (1, xi, xi^2),
 * then nu' = nu (1 + X.phi) and Q = I - f nu' (so sum Q phi_k = 0).
 * nu_corr (FP32, may alias nu), q (FP64, may be NULL, leading dim ld) and
 * x[5*ncells] (FP64, may be NULL).  Replaces before_correction,
 * linear_solver and correct_frequency (collision_integral.cu:217-526,
 * 669-744) with the intended per-cell solve. */
int gd_project(gd_ctx *ctx, const float *f, const float *nu, const float *gain, int ncells,
               int ld, float *nu_corr, double *q, double *x, gd_stream stream);
/* Explicit relaxation f <- f + dt (I - f nu') with
 * mode GD_DT_COURANT: dt = param / max(nu') over all nodes and cells
 *                     (get_delta_t, collision_integral.cu:776-807);
 * mode GD_DT_FIXED:   dt = param.
 * time_dev (device float, may be NULL) is advanced by dt; dt_dev (device
 * float, may be NULL) receives dt.  Replaces relax_f and evolve_f
 * (collision_integral.h:19-24, collision_integral.cu:809-880). */
enum { GD_DT_COURANT = 0, GD_DT_FIXED = 1 };
int gd_relax(gd_ctx *ctx, float *f, const float *nu_corr, const float *gain, int ncells, int ld,
             int mode, float param, float *time_dev, float *dt_dev, gd_stream stream);
/* One full step: collision, projection and relaxation (FP64 Q), with the
 * per-cell moments (n, n u_x, n u_y, n u_z, sum f xi^2 d3v) of f before the
 * update in m5[5*ncells] (device FP64, may be NULL).  nu/gain/q receive the
 * step's corrected frequency, gain and Q (each may be NULL). */
int gd_step(gd_ctx *ctx, float *f, int ncells, int ld, int mode, float param, float *nu,
            float *gain, double *q, double *m5, float *time_dev, float *dt_dev, gd_stream stream);
/* Per-cell moments sum f phi_k d3v, phi = (1, xi_x, xi_y, xi_z, xi^2), FP64,
 * m5[5*ncells] on the device.  Restates print_moments (determ.cu:123-144)
 * per cell. */
int gd_moments(gd_ctx *ctx, const float *f, int ncells, int ld, double *m5, gd_stream stream);
/* Numeric health of the context's work since the last check: synchronises
 * the stream and returns GD_ERR_SINGULAR when a projection met a cell with
 * non-finite f, nu or gain sums or a singular 5x5 system (that cell's
 * frequency was left uncorrected; the message names the first such cell),
 * or GD_ERR_CUDA when a tensor-core pipeline wait of the context's gain or
 * loss kernels timed out (the message names every record that was set);
 * reads and clears all records.  The collision, projection and step calls
 * themselves never synchronise, on any gain path. */
int gd_ctx_check(gd_ctx *ctx, gd_stream stream);

/* ---- collision-matrix path (tensor cores) ------------------------------ */
/* The gain as the bilinear form I_i = sum_ab G_i[a][b] f_a f_b with the
 * collision matrices G_i assembled on the GPU from the analytic weights and
 * contracted on the tcgen05 tensor cores with FP32 accumulation.  G_i is
 * symmetric, so only the 256 x 64 tiles of its block upper triangle that hold
 * a nonzero entry are stored (off-diagonal entries doubled), and only for one
 * node per orbit of the lattice's reflections (x_a -> n_a - 1 - x_a on each
 * axis; the node set is symmetric since the sphere is centred in the box and
 * n_a is even): node R(i) uses G_i with f reflected by R.  At 20^3
 * (R = 4.8) that is ~5 GB in BF16, twice that for GD_CMATRIX_BF16X3 (8x less
 * than one matrix per node).  GD_CMATRIX_BF16 rounds f and G to BF16
 * (relative error ~3e-4 on I); GD_CMATRIX_BF16X3 splits both into BF16 hi +
 * lo parts and sums hi*hi + hi*lo + lo*hi (~4e-6).  With a context's gain
 * path set to either mode (or to GD_GAIN_PAIR_TC), its loss nu = B f also
 * runs on the tensor cores (B and f split into BF16 hi + lo, three products
 * per K step in one launch, ~5e-6) when ld is a multiple of 4.  No reference
 * counterpart: the reference forms these matrices only implicitly in its
 * gain loop (collision_integral.cu:75-188). */
typedef struct gd_cmatrix gd_cmatrix;
enum { GD_CMATRIX_BF16 = 0, GD_CMATRIX_BF16X3 = 1 };
int gd_cmatrix_create(gd_ctx *ctx, int mode, gd_cmatrix **out);
int gd_cmatrix_gain(gd_cmatrix *cm, const float *f, int ncells, int ld, float *gain, gd_stream stream);
int gd_cmatrix_destroy(gd_cmatrix *cm);
/* CTAs per tensor-core MMA of the gain kernel: 2 (the default) or 1.  With
 * 2, the CTAs of a node's two adjacent 128-cell tiles form a cluster and run
 * each MMA as a CTA pair (M = 256 cells): each loads its own cells and half
 * of every collision-matrix tile; a call with at most 128 cells runs one CTA
 * per MMA.  Results are bitwise the same either way. */
int gd_cmatrix_set_cluster(gd_cmatrix *cm, int ctas);
/* Longest run of stored tiles (an even count; 0 = unlimited) summed into
 * one tensor-memory accumulator before the epilogue folds it into the FP32
 * gain (compensated).  The tensor cores' FP32 accumulation loses precision
 * over long sums: at 20^3 the BF16x3 gain is 6.4e-7 from FP64 (median over
 * cells) with 4 tiles, 2.5e-6 unlimited.  Default: 4 in BF16x3 mode,
 * unlimited for one BF16 pass (whose error is the operands' rounding).  The
 * tensor-core loss always sums K in 256-column chunks, added in FP32 (one
 * chain over K carried a -1.2e-5 bias). */
int gd_cmatrix_set_chain(gd_cmatrix *cm, int tiles);
/* gd_cmatrix_gain only enqueues work on the stream.  Its kernels record a
 * pipeline time-out (a bounded wait that ran out) instead of hanging;
 * gd_cmatrix_check synchronises the stream, returns GD_ERR_CUDA when such a
 * record is set, and clears it (gd_ctx_check does the same for a context's
 * own matrices). */
int gd_cmatrix_check(gd_cmatrix *cm, gd_stream stream);
/* Gain algorithm used by gd_collision and gd_step for this context:
 * GD_GAIN_PAIR (default, FP32 pair-product kernel), GD_GAIN_CMATRIX_BF16 or
 * GD_GAIN_CMATRIX_BF16X3 (builds the context's collision matrices), or
 * GD_GAIN_PAIR_TC (the pair-product formulation with its weight contraction on
 * the tensor cores, pair products and weights split into BF16 hi + lo, each
 * cell's outputs summed in 64-bit fixed point scaled by a bound on its gain;
 * builds a per-class-box weight table of a few GB at 24^3 instead of n^3
 * matrices, so it serves the grids whose collision matrices do not fit).
 * The two pair paths need n_pnt * ld < 2^31 (GD_ERR_UNSUPPORTED otherwise). */
enum { GD_GAIN_PAIR = 0, GD_GAIN_CMATRIX_BF16 = 1, GD_GAIN_CMATRIX_BF16X3 = 2, GD_GAIN_PAIR_TC = 3 };
int gd_ctx_set_gain_path(gd_ctx *ctx, int path);

/* Layout conversion between the full box [nx*ny*nz][ld_box] of the reference
 * (determ.cu:107-120) and the compact in-sphere layout [n_pnt][ld]; nodes
 * outside the sphere come out as 0.  Needed only when R cuts the box. */
int gd_box_to_compact(gd_ctx *ctx, const float *box, int ncells, int ld_box, float *compact, int ld,
                      gd_stream stream);
int gd_compact_to_box(gd_ctx *ctx, const float *compact, int ncells, int ld, float *box, int ld_box,
                      gd_stream stream);

/* Gain I[i][c] exactly as gd_collision computes it on the FP32 pair kernel
 * (GD_GAIN_PAIR, whichever gain path the context has selected), but with no
 * device allocation of any kind during the call.  No counterpart in the reference:
 * it exists for callers that cannot let a library call cudaMalloc (a custom
 * allocator or memory pool owns the device, a latency-critical loop must not
 * hit cudaMalloc's implicit synchronisation, or allocation is forbidden after
 * start-up).  Its partial sums live in a fixed 64 MiB array inside the
 * library image, held on every GPU that loads the library until exit; a batch
 * needing more (about 4500 cells on a 20^3 grid cut to R=4.8) is rejected with
 * GD_ERR_UNSUPPORTED.  The result is bitwise equal to gd_collision's FP32
 * pair gain when the s-chunk count that call picks fits the array (at most
 * 64 chunks; then both sum in the same order); otherwise the array holds
 * fewer chunks and the sums, ordered differently, agree within FP32
 * rounding.  The first call on a device looks the array's address up, which
 * may also load the library's device code on that device and so reserve the
 * 64 MiB there (the CUDA driver's allocation, not a cudaMalloc): a caller that
 * wants no allocation at all inside its hot loop makes one warm-up call at
 * start-up, before any stream capture.  All calls share the array: calls
 * that overlap on the GPU race, so order them. */
int gd_gain_noalloc(gd_ctx *ctx, const float *f, int ncells, int ld, float *gain, gd_stream stream);

/* ---- batches of grids, CUDA graphs, autotuning --------------------------- */
/* A batch steps several (context, cells) groups together: groups on distinct
 * contexts run concurrently on their own streams, groups on one context in
 * order.  gd_batch_step performs one gd_step (collision, FP64 projection,
 * relaxation; moments into m5 when given) for every group.  Its first call
 * runs eagerly and sizes every buffer; with use_graph each later call replays
 * one CUDA graph captured on the second call (one cudaGraphLaunch per step).
 * Adding a group drops the graph.  Steps are ordered after earlier work on
 * `stream`, and later work on `stream` after them.  Steps never synchronise;
 * gd_batch_check (synchronising) runs gd_ctx_check on every group's context
 * and returns the first error.  No reference counterpart: the reference steps one
 * grid, one batch of npx <= 1024 cells, from a host loop (determ.cu:62-80). */
typedef struct gd_batch gd_batch;
int gd_batch_create(gd_batch **out);
int gd_batch_destroy(gd_batch *b);
int gd_batch_add(gd_batch *b, gd_ctx *ctx, float *f, int ncells, int ld, int mode, float param, double *m5,
                 float *time_dev, float *dt_dev);
int gd_batch_step(gd_batch *b, int use_graph, gd_stream stream);
/* GD_BATCH_STREAMS (default): each group's gd_step on its context's stream,
 * as above.  GD_BATCH_FUSED_PAIR_TC: the gains of all groups (at most 4, on
 * distinct contexts whose gain path is GD_GAIN_PAIR_TC) in one persistent
 * launch of the pair-product kernel that walks a device list of (grid,
 * 128-cell tile, s-chunk) units, each group's loss, projection and
 * relaxation around it on the batch stream; results equal gd_step on each
 * group's context bit for bit.  A pipeline time-out of the fused launch is
 * recorded on the first group's context.  GD_BATCH_FUSED_CMATRIX: the same
 * with the gains of all groups (at most 4, on distinct contexts whose gain
 * path is the same collision-matrix mode) in one launch of the
 * collision-matrix kernel over every grid's (cell tile, node) pairs; results
 * equal gd_step bit for bit, time-outs are recorded per context. */
enum { GD_BATCH_STREAMS = 0, GD_BATCH_FUSED_PAIR_TC = 1, GD_BATCH_FUSED_CMATRIX = 2 };
int gd_batch_set_mode(gd_batch *b, int mode);
int gd_batch_check(gd_batch *b);
int gd_batch_info(const gd_batch *b, int *groups, int *streams, int *graph_nodes, int64_t *steps);

/* Times the gain candidates of a context on the given cells and keeps the
 * fastest (gain path, and for the pair kernel the minimum CTAs per SM of its
 * s-chunk split).  path_mask: bits (1 << GD_GAIN_*) that may be chosen; the
 * collision-matrix paths only when their stored tiles (at most every 256 x 64
 * tile of each G_i's block upper triangle, 2 bytes per entry in BF16, 4 in
 * BF16X3) fit mem_budget bytes, GD_GAIN_PAIR_TC only when its weight table
 * does.  Allocates a gain buffer for
 * the duration of the call.  Candidates that run out of memory are skipped
 * (cand_ms = -1). */
#define GD_AUTOTUNE_MAX 8
typedef struct {
    int path, waves;  /* chosen gain path; pair kernel: minimum CTAs per SM */
    float best_ms;
    int n_candidates;
    int cand_path[GD_AUTOTUNE_MAX], cand_waves[GD_AUTOTUNE_MAX];
    float cand_ms[GD_AUTOTUNE_MAX];
    int cluster;      /* collision matrices: CTAs per cluster (1 or 2) */
    int cand_cluster[GD_AUTOTUNE_MAX];
} gd_autotune_result;
int gd_ctx_autotune(gd_ctx *ctx, const float *f, int ncells, int ld, int path_mask, double mem_budget,
                    gd_autotune_result *res, gd_stream stream);

/* ---- learned surrogate ---------------------------------------------------- */
/* A small network trained on (f, Q(f)) pairs of the plain method, with BF16
 * weights, FP32 accumulation and every product on the tcgen05 tensor cores:
 *   h0 = W0 x + b0 (n_in -> 256), h1 = GELU(W1 h0 + b1) (-> 512),
 *   h2 = GELU(W2 h1 + b2) (-> 512), z = W3 h2 + b3 + h0 (-> 256),
 *   y = W4 z + b4 (-> n_out).
 * x and y use the library layout [feature][cell] with stride ld.
 * GD_MLP_SCALE_INPUT divides each cell's x by its mean over the n_in
 * features; GD_MLP_SCALE_OUTPUT multiplies y by the square of that mean (Q is
 * quadratic in f).  Training minimises the mean over the batch of
 * sum_i (y_i - t_i)^2 / den, den = sum_i tden_i^2 (tden defaults to t;
 * scaled like y), den = the batch mean of that sum with GD_MLP_LOSS_BATCH, or
 * den = n_out with GD_MLP_LOSS_MSE, with Adam (beta 0.9, 0.999, eps 1e-8,
 * decoupled weight decay).  Global gains (gd_mlp_set_io_scale, default 1)
 * multiply the scaled input before the first layer and the network output
 * before the per-cell output scaling, so the weights work on O(1) values.
 * No reference counterpart. */
typedef struct gd_mlp gd_mlp;
enum { GD_MLP_SCALE_INPUT = 1, GD_MLP_SCALE_OUTPUT = 2, GD_MLP_LOSS_MSE = 4, GD_MLP_LOSS_BATCH = 8 };
typedef struct {
    int n_in, n_out, n_in_padded, n_out_padded, batch_cap, flags;
    int64_t steps, num_params;
    double forward_flop_per_cell;
    float in_gain, out_gain;
} gd_mlp_info_t;
/* batch_cap: largest batch, a multiple of 64.  Weights ~ U(-1/sqrt(fan_in),
 * 1/sqrt(fan_in)) from a 64-bit LCG seeded by seed, biases 0. */
int gd_mlp_create(int n_in, int n_out, int batch_cap, int flags, uint64_t seed, gd_mlp **out);
int gd_mlp_destroy(gd_mlp *mlp);
int gd_mlp_set_io_scale(gd_mlp *mlp, float in_gain, float out_gain);
int gd_mlp_info(const gd_mlp *mlp, gd_mlp_info_t *info);
/* y[n_out][ldy] = net(x[n_in][ldx]) for batch cells (1 <= batch <= cap). */
int gd_mlp_forward(gd_mlp *mlp, const float *x, int ldx, int batch, float *y, int ldy, gd_stream stream);
/* One Adam step on batch cells (a multiple of 64); *loss (device, may be
 * NULL) receives the batch's mean loss before the update. */
int gd_mlp_train_step(gd_mlp *mlp, const float *x, int ldx, const float *t, int ldt, const float *tden, int ldd,
                      int batch, float lr, float weight_decay, float *loss, gd_stream stream);
/* Per-cell loss row_loss[batch] (device) without an update. */
int gd_mlp_loss(gd_mlp *mlp, const float *x, int ldx, const float *t, int ldt, const float *tden, int ldd, int batch,
                float *row_loss, gd_stream stream);
/* Synchronises the stream and reports a tensor-core pipeline time-out. */
int gd_mlp_check(gd_mlp *mlp, gd_stream stream);
/* FP32 host block of num_params floats: W_k [out][in] then b_k [out] for
 * k = 0..4, n_in and n_out padded to multiples of 64 (pads are zero).
 * gd_mlp_get_grads gives the gradients of the last training step. */
int gd_mlp_get_params(gd_mlp *mlp, float *host);
int gd_mlp_set_params(gd_mlp *mlp, const float *host);
int gd_mlp_get_grads(gd_mlp *mlp, float *host);

/* Surrogate gain with plain-method fallback.  net maps f (n_pnt) to Q
 * (n_pnt); est (may be NULL) maps f to an estimate of log10 of the relative
 * L2 error of the surrogate's Q for that cell.  gd_surrogate_gain writes the
 * exact loss frequency nu, and the gain I = net(f) + nu f for every cell
 * whose estimate is <= log10(tol); every other cell (all of them when
 * tol <= 0, none when est is NULL and tol > 0) gets the plain gain of the
 * context's gain path.  *n_fallback receives that count; est_out (device,
 * ncells, may be NULL) the estimates.  The call synchronises the stream once
 * (the fallback count sizes the plain launch).  Follow with gd_project for
 * the FP64 conservation projection, exactly as after gd_collision.  All
 * buffers are allocated by gd_surrogate_create for max_cells cells; nothing
 * is allocated per call.  No reference counterpart. */
typedef struct gd_surrogate gd_surrogate;
int gd_surrogate_create(gd_ctx *ctx, gd_mlp *net, gd_mlp *est, int max_cells, gd_surrogate **out);
int gd_surrogate_destroy(gd_surrogate *s);
int gd_surrogate_gain(gd_surrogate *s, const float *f, int ncells, int ld, float tol, float *nu, float *gain,
                      float *est_out, int *n_fallback, gd_stream stream);
/* out[c] = ||a[:,c] - b[:,c]||_2 / ||b[:,c]||_2 over n rows (FP64). */
int gd_cell_rel_l2(const double *a, int lda, const double *b, int ldb, int n, int ncells, double *out,
                   gd_stream stream);

/* The pair-product formulation's tables exactly as the gain kernels read
 * them, copied to host buffers, for checks of the gain's index map against
 * an independent enumeration of the reference's (i, i1, n) -> (l, l1) map
 * (collision_integral.cu:88-94, 115-131, 154-155).  sizes is always filled;
 * each array may be NULL (then it is not written).
 *   grp_row_off[n_groups + 1]  entries of group m: [grp_row_off[m], grp_row_off[m+1])
 *   entry_class[n_entries], entry_w[n_entries]: class-box index
 *     (x2 * hy + y2) * hz + z2 of the offset n (n_a = 2 a2 + parity of the
 *     pair sum) and the FP32 weight (rows padded with w = 0 to multiples of 8)
 *   item_off[nx*ny*nz + 1]: work items of D (box-indexed, D_a = min(s_a,
 *     2 n_a - 2 - s_a)): [item_off[D], item_off[D+1])
 *   items[3 * n_items]: {group, first member, end member} per item
 *   members[n_members]: member g as x2 | y2 << 6 | z2 << 12 (g_a = 2 a2 +
 *     parity), the members of the group that lie in B(D)
 * gd_pair_tc_table copies the per-D weight table of GD_GAIN_PAIR_TC (built
 * when that path is selected, else GD_ERR_UNSUPPORTED): *rows rows of 64
 * BF16 (hi and lo parts, raw bits), wrow[nx*ny*nz] the first row of each D;
 * row wrow[D] + chunk * pad16(items of D) + item holds the item's weights at
 * the box's class offsets (x2 * ey + y2) * ez + z2 = chunk * 64 + column.
 * No reference counterpart (the reference has only the dense table a). */
typedef struct {
    int n_groups, nclass;
    int64_t n_entries, n_items, n_members;
} gd_pair_table_sizes;
int gd_pair_tables(gd_ctx *ctx, gd_pair_table_sizes *sizes, int *grp_row_off, int *entry_class, float *entry_w,
                   int *item_off, int *items, uint32_t *members);
int gd_pair_tc_table(gd_ctx *ctx, int64_t *rows, int *wrow, uint16_t *wh, uint16_t *wl);

/* Failure-detection test hooks (host-side injection; nothing faults).  The
 * next launch of the named tensor-core GEMM makes every CTA wait `polls`
 * polls (1..2^20) on an mbarrier that nothing arrives at, before it has
 * issued any copy or MMA.  That bounded wait runs out, the CTA records the
 * time-out, frees its tensor memory and returns; later kernels of the same
 * object see the record and skip their work.  The record is reported and
 * cleared by gd_mlp_check (for gd_mlp_inject_timeout: the first GEMM of the
 * next forward pass or training step) or gd_ctx_check (for
 * gd_ctx_inject_timeout: the first GEMM of the next tensor-core loss of a
 * context on a collision-matrix gain path, else GD_ERR_UNSUPPORTED).  The
 * call after that computes normally.  No reference counterpart: the
 * reference has no failure handling (collision_integral.cu:601,622). */
int gd_mlp_inject_timeout(gd_mlp *net, int polls);
int gd_ctx_inject_timeout(gd_ctx *ctx, int polls);

/* Measured fused multiply-add throughput of `device` in FLOP/s (2 per FMA),
 * precision 32 (FP32 FFMA) or 64 (FP64 DFMA): the roofline denominator of the
 * SIMT kernels.  Synchronous; allocates a few bytes.  No reference
 * counterpart (the reference only times whole phases, gputimer.hpp:10-46). */
int gd_fma_peak(int device, int precision, double *flops_per_s);

#ifdef __cplusplus
}
#endif
#endif
