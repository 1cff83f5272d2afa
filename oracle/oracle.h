/*
 * oracle.h -- CPU restatement of the gpu_determ collision-integral path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle for the CUDA path in
 * gpu_determ_gb300/csrc: tests, the smoke check and the CPU-baseline leg of
 * bench.py load it; the product never links or calls it.
 *
 * Every function names the reference file:line it restates (paths inside the
 * savthe/gpu_determ project).  Arrays follow the reference layout
 * f[node][cell] with the cell index fastest; "box" node indices run over the
 * full nx*ny*nz lattice in (i, j, k) order, "compact" indices over the nodes
 * inside the velocity sphere in the same order (VelocityGrid's index lists).
 */
#ifndef GD_ORACLE_H
#define GD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_ERR 1.0e-10 /* velocity.h:37 */

/* ---- velocity grid (velocity_grid.cu:6-14, :73-126) ---------------------- */
int or_grid_count(int nx, int ny, int nz, const float *vmin, const float *vmax, float R);
/* u[nx], v[ny], w[nz] node centres; ui/vi/wi[n_pnt] compact index lists;
 * steps[4] = {d_u, d_v, d_w, d3v}. Returns n_pnt. */
int or_grid_fill(int nx, int ny, int nz, const float *vmin, const float *vmax, float R,
                 float *u, float *v, float *w, int *ui, int *vi, int *wi, float *steps);

/* ---- analytic hard-sphere weights (compute_matrix.cu:21-257, :505-562) --- */
float or_relative_speed(float du, float dv, float dw, int gi, int gj, int gk);
double or_box_sphere_area(double du, double dv, double dw, int in, int jn, int kn, double g);
/* b[nxyz] and a[(nx/2)*nx*(ny/2)*(nz/2)*ny*nz] in the reference layout */
void or_build_dense_tables(int nx, int ny, int nz, float du, float dv, float dw, float d3v,
                           float *b, float *a);

/* ---- context: grid + dense tables + per-|g| nonzero lists ---------------- */
typedef struct or_ctx or_ctx;
or_ctx *or_create(int nx, int ny, int nz, const float *vmin, const float *vmax, float R);
void or_destroy(or_ctx *c);
int or_n_pnt(const or_ctx *c);
const float *or_table_a(const or_ctx *c);
const float *or_table_b(const or_ctx *c);
const int *or_compact_of_box(const or_ctx *c);
/* counts of the work: nonzero weight entries, valid (i,i1,n) terms with the
 * output node in the sphere, sub-terms whose two nodes are both in the sphere */
void or_count_work(const or_ctx *c, int64_t *out3);
/* digest of the gain's index map (i, s = i + i1, n) over in-sphere outputs,
 * box partners, nonzero weights and in-box post-collision pairs:
 * {count, sum mix_a(key), xor mix_b(key), FP64 sum of the weights as bits} */
void or_index_map_digest(const or_ctx *c, uint64_t *out4);

/* ---- loss / gain on box-layout f (zero outside the sphere) -------------- */
/* FP64: nu[k][cell] = sum_j b(|i-j|) f[j][cell] for box node i = nodes[k]
 * (collision_integral.cu:32-72). */
void or_loss_f64(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 double *nu);
/* FP64 gain I[k][cell] for box node nodes[k] (collision_integral.cu:75-188). */
void or_gain_f64(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 double *gain);
/* FP32 gain with cell-innermost loops (the OpenMP host path timed as the CPU
 * baseline); same enumeration as or_gain_f64, FP32 arithmetic. */
void or_gain_f32(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 float *gain);
void or_loss_f32(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 float *nu);
/* Literal FP32 restatement in the reference's launch and loop order
 * (in1, jn1, kn1 outer; i1, j1, k1 inner), one cell column `cell` of a
 * [nxyz][npx] array; used to reproduce true_results.out. */
void or_loss_literal(const or_ctx *c, const float *f_box, int npx, int cell, const int *nodes,
                     int nn, float *nu);
void or_gain_literal(const or_ctx *c, const float *f_box, int npx, int cell, const int *nodes,
                     int nn, float *gain);

/* ---- conservation projection and relaxation (FP64) --------------------- */
/* Per cell, over the compact nodes: A_kl = sum f nu phi_k phi_l,
 * B_k = sum (I - f nu) phi_k, A X = B, nu' = nu (1 + X.phi), Q = I - f nu'
 * (collision_integral.cu:217-526, intended per-cell semantics).
 * f, nu, gain: [n_pnt][ncells]; outputs nu_corr (FP64), q (FP64), x[5*ncells].
 * Returns the number of cells whose 5x5 system was singular. */
int or_project(const or_ctx *c, const float *f, const float *nu, const float *gain, int ncells,
               double *nu_corr, double *q, double *x);
/* moments per cell: n, n*ux, n*uy, n*uz, energy (sum f phi_k d3v) */
void or_moments(const or_ctx *c, const double *f, int ncells, double *m5);

#ifdef __cplusplus
}
#endif
#endif
