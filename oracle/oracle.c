/*
 * oracle.c -- CPU restatement of the gpu_determ collision-integral path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA kernels are tested against, and
 * the timed OpenMP host baseline.  Nothing in the product links it.
 *
 * Built with -ffp-contract=off so that float and double expressions round
 * exactly as written (the reference's host code is compiled that way on
 * x86-64, and the GPU weight builder is compiled with -fmad=false to match).
 * Citations are file:line inside the savthe/gpu_determ sources.
 */
#define _USE_MATH_DEFINES
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_PI_2
#define M_PI_2 1.57079632679489661923
#endif

/* ------------------------------------------------------------------------ */
/* Velocity grid                                                             */
/* ------------------------------------------------------------------------ */

/* Sphere membership of box node (i, j, k): velocity_grid.cu:6-14.  The
 * centre is formed as (extent * (2i+1-n)) in float, then divided by 2 and by
 * n in double and rounded back to float; the test u^2+v^2+w^2 < R^2 is in
 * float.  R <= 0 keeps every node. */
static int node_in_sphere(int nx, int ny, int nz, const float *vmin, const float *vmax, int i,
                          int j, int k, float R)
{
    float tu = (vmax[0] - vmin[0]) * (float)(2 * i + 1 - nx);
    float tv = (vmax[1] - vmin[1]) * (float)(2 * j + 1 - ny);
    float tw = (vmax[2] - vmin[2]) * (float)(2 * k + 1 - nz);
    float u = (float)((double)tu / 2. / (double)nx);
    float v = (float)((double)tv / 2. / (double)ny);
    float w = (float)((double)tw / 2. / (double)nz);
    if (R <= 0) return 1;
    float r2 = u * u;
    r2 = r2 + v * v;
    r2 = r2 + w * w;
    return r2 < R * R;
}

int or_grid_count(int nx, int ny, int nz, const float *vmin, const float *vmax, float R)
{
    int n = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) n += node_in_sphere(nx, ny, nz, vmin, vmax, i, j, k, R);
    return n;
}

/* VelocityGrid::init, velocity_grid.cu:73-126: steps d = (max-min)/n in
 * float, d3v = du*dv*dw, centres min + d*(2i+1)/2 evaluated in double. */
int or_grid_fill(int nx, int ny, int nz, const float *vmin, const float *vmax, float R,
                 float *u, float *v, float *w, int *ui, int *vi, int *wi, float *steps)
{
    float du = (vmax[0] - vmin[0]) / (float)nx;
    float dv = (vmax[1] - vmin[1]) / (float)ny;
    float dw = (vmax[2] - vmin[2]) / (float)nz;
    float d3v = du * dv;
    d3v = d3v * dw;
    for (int i = 0; i < nx; i++) u[i] = (float)((double)vmin[0] + (double)du * (2. * i + 1.) / 2.);
    for (int i = 0; i < ny; i++) v[i] = (float)((double)vmin[1] + (double)dv * (2. * i + 1.) / 2.);
    for (int i = 0; i < nz; i++) w[i] = (float)((double)vmin[2] + (double)dw * (2. * i + 1.) / 2.);
    int n = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++)
                if (node_in_sphere(nx, ny, nz, vmin, vmax, i, j, k, R)) {
                    ui[n] = i;
                    vi[n] = j;
                    wi[n] = k;
                    n++;
                }
    steps[0] = du;
    steps[1] = dv;
    steps[2] = dw;
    steps[3] = d3v;
    return n;
}

/* ------------------------------------------------------------------------ */
/* Analytic hard-sphere weights                                              */
/* ------------------------------------------------------------------------ */

/* |g| for lattice offset (gi, gj, gk): compute_matrix.cu:517,524-527,549-553.
 * Components in float, squared sum in float, float square root. */
float or_relative_speed(float du, float dv, float dw, int gi, int gj, int gk)
{
    float gu = du * (float)gi, gv = dv * (float)gj, gw = dw * (float)gk;
    float s = gu * gu;
    s = s + gv * gv;
    s = s + gw * gw;
    return sqrtf(s);
}

/*
 * Antiderivatives, in the normalised height p, of the four azimuth bounds a
 * box face imposes on a circle of latitude of the unit sphere (the circle has
 * radius rho = sqrt(1 - p^2); area element dphi dp):
 *   kind 1: phi <= acos(A/rho)  (face u >= u_lo)   compute_matrix.cu:21-42
 *   kind 2: phi >= acos(A/rho)  (face u <= u_hi)   compute_matrix.cu:45-64
 *   kind 3: phi >= asin(A/rho)  (face v >= v_lo)   compute_matrix.cu:67-86
 *   kind 4: phi <= asin(A/rho)  (face v <= v_hi)   compute_matrix.cu:89-108
 * The closed form of the acos bound is p atan(s/A) + A atan(s/p) + atan(Ap/s)
 * with s = sqrt(1 - A^2 - p^2); the asin bound is pi/2 p minus it.  The
 * degenerate cases (A, p or 1-A^2-p^2 within 1e-10 of zero, A near 1) take
 * the limits the reference takes, in the same order, because those guards
 * decide which weights come out exactly zero.
 */
static double azimuth_primitive(int kind, double p, double A)
{
    const double q = 1. - A * A - p * p;
    const int p_small = (p < OR_ERR) && (p > -OR_ERR);
    const int q_small = (q < OR_ERR) && (q > -OR_ERR);
    const int q_regular = (q >= OR_ERR) && (p >= OR_ERR);
    if (kind == 1 || kind == 2) {
        if (kind == 1 && (A < OR_ERR) && (A > -OR_ERR)) return M_PI_2 * p;
        if (kind == 2 && A > (1 - OR_ERR)) return 0.;
        if (p_small) return M_PI_2 * A;
        if (q_small) return M_PI_2;
        if (q_regular && (kind == 2 || A >= OR_ERR)) {
            const double s = sqrt(q);
            return p * atan(s / A) + A * atan(s / p) + atan(A * p / s);
        }
        return 0.;
    }
    if (kind == 3 && A < OR_ERR) return 0.;
    if (kind == 4 && A > (1. - OR_ERR)) return M_PI_2 * p;
    if (p_small) return -M_PI_2 * A;
    if (q_small) return M_PI_2 * (p - 1.);
    if (q_regular) {
        const double s = sqrt(q);
        return M_PI_2 * p - p * atan(s / A) - A * atan(s / p) - atan(A * p / s);
    }
    return 0.;
}

/*
 * Area of the sphere |x| = g that lies in the box
 * [du(in-1), du(in+1)] x [dv(jn-1), dv(jn+1)] x [dw(kn-1), dw(kn+1)]
 * (the lower face clamped at 0 on the n = 0 layer), divided by g^2:
 * compute_matrix.cu:110-257.
 *
 * The area is the integral over the height z/g of the azimuth interval the
 * four side faces leave open.  Sorting the heights h0 <= {h1, h3} <= h2 at
 * which the sphere crosses the four vertical box edges, each bound is active
 * on one fixed height range:
 *   v <= v_hi on [h0, h1],  u >= u_lo on [h1, h2]   (upper bounds, added)
 *   u <= u_hi on [h0, h3],  v >= v_lo on [h3, h2]   (lower bounds, subtracted)
 * and each contributes F(end) - F(start) over the part of its range inside
 * [z_lo, z_hi].  Terms are accumulated left to right in the order
 * (v<=v_hi, u>=u_lo, u<=u_hi, v>=v_lo), which reproduces the reference's
 * case tree term for term.
 */
double or_box_sphere_area(double du, double dv, double dw, int in, int jn, int kn, double g)
{
    const double u_lo = in > 0 ? du * (in - 1) : 0., u_hi = du * (in + 1);
    const double v_lo = jn > 0 ? dv * (jn - 1) : 0., v_hi = dv * (jn + 1);
    const double w_lo = kn > 0 ? dw * (kn - 1) : 0., w_hi = dw * (kn + 1);
    const double g2 = g * g;
    const double uu_lo = u_lo * u_lo, uu_hi = u_hi * u_hi;
    const double vv_lo = v_lo * v_lo, vv_hi = v_hi * v_hi;
    const double ww_lo = w_lo * w_lo, ww_hi = w_hi * w_hi;

    /* the sphere must pass between the nearest and the farthest box corner */
    if (!(uu_lo + vv_lo + ww_lo < g2 && uu_hi + vv_hi + ww_hi > g2)) return 0.;
    /* azimuth window of the (u >= u_lo, v >= v_lo) quadrant at the equator */
    const double phi_max = in > 1 ? atan(sqrt(g2 / uu_lo - 1.)) : M_PI_2;
    const double phi_min = jn > 1 ? M_PI_2 - atan(sqrt(g2 / vv_lo - 1.)) : 0;
    if (!(phi_max > phi_min)) return 0.;

    /* edge crossing heights: corners (u_hi,v_hi), (u_lo,v_hi), (u_lo,v_lo), (u_hi,v_lo) */
    const double r2[4] = {uu_hi + vv_hi, uu_lo + vv_hi, uu_lo + vv_lo, uu_hi + vv_lo};
    double h[4];
    for (int e = 0; e < 4; e++) {
        const double t = 1. - r2[e] / g2;
        h[e] = t < 0 ? 0. : sqrt(t);
    }
    const double z_lo = w_lo / g;
    const double z_hi = w_hi / g > 1. ? 1. : w_hi / g;

    struct bound { int kind; double A, from, to; int sign; };
    const struct bound bounds[4] = {
        {4, v_hi / g, h[0], h[1], +1},
        {1, u_lo / g, h[1], h[2], +1},
        {2, u_hi / g, h[0], h[3], -1},
        {3, v_lo / g, h[3], h[2], -1},
    };
    double area = 0.;
    for (int b = 0; b < 4; b++) {
        const struct bound *bd = &bounds[b];
        if (!(z_lo <= bd->to && z_hi > bd->from)) continue;
        const double end = z_hi <= bd->to ? z_hi : bd->to;
        const double start = z_lo <= bd->from ? bd->from : z_lo;
        const double fe = azimuth_primitive(bd->kind, end, bd->A);
        const double fs = azimuth_primitive(bd->kind, start, bd->A);
        if (bd->sign > 0) {
            area = area + fe;
            area = area - fs;
        } else {
            area = area - fe;
            area = area + fs;
        }
    }
    return area;
}

/* store_matrix_elements, compute_matrix.cu:505-562.  b = 4 pi |g| d3v;
 * a = (area < 1e-10) ? 0 : area * 2 |g| d3v, evaluated in double and stored
 * as float, at index (((in1*nx + gi)*(ny/2*nz/2) + jn1*(nz/2) + kn1)*ny*nz
 * + gj*nz + gk) with in = (gi&1) | (in1<<1) and likewise for jn, kn. */
void or_build_dense_tables(int nx, int ny, int nz, float du, float dv, float dw, float d3v,
                           float *b, float *a)
{
    const int nyz = ny * nz;
    for (int gi = 0; gi < nx; gi++)
        for (int gj = 0; gj < ny; gj++)
            for (int gk = 0; gk < nz; gk++) {
                float g = or_relative_speed(du, dv, dw, gi, gj, gk);
                b[gi * nyz + gj * nz + gk] = (float)(4.0 * M_PI * (double)g * (double)d3v);
            }
    const int hx = nx / 2, hy = ny / 2, hz = nz / 2;
#pragma omp parallel for collapse(2) schedule(dynamic)
    for (int in1 = 0; in1 < hx; in1++)
        for (int gi = 0; gi < nx; gi++) {
            const int in = (gi & 1) | (in1 << 1);
            for (int jn1 = 0; jn1 < hy; jn1++)
                for (int kn1 = 0; kn1 < hz; kn1++) {
                    float *row = a + ((size_t)(in1 * nx + gi) * (hy * hz) + jn1 * hz + kn1) * nyz;
                    for (int gj = 0; gj < ny; gj++)
                        for (int gk = 0; gk < nz; gk++) {
                            const int jn = (gj & 1) | (jn1 << 1);
                            const int kn = (gk & 1) | (kn1 << 1);
                            const double g1 = (double)or_relative_speed(du, dv, dw, gi, gj, gk);
                            const double A = or_box_sphere_area(du, dv, dw, in, jn, kn, g1);
                            row[gj * nz + gk] = (A < OR_ERR) ? 0.0f
                                                             : (float)(A * 2.0 * g1 * (double)d3v);
                        }
                }
        }
}

/* ------------------------------------------------------------------------ */
/* Context                                                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    int16_t n[3];
    float w;
} or_entry;

struct or_ctx {
    int nx, ny, nz, nyz, nxyz, n_pnt;
    float du, dv, dw, d3v;
    float *u, *v, *w;
    int *ui, *vi, *wi;
    int *compact; /* box index -> compact index or -1 */
    unsigned char *inside;
    float *a, *b;
    int64_t *list_off; /* per |g| box index */
    or_entry *list;
};

or_ctx *or_create(int nx, int ny, int nz, const float *vmin, const float *vmax, float R)
{
    if (nx < 2 || ny < 2 || nz < 2 || (nx & 1) || (ny & 1) || (nz & 1)) return NULL;
    or_ctx *c = (or_ctx *)calloc(1, sizeof(or_ctx));
    c->nx = nx;
    c->ny = ny;
    c->nz = nz;
    c->nyz = ny * nz;
    c->nxyz = nx * ny * nz;
    int np = or_grid_count(nx, ny, nz, vmin, vmax, R);
    c->u = (float *)malloc(sizeof(float) * nx);
    c->v = (float *)malloc(sizeof(float) * ny);
    c->w = (float *)malloc(sizeof(float) * nz);
    c->ui = (int *)malloc(sizeof(int) * (np + 1));
    c->vi = (int *)malloc(sizeof(int) * (np + 1));
    c->wi = (int *)malloc(sizeof(int) * (np + 1));
    float steps[4];
    c->n_pnt = or_grid_fill(nx, ny, nz, vmin, vmax, R, c->u, c->v, c->w, c->ui, c->vi, c->wi, steps);
    c->du = steps[0];
    c->dv = steps[1];
    c->dw = steps[2];
    c->d3v = steps[3];
    c->compact = (int *)malloc(sizeof(int) * c->nxyz);
    c->inside = (unsigned char *)calloc(c->nxyz, 1);
    for (int i = 0; i < c->nxyz; i++) c->compact[i] = -1;
    for (int p = 0; p < c->n_pnt; p++) {
        int bi = (c->ui[p] * ny + c->vi[p]) * nz + c->wi[p];
        c->compact[bi] = p;
        c->inside[bi] = 1;
    }
    const size_t na = (size_t)(nx / 2) * nx * (ny / 2) * (nz / 2) * ny * nz;
    c->a = (float *)malloc(sizeof(float) * na);
    c->b = (float *)malloc(sizeof(float) * c->nxyz);
    or_build_dense_tables(nx, ny, nz, c->du, c->dv, c->dw, c->d3v, c->b, c->a);

    /* nonzero (n, w) lists per |g|, in (in1, jn1, kn1) order */
    const int hx = nx / 2, hy = ny / 2, hz = nz / 2;
    c->list_off = (int64_t *)malloc(sizeof(int64_t) * (c->nxyz + 1));
    int64_t cnt = 0;
    for (int pass = 0; pass < 2; pass++) {
        cnt = 0;
        for (int gi = 0; gi < nx; gi++)
            for (int gj = 0; gj < ny; gj++)
                for (int gk = 0; gk < nz; gk++) {
                    int gidx = (gi * ny + gj) * nz + gk;
                    if (pass == 0) c->list_off[gidx] = cnt;
                    for (int in1 = 0; in1 < hx; in1++)
                        for (int jn1 = 0; jn1 < hy; jn1++)
                            for (int kn1 = 0; kn1 < hz; kn1++) {
                                float wv = c->a[((size_t)(in1 * nx + gi) * (hy * hz) + jn1 * hz + kn1) *
                                                    c->nyz +
                                                gj * nz + gk];
                                if (wv == 0.0f) continue;
                                if (pass == 1) {
                                    or_entry *e = &c->list[cnt];
                                    e->n[0] = (int16_t)((gi & 1) | (in1 << 1));
                                    e->n[1] = (int16_t)((gj & 1) | (jn1 << 1));
                                    e->n[2] = (int16_t)((gk & 1) | (kn1 << 1));
                                    e->w = wv;
                                }
                                cnt++;
                            }
                }
        if (pass == 0) {
            c->list_off[c->nxyz] = cnt;
            c->list = (or_entry *)malloc(sizeof(or_entry) * (cnt + 1));
        }
    }
    return c;
}

void or_destroy(or_ctx *c)
{
    if (!c) return;
    free(c->u);
    free(c->v);
    free(c->w);
    free(c->ui);
    free(c->vi);
    free(c->wi);
    free(c->compact);
    free(c->inside);
    free(c->a);
    free(c->b);
    free(c->list_off);
    free(c->list);
    free(c);
}

int or_n_pnt(const or_ctx *c) { return c->n_pnt; }
const float *or_table_a(const or_ctx *c) { return c->a; }
const float *or_table_b(const or_ctx *c) { return c->b; }
const int *or_compact_of_box(const or_ctx *c) { return c->compact; }

/* ------------------------------------------------------------------------ */
/* Gain enumeration                                                          */
/* ------------------------------------------------------------------------ */

/* For output node i and partner i1 (s = i + i1 per axis) and post-collision
 * offset n (parity of s), the post-collision nodes are l = (s+n)/2 and
 * l1 = (s-n)/2 per axis (collision_integral.cu:88-94, 115-131).  The four
 * products pair x of l with the y/z components of l or l1 in the four
 * sign patterns (collision_integral.cu:150-160):
 *   P1 = f(lx,ly,lz)  f(l1x,l1y,l1z)     P2 = f(lx,l1y,l1z) f(l1x,ly,lz)
 *   P3 = f(lx,ly,l1z) f(l1x,l1y,lz)      P4 = f(lx,l1y,lz)  f(l1x,ly,l1z)
 * All four exist exactly when lx < nx, l1x >= 0 and the same for y and z. */
typedef struct {
    int idx[8];
} or_octet;

static inline int octet_for(const or_ctx *c, int sx, int sy, int sz, const int16_t *n, or_octet *o)
{
    const int lx2 = sx + n[0], l1x2 = sx - n[0];
    const int ly2 = sy + n[1], l1y2 = sy - n[1];
    const int lz2 = sz + n[2], l1z2 = sz - n[2];
    if (lx2 > 2 * (c->nx - 1) || l1x2 < 0) return 0;
    if (ly2 > 2 * (c->ny - 1) || l1y2 < 0) return 0;
    if (lz2 > 2 * (c->nz - 1) || l1z2 < 0) return 0;
    const int lx = lx2 >> 1, l1x = l1x2 >> 1, ly = ly2 >> 1, l1y = l1y2 >> 1, lz = lz2 >> 1,
              l1z = l1z2 >> 1;
    const int ny = c->ny, nz = c->nz;
#define BOX(x, y, z) (((x) * ny + (y)) * nz + (z))
    o->idx[0] = BOX(lx, ly, lz);
    o->idx[1] = BOX(l1x, l1y, l1z);
    o->idx[2] = BOX(lx, l1y, l1z);
    o->idx[3] = BOX(l1x, ly, lz);
    o->idx[4] = BOX(lx, ly, l1z);
    o->idx[5] = BOX(l1x, l1y, lz);
    o->idx[6] = BOX(lx, l1y, lz);
    o->idx[7] = BOX(l1x, ly, l1z);
#undef BOX
    return 1;
}

static inline int octet_live(const or_ctx *c, const or_octet *o)
{
    const unsigned char *in = c->inside;
    return (in[o->idx[0]] && in[o->idx[1]]) || (in[o->idx[2]] && in[o->idx[3]]) ||
           (in[o->idx[4]] && in[o->idx[5]]) || (in[o->idx[6]] && in[o->idx[7]]);
}

void or_gain_f64(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 double *gain)
{
#pragma omp parallel
    {
        double *acc = (double *)malloc(sizeof(double) * ncells);
#pragma omp for schedule(dynamic, 1)
        for (int q = 0; q < nn; q++) {
            const int bi = nodes[q];
            const int ix = bi / c->nyz, iy = (bi / c->nz) % c->ny, iz = bi % c->nz;
            for (int cc = 0; cc < ncells; cc++) acc[cc] = 0.;
            for (int jx = 0; jx < c->nx; jx++)
                for (int jy = 0; jy < c->ny; jy++)
                    for (int jz = 0; jz < c->nz; jz++) {
                        const int gi = abs(ix - jx), gj = abs(iy - jy), gk = abs(iz - jz);
                        const int gidx = (gi * c->ny + gj) * c->nz + gk;
                        for (int64_t e = c->list_off[gidx]; e < c->list_off[gidx + 1]; e++) {
                            or_octet o;
                            if (!octet_for(c, ix + jx, iy + jy, iz + jz, c->list[e].n, &o)) continue;
                            if (!octet_live(c, &o)) continue;
                            const double w = c->list[e].w;
                            const float *p[8];
                            for (int t = 0; t < 8; t++) p[t] = f_box + (size_t)o.idx[t] * ncells;
                            for (int cc = 0; cc < ncells; cc++) {
                                const double t1 = (double)p[0][cc] * p[1][cc] + (double)p[2][cc] * p[3][cc];
                                const double t2 = (double)p[4][cc] * p[5][cc] + (double)p[6][cc] * p[7][cc];
                                acc[cc] += w * (t1 + t2);
                            }
                        }
                    }
            for (int cc = 0; cc < ncells; cc++) gain[(size_t)q * ncells + cc] = acc[cc];
        }
        free(acc);
    }
}

void or_gain_f32(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 float *gain)
{
#pragma omp parallel
    {
        float *acc = (float *)malloc(sizeof(float) * ncells);
#pragma omp for schedule(dynamic, 1)
        for (int q = 0; q < nn; q++) {
            const int bi = nodes[q];
            const int ix = bi / c->nyz, iy = (bi / c->nz) % c->ny, iz = bi % c->nz;
            for (int cc = 0; cc < ncells; cc++) acc[cc] = 0.f;
            for (int jx = 0; jx < c->nx; jx++)
                for (int jy = 0; jy < c->ny; jy++)
                    for (int jz = 0; jz < c->nz; jz++) {
                        const int gi = abs(ix - jx), gj = abs(iy - jy), gk = abs(iz - jz);
                        const int gidx = (gi * c->ny + gj) * c->nz + gk;
                        for (int64_t e = c->list_off[gidx]; e < c->list_off[gidx + 1]; e++) {
                            or_octet o;
                            if (!octet_for(c, ix + jx, iy + jy, iz + jz, c->list[e].n, &o)) continue;
                            if (!octet_live(c, &o)) continue;
                            const float w = c->list[e].w;
                            const float *p[8];
                            for (int t = 0; t < 8; t++) p[t] = f_box + (size_t)o.idx[t] * ncells;
                            for (int cc = 0; cc < ncells; cc++) {
                                const float t1 = p[0][cc] * p[1][cc] + p[2][cc] * p[3][cc];
                                const float t2 = p[4][cc] * p[5][cc] + p[6][cc] * p[7][cc];
                                acc[cc] += w * (t1 + t2);
                            }
                        }
                    }
            for (int cc = 0; cc < ncells; cc++) gain[(size_t)q * ncells + cc] = acc[cc];
        }
        free(acc);
    }
}

void or_count_work(const or_ctx *c, int64_t *out3)
{
    int64_t terms = 0, subterms = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : terms, subterms)
    for (int p = 0; p < c->n_pnt; p++) {
        const int ix = c->ui[p], iy = c->vi[p], iz = c->wi[p];
        for (int jx = 0; jx < c->nx; jx++)
            for (int jy = 0; jy < c->ny; jy++)
                for (int jz = 0; jz < c->nz; jz++) {
                    const int gidx = (abs(ix - jx) * c->ny + abs(iy - jy)) * c->nz + abs(iz - jz);
                    for (int64_t e = c->list_off[gidx]; e < c->list_off[gidx + 1]; e++) {
                        or_octet o;
                        if (!octet_for(c, ix + jx, iy + jy, iz + jz, c->list[e].n, &o)) continue;
                        terms++;
                        for (int t = 0; t < 8; t += 2)
                            subterms += c->inside[o.idx[t]] && c->inside[o.idx[t + 1]];
                    }
                }
    }
    out3[0] = c->list_off[c->nxyz];
    out3[1] = terms;
    out3[2] = subterms;
}

/* The index map of the gain as a digest: every (output node i in the sphere,
 * partner i1 in the box, post-collision offset n) with a nonzero weight whose
 * post-collision nodes l, l1 stay in the box (collision_integral.cu:88-94,
 * 115-131; out-of-box partners hit the N_YZ sentinel, :130-131, 154-155), as
 * the key k = i << 32 | s << 15 | n with i the compact index, s = i + i1 the
 * linear pair-sum index over (2nx-1)(2ny-1)(2nz-1) and n the box index of the
 * offset.  out4 = {count, sum of mix_a(k), xor of mix_b(k), sum of the FP64
 * weights}; the sums wrap mod 2^64, so the digest is independent of the
 * enumeration order and any other enumeration of the same set reproduces it. */
static inline uint64_t or_mix_a(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull; /* splitmix64 finaliser */
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static inline uint64_t or_mix_b(uint64_t z)
{
    z ^= 0x5851f42d4c957f2dull;
    z = (z ^ (z >> 33)) * 0xff51afd7ed558ccdull; /* murmur3 finaliser */
    z = (z ^ (z >> 33)) * 0xc4ceb9fe1a85ec53ull;
    return z ^ (z >> 33);
}

void or_index_map_digest(const or_ctx *c, uint64_t *out4)
{
    const int sy = 2 * c->ny - 1, sz = 2 * c->nz - 1;
    uint64_t cnt = 0, sa = 0, xb = 0;
    double wsum = 0.0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : cnt, sa, wsum) reduction(^ : xb)
    for (int p = 0; p < c->n_pnt; p++) {
        const int ix = c->ui[p], iy = c->vi[p], iz = c->wi[p];
        for (int jx = 0; jx < c->nx; jx++)
            for (int jy = 0; jy < c->ny; jy++)
                for (int jz = 0; jz < c->nz; jz++) {
                    const int gidx = (abs(ix - jx) * c->ny + abs(iy - jy)) * c->nz + abs(iz - jz);
                    const uint64_t s_lin = ((uint64_t)(ix + jx) * sy + (iy + jy)) * sz + (iz + jz);
                    for (int64_t e = c->list_off[gidx]; e < c->list_off[gidx + 1]; e++) {
                        or_octet o;
                        const int16_t *n = c->list[e].n;
                        if (!octet_for(c, ix + jx, iy + jy, iz + jz, n, &o)) continue;
                        const uint64_t n_box = ((uint64_t)n[0] * c->ny + n[1]) * c->nz + n[2];
                        const uint64_t k = ((uint64_t)p << 32) | (s_lin << 15) | n_box;
                        cnt++;
                        sa += or_mix_a(k);
                        xb ^= or_mix_b(k);
                        wsum += c->list[e].w;
                    }
                }
    }
    out4[0] = cnt;
    out4[1] = sa;
    out4[2] = xb;
    memcpy(&out4[3], &wsum, sizeof(double));
}

/* ------------------------------------------------------------------------ */
/* Loss                                                                      */
/* ------------------------------------------------------------------------ */

void or_loss_f64(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 double *nu)
{
#pragma omp parallel
    {
        double *acc = (double *)malloc(sizeof(double) * ncells);
#pragma omp for schedule(dynamic, 4)
        for (int q = 0; q < nn; q++) {
            const int bi = nodes[q];
            const int ix = bi / c->nyz, iy = (bi / c->nz) % c->ny, iz = bi % c->nz;
            for (int cc = 0; cc < ncells; cc++) acc[cc] = 0.;
            for (int j = 0; j < c->nxyz; j++) {
                if (!c->inside[j]) continue;
                const int jx = j / c->nyz, jy = (j / c->nz) % c->ny, jz = j % c->nz;
                const double bb =
                    c->b[(abs(ix - jx) * c->ny + abs(iy - jy)) * c->nz + abs(iz - jz)];
                const float *fj = f_box + (size_t)j * ncells;
                for (int cc = 0; cc < ncells; cc++) acc[cc] += bb * (double)fj[cc];
            }
            for (int cc = 0; cc < ncells; cc++) nu[(size_t)q * ncells + cc] = acc[cc];
        }
        free(acc);
    }
}

void or_loss_f32(const or_ctx *c, const float *f_box, int ncells, const int *nodes, int nn,
                 float *nu)
{
#pragma omp parallel
    {
        float *acc = (float *)malloc(sizeof(float) * ncells);
#pragma omp for schedule(dynamic, 4)
        for (int q = 0; q < nn; q++) {
            const int bi = nodes[q];
            const int ix = bi / c->nyz, iy = (bi / c->nz) % c->ny, iz = bi % c->nz;
            for (int cc = 0; cc < ncells; cc++) acc[cc] = 0.f;
            for (int j = 0; j < c->nxyz; j++) {
                if (!c->inside[j]) continue;
                const int jx = j / c->nyz, jy = (j / c->nz) % c->ny, jz = j % c->nz;
                const float bb = c->b[(abs(ix - jx) * c->ny + abs(iy - jy)) * c->nz + abs(iz - jz)];
                const float *fj = f_box + (size_t)j * ncells;
                for (int cc = 0; cc < ncells; cc++) acc[cc] += bb * fj[cc];
            }
            for (int cc = 0; cc < ncells; cc++) nu[(size_t)q * ncells + cc] = acc[cc];
        }
        free(acc);
    }
}

/* evolve_direct_colisions, collision_integral.cu:32-72: partner loop i1,
 * j1, k1 in box order, one fused multiply-add per partner into the FP32 sum. */
void or_loss_literal(const or_ctx *c, const float *f_box, int npx, int cell, const int *nodes,
                     int nn, float *nu)
{
    for (int q = 0; q < nn; q++) {
        const int bi = nodes[q];
        const int i = bi / c->nyz, j = (bi / c->nz) % c->ny, k = bi % c->nz;
        float acc = 0.f;
        for (int i1 = 0; i1 < c->nx; i1++) {
            const int gi = i > i1 ? i - i1 : i1 - i;
            for (int j1 = 0, idx1 = 0; j1 < c->ny; j1++)
                for (int k1 = 0; k1 < c->nz; k1++, idx1++) {
                    const int gj = j > j1 ? j - j1 : j1 - j;
                    const int gk = k > k1 ? k - k1 : k1 - k;
                    acc = fmaf(c->b[gi * c->nyz + gj * c->nz + gk],
                               f_box[((size_t)i1 * c->nyz + idx1) * npx + cell], acc);
                }
        }
        nu[q] = acc;
    }
}

/* evolve_inverse_colisions and its host loop, collision_integral.cu:75-188,
 * 637-648: launches over (in1, jn1, kn1); per launch partner planes i1 are
 * skipped when l or l1 leaves the box in x; per (j1, k1) the two paired
 * products of one half are summed, scaled by the weight, and the two halves
 * added into tmp before tmp is added to the output (FP32, no contraction).
 * The output goes to the intended node (i, j, k). */
void or_gain_literal(const or_ctx *c, const float *f_box, int npx, int cell, const int *nodes,
                     int nn, float *gain)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz, nyz = c->nyz;
    const int hy = ny / 2, hz = nz / 2;
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < nn; q++) {
        const int bi = nodes[q];
        const int i = bi / nyz, j = (bi / nz) % ny, k = bi % nz;
        float acc = 0.f;
        for (int in1 = 0; in1 < nx / 2; in1++)
            for (int jn1 = 0; jn1 < hy; jn1++)
                for (int kn1 = 0; kn1 < hz; kn1++)
                    for (int i1 = 0; i1 < nx; i1++) {
                        const int in = (in1 << 1) | ((i + i1) & 1);
                        const int il = (i + i1 + in) >> 1;
                        if (il > nx - 1) continue;
                        int il1 = i + i1 - in;
                        if (il1 < 0) continue;
                        il1 >>= 1;
                        const int gi = i > i1 ? i - i1 : i1 - i;
                        const float *row = c->a + ((size_t)(in1 * nx + gi) * (hy * hz) + jn1 * hz + kn1) * nyz;
                        const float *fl = f_box + (size_t)il * nyz * npx + cell;
                        const float *fl1 = f_box + (size_t)il1 * nyz * npx + cell;
                        for (int j1 = 0; j1 < ny; j1++) {
                            const int gj = j > j1 ? j - j1 : j1 - j;
                            const int jn = (gj & 1) | (jn1 << 1);
                            const int jl = (j + j1 + jn) >> 1;
                            const int jl1 = j + j1 - jn;
                            for (int k1 = 0; k1 < nz; k1++) {
                                const int gk = k > k1 ? k - k1 : k1 - k;
                                const int kn = (gk & 1) | (kn1 << 1);
                                const float wv = row[gj * nz + gk];
                                const int kl = (k + k1 + kn) >> 1;
                                const int kl1 = k + k1 - kn;
                                int l = (jl < ny && kl < nz) ? jl * nz + kl : nyz;
                                int l1 = (jl1 >= 0 && kl1 >= 0) ? (jl1 >> 1) * nz + (kl1 >> 1) : nyz;
                                float tmp = 0.f;
                                if (!(l == nyz || l1 == nyz)) {
                                    float p = fl[(size_t)l * npx] * fl1[(size_t)l1 * npx];
                                    p = p + fl[(size_t)l1 * npx] * fl1[(size_t)l * npx];
                                    tmp = wv * p;
                                }
                                l = (jl < ny && kl1 >= 0) ? jl * nz + (kl1 >> 1) : nyz;
                                l1 = (jl1 >= 0 && kl < nz) ? (jl1 >> 1) * nz + kl : nyz;
                                if (!(l == nyz || l1 == nyz)) {
                                    float p = fl[(size_t)l * npx] * fl1[(size_t)l1 * npx];
                                    p = p + fl[(size_t)l1 * npx] * fl1[(size_t)l * npx];
                                    tmp = tmp + wv * p;
                                }
                                acc = acc + tmp;
                            }
                        }
                    }
        gain[q] = acc;
    }
}

/* ------------------------------------------------------------------------ */
/* Conservation projection (intended semantics of collision_integral.cu:    */
/* 217-526, solved per cell in FP64)                                         */
/* ------------------------------------------------------------------------ */

/* Solve the symmetric 5x5 system by Gaussian elimination with partial
 * pivoting.  Returns 0 when a pivot vanishes (x is then left zero). */
static int solve5(double A[5][5], double bvec[5], double x[5])
{
    int perm[5] = {0, 1, 2, 3, 4};
    for (int k = 0; k < 5; k++) {
        int piv = k;
        double best = fabs(A[k][k]);
        for (int r = k + 1; r < 5; r++)
            if (fabs(A[r][k]) > best) {
                best = fabs(A[r][k]);
                piv = r;
            }
        if (!(best > 0.0)) {
            for (int t = 0; t < 5; t++) x[t] = 0.;
            return 0;
        }
        if (piv != k) {
            for (int t = 0; t < 5; t++) {
                double tmp = A[k][t];
                A[k][t] = A[piv][t];
                A[piv][t] = tmp;
            }
            double tmp = bvec[k];
            bvec[k] = bvec[piv];
            bvec[piv] = tmp;
            int tp = perm[k];
            perm[k] = perm[piv];
            perm[piv] = tp;
        }
        for (int r = k + 1; r < 5; r++) {
            const double m = A[r][k] / A[k][k];
            for (int t = k; t < 5; t++) A[r][t] -= m * A[k][t];
            bvec[r] -= m * bvec[k];
        }
    }
    for (int k = 4; k >= 0; k--) {
        double s = bvec[k];
        for (int t = k + 1; t < 5; t++) s -= A[k][t] * x[t];
        x[k] = s / A[k][k];
    }
    return 1;
}

int or_project(const or_ctx *c, const float *f, const float *nu, const float *gain, int ncells,
               double *nu_corr, double *q, double *x)
{
    int singular = 0;
#pragma omp parallel for schedule(static) reduction(+ : singular)
    for (int cc = 0; cc < ncells; cc++) {
        double A[5][5] = {{0}}, B[5] = {0};
        for (int p = 0; p < c->n_pnt; p++) {
            const double xu = c->u[c->ui[p]], xv = c->v[c->vi[p]], xw = c->w[c->wi[p]];
            const double phi[5] = {1., xu, xv, xw, xu * xu + xv * xv + xw * xw};
            const size_t o = (size_t)p * ncells + cc;
            const double fn = (double)f[o] * (double)nu[o];
            const double r = (double)gain[o] - fn;
            for (int k = 0; k < 5; k++) {
                B[k] += r * phi[k];
                for (int l = 0; l < 5; l++) A[k][l] += fn * phi[k] * phi[l];
            }
        }
        double X[5];
        if (!solve5(A, B, X)) singular++;
        for (int k = 0; k < 5; k++) x[(size_t)cc * 5 + k] = X[k];
        for (int p = 0; p < c->n_pnt; p++) {
            const double xu = c->u[c->ui[p]], xv = c->v[c->vi[p]], xw = c->w[c->wi[p]];
            const double xi2 = xu * xu + xv * xv + xw * xw;
            const size_t o = (size_t)p * ncells + cc;
            const double scale = 1. + X[0] + X[1] * xu + X[2] * xv + X[3] * xw + X[4] * xi2;
            const double nc = (double)nu[o] * scale;
            nu_corr[o] = nc;
            q[o] = (double)gain[o] - (double)f[o] * nc;
        }
    }
    return singular;
}

void or_moments(const or_ctx *c, const double *f, int ncells, double *m5)
{
    for (int cc = 0; cc < ncells; cc++) {
        double m[5] = {0};
        for (int p = 0; p < c->n_pnt; p++) {
            const double xu = c->u[c->ui[p]], xv = c->v[c->vi[p]], xw = c->w[c->wi[p]];
            const double fv = f[(size_t)p * ncells + cc];
            m[0] += fv;
            m[1] += fv * xu;
            m[2] += fv * xv;
            m[3] += fv * xw;
            m[4] += fv * (xu * xu + xv * xv + xw * xw);
        }
        for (int k = 0; k < 5; k++) m5[(size_t)cc * 5 + k] = m[k] * (double)c->d3v;
    }
}
