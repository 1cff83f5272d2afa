// gd_project.cu -- FP64 conservation projection, relaxation step, moments and
// the correction basis (sm_103a).
//
// Projection (intended semantics of collision_integral.cu:217-526, one 5x5
// system per cell): with phi = (1, xi_x, xi_y, xi_z, xi^2),
//   A_kl = sum_i f_i nu_i phi_k phi_l,  B_k = sum_i (I_i - f_i nu_i) phi_k,
//   A X = B,  nu'_i = nu_i (1 + X.phi_i),  Q_i = I_i - f_i nu'_i,
// after which sum_i Q_i phi_k = 0 (mass, momentum, energy) up to FP64 rounding.
// Lane = cell; warps split the nodes; the per-warp FP64 partial sums are
// combined across warps in warp order, so the sums are reproducible.
#include "gd_internal.h"

#include <algorithm>
#include <cfloat>

namespace gd {
namespace {

constexpr int kWarps = 8;
constexpr int kSums = 25;  // 5 B, 15 A (upper triangle), 5 moments

struct ProjArgs {
    Dims d;
    const float *f, *nu, *gain;
    int ld, ncells;
    const double *phi;  // [5][n_pnt]
    float *nu_corr;
    double *q;
    double *x;
    int update;  // 1: write f_out = f + dt Q
    float dt;
    float *f_out;
    double *m5;
    unsigned int *status;  // [0] flags (1 non-finite sums, 2 singular system), [1] first cell
};

// Gaussian elimination with partial pivoting on a symmetric 5x5 system.
__device__ bool solve5(double A[5][5], double b[5], double x[5])
{
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
            return false;
        }
        if (piv != k) {
            for (int t = 0; t < 5; t++) {
                const double tmp = A[k][t];
                A[k][t] = A[piv][t];
                A[piv][t] = tmp;
            }
            const double tb = b[k];
            b[k] = b[piv];
            b[piv] = tb;
        }
        for (int r = k + 1; r < 5; r++) {
            const double m = A[r][k] / A[k][k];
            for (int t = k; t < 5; t++) A[r][t] -= m * A[k][t];
            b[r] -= m * b[k];
        }
    }
    for (int k = 4; k >= 0; k--) {
        double s = b[k];
        for (int t = k + 1; t < 5; t++) s -= A[k][t] * x[t];
        x[k] = s / A[k][k];
    }
    return true;
}

__global__ void __launch_bounds__(kWarps * 32) project_kernel(ProjArgs a)
{
    __shared__ double red[kSums][32];
    __shared__ double xs[5][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cell = blockIdx.x * 32 + lane;
    const bool live = cell < a.ncells;
    const int n = a.d.n_pnt;
    double s[kSums];
#pragma unroll
    for (int k = 0; k < kSums; k++) s[k] = 0.;
    if (live) {
        for (int i = warp; i < n; i += kWarps) {
            const size_t o = (size_t)i * a.ld + cell;
            const double fv = a.f[o], nv = a.nu[o], gv = a.gain[o];
            const double ph[5] = {1.0, a.phi[n + i], a.phi[2 * n + i], a.phi[3 * n + i], a.phi[4 * n + i]};
            const double fn = fv * nv, r = gv - fn;
#pragma unroll
            for (int k = 0; k < 5; k++) s[k] += r * ph[k];
            int t = 5;
#pragma unroll
            for (int k = 0; k < 5; k++)
#pragma unroll
                for (int l = k; l < 5; l++) s[t++] += fn * ph[k] * ph[l];
#pragma unroll
            for (int k = 0; k < 5; k++) s[20 + k] += fv * ph[k];
        }
    }
    // combine the warps' partial sums in warp order
    for (int w = 0; w < kWarps; w++) {
        if (warp == w)
#pragma unroll
            for (int k = 0; k < kSums; k++) red[k][lane] = (w == 0 ? 0. : red[k][lane]) + s[k];
        __syncthreads();
    }
    if (warp == 0) {
        double tot[kSums];
#pragma unroll
        for (int k = 0; k < kSums; k++) tot[k] = red[k][lane];
        double A[5][5], B[5], X[5];
        int t = 5;
        for (int k = 0; k < 5; k++) B[k] = tot[k];
        for (int k = 0; k < 5; k++)
            for (int l = k; l < 5; l++) {
                A[k][l] = tot[t];
                A[l][k] = tot[t];
                t++;
            }
        bool finite = true;
#pragma unroll
        for (int k = 0; k < kSums; k++) finite = finite && isfinite(tot[k]);
        const bool solved = finite && solve5(A, B, X);
        if (!solved) {
            for (int k = 0; k < 5; k++) X[k] = 0.;
            // recorded for gd_ctx_check: the flags OR together, the smallest
            // failing cell wins, so the record does not depend on scheduling
            if (live && a.status && (!finite || tot[20] != 0.0)) {  // an empty cell has nothing to correct
                atomicOr(a.status, finite ? 2u : 1u);
                atomicMin(a.status + 1, (unsigned int)cell);
            }
        }
        for (int k = 0; k < 5; k++) xs[k][lane] = X[k];
        if (live) {
            if (a.x)
                for (int k = 0; k < 5; k++) a.x[(size_t)cell * 5 + k] = X[k];
            if (a.m5)
                for (int k = 0; k < 5; k++) a.m5[(size_t)cell * 5 + k] = tot[20 + k] * (double)a.d.d3v;
        }
    }
    __syncthreads();
    if (!live) return;
    const double X0 = xs[0][lane], X1 = xs[1][lane], X2 = xs[2][lane], X3 = xs[3][lane], X4 = xs[4][lane];
    for (int i = warp; i < n; i += kWarps) {
        const size_t o = (size_t)i * a.ld + cell;
        const double fv = a.f[o], nv = a.nu[o], gv = a.gain[o];
        const double scale = 1. + X0 + X1 * a.phi[n + i] + X2 * a.phi[2 * n + i] +
                             X3 * a.phi[3 * n + i] + X4 * a.phi[4 * n + i];
        const double nc = nv * scale;
        const double qv = gv - fv * nc;
        if (a.nu_corr) a.nu_corr[o] = (float)nc;
        if (a.q) a.q[o] = qv;
        if (a.update) a.f_out[o] = (float)(fv + (double)a.dt * qv);
    }
}

// Per-block maximum of nu' (non-negative); a second launch with one block
// reduces the block maxima.  Block b takes the rows b, b + gridDim.x, ..., its
// threads the cells of each row (32-bit indices, four loads in flight per
// thread).  The maximum does not depend on the order.
__global__ void max_kernel(const float *__restrict__ v, int n_pnt, int ncells, int ld,
                           float *__restrict__ out)
{
    __shared__ float sm[256];
    float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
    const int step = blockDim.x;
    for (int node = blockIdx.x; node < n_pnt; node += gridDim.x) {
        const float *row = v + (size_t)node * ld;
        int c = threadIdx.x;
        for (; c + 3 * step < ncells; c += 4 * step) {
            m0 = fmaxf(m0, __ldg(row + c));
            m1 = fmaxf(m1, __ldg(row + c + step));
            m2 = fmaxf(m2, __ldg(row + c + 2 * step));
            m3 = fmaxf(m3, __ldg(row + c + 3 * step));
        }
        for (; c < ncells; c += step) m0 = fmaxf(m0, __ldg(row + c));
    }
    sm[threadIdx.x] = fmaxf(fmaxf(m0, m1), fmaxf(m2, m3));
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sm[0];
}

// dt = courant / max nu' (get_delta_t, collision_integral.cu:776-807: the
// minimum of courant/nu over all nodes and cells equals courant over the
// largest nu after rounding, since division is monotone), or a fixed dt.
__global__ void dt_kernel(const float *__restrict__ blockmax, int nb, int mode, float param,
                          float *__restrict__ dt_out, float *__restrict__ time_dev,
                          float *__restrict__ dt_user)
{
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    float dt = param;
    if (mode == GD_DT_COURANT) {
        // one warp: lanes take strided block maxima, then a shuffle maximum
        float m = 0.f;
        for (int k = threadIdx.x; k < nb; k += 32) m = fmaxf(m, blockmax[k]);
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        dt = m > 0.f ? param / m : 1.0e10f;
    }
    if (threadIdx.x != 0) return;
    *dt_out = dt;
    if (dt_user) *dt_user = dt;
    if (time_dev) *time_dev += dt;
}

// f <- f + dt (I - f nu')  (evolve_f, collision_integral.cu:809-833), in FP64.
// Block b takes the rows b, b + gridDim.x, ..., its threads the cells of each
// row (32-bit indices).
__global__ void relax_kernel(float *__restrict__ f, const float *__restrict__ nu,
                             const float *__restrict__ gain, const double *__restrict__ q, int n_pnt,
                             int ncells, int ld, const float *__restrict__ dt_dev)
{
    const double dt = *dt_dev;
    for (int node = blockIdx.x; node < n_pnt; node += gridDim.x) {
        const size_t r = (size_t)node * ld;
        for (int c = threadIdx.x; c < ncells; c += blockDim.x) {
            const size_t o = r + c;
            const double fv = f[o];
            const double qv = q ? q[o] : (double)gain[o] - fv * (double)nu[o];
            f[o] = (float)(fv + dt * qv);
        }
    }
}

__global__ void __launch_bounds__(kWarps * 32) moments_kernel(Dims d, const float *__restrict__ f,
                                                              int ld, int ncells,
                                                              const double *__restrict__ phi,
                                                              double *__restrict__ m5)
{
    __shared__ double red[kWarps][5][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cell = blockIdx.x * 32 + lane;
    const bool live = cell < ncells;
    const int n = d.n_pnt;
    double s[5] = {0., 0., 0., 0., 0.};
    if (live)
        for (int i = warp; i < n; i += kWarps) {
            const double fv = f[(size_t)i * ld + cell];
            s[0] += fv;
#pragma unroll
            for (int k = 1; k < 5; k++) s[k] += fv * phi[k * n + i];
        }
#pragma unroll
    for (int k = 0; k < 5; k++) red[warp][k][lane] = s[k];
    __syncthreads();
    if (warp == 0 && live)
        for (int k = 0; k < 5; k++) {
            double v = 0.;
            for (int w = 0; w < kWarps; w++) v += red[w][k][lane];
            m5[(size_t)cell * 5 + k] = v * (double)d.d3v;
        }
}

// The 14 basis rows of fill_correction_array (velocity.cu:17-50) over the box,
// in float as the reference forms them.
__global__ void basis_kernel(Dims d, const float *__restrict__ u, const float *__restrict__ v,
                             const float *__restrict__ w, float *__restrict__ out)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= d.nxyz) return;
    const int k = idx % d.nz, j = (idx / d.nz) % d.ny, i = idx / d.nyz;
    const float xx = u[i], xy = v[j], xz = w[k];
    float x2 = xx * xx;
    x2 = x2 + xy * xy;
    x2 = x2 + xz * xz;
    const float vals[14] = {xx, xy, xz, x2, xx * xx, xx * xy, xx * xz, xx * x2,
                            xy * xy, xy * xz, xy * x2, xz * xz, xz * x2, x2 * x2};
#pragma unroll
    for (int r = 0; r < 14; r++) out[(size_t)r * d.nxyz + idx] = vals[r];
}

}  // namespace

int run_project(Context &c, const float *f, const float *nu, const float *gain, int ncells, int ld,
                float *nu_corr, double *q, double *x, int fixed_dt_mode, float dt, float *f_out,
                double *m5, cudaStream_t st)
{
    ProjArgs a{c.d, f, nu, gain, ld, ncells, c.d_phi, nu_corr, q, x, fixed_dt_mode ? 1 : 0, dt, f_out, m5,
               c.d_status};
    project_kernel<<<(ncells + 31) / 32, kWarps * 32, 0, st>>>(a);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

int run_relax_q(Context &c, float *f, const float *nu_corr, const float *gain, const double *q,
                int ncells, int ld, int mode, float param, float *time_dev, float *dt_dev,
                cudaStream_t st)
{
    // blocks of the maximum: a few per SM, within the reduction buffer
    const int nb = std::max(1, std::min(std::min(4 * c.sm_count, kReduceFloats - 1), c.d.n_pnt));
    float *blockmax = c.d_reduce;        // [nb]
    float *dt_scalar = c.d_reduce + nb;  // [1]
    if (mode == GD_DT_COURANT) {
        max_kernel<<<nb, 256, 0, st>>>(nu_corr, c.d.n_pnt, ncells, ld, blockmax);
        GD_CUDA(cudaGetLastError());
    }
    dt_kernel<<<1, 32, 0, st>>>(blockmax, nb, mode, param, dt_scalar, time_dev, dt_dev);
    GD_CUDA(cudaGetLastError());
    const int blocks = std::min(c.d.n_pnt, c.sm_count * 16);
    relax_kernel<<<std::max(blocks, 1), 256, 0, st>>>(f, nu_corr, gain, q, c.d.n_pnt, ncells, ld, dt_scalar);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

int run_relax(Context &c, float *f, const float *nu_corr, const float *gain, int ncells, int ld,
              int mode, float param, float *time_dev, float *dt_dev, cudaStream_t st)
{
    return run_relax_q(c, f, nu_corr, gain, nullptr, ncells, ld, mode, param, time_dev, dt_dev, st);
}

int run_moments(Context &c, const float *f, int ncells, int ld, double *m5, cudaStream_t st)
{
    moments_kernel<<<(ncells + 31) / 32, kWarps * 32, 0, st>>>(c.d, f, ld, ncells, c.d_phi, m5);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

int run_basis(Context &c, float *basis, cudaStream_t st)
{
    float *du = nullptr;
    const size_t n = c.u.size() + c.v.size() + c.w.size();
    GD_CUDA(cudaMallocAsync(&du, sizeof(float) * n, st));
    cudaError_t e = cudaMemcpyAsync(du, c.u.data(), sizeof(float) * c.u.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(du + c.u.size(), c.v.data(), sizeof(float) * c.v.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(du + c.u.size() + c.v.size(), c.w.data(), sizeof(float) * c.w.size(),
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        basis_kernel<<<(c.d.nxyz + 255) / 256, 256, 0, st>>>(c.d, du, du + c.u.size(),
                                                             du + c.u.size() + c.v.size(), basis);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(du, st);
    if (e != cudaSuccess) return cuda_error(e, "correction basis");
    if (e2 != cudaSuccess) return cuda_error(e2, "correction basis free");
    return GD_OK;
}

}  // namespace gd
