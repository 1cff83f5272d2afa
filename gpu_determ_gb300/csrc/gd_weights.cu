// gd_weights.cu -- analytic FP64 hard-sphere weight builder (sm_103a).
//
// Compiled with -fmad=false: every float and double expression rounds as
// written, so |g|, b and the case selection of the area formula match the
// host restatement operation for operation (only CUDA's atan and the
// host's atan may differ in the last ulp).
//
// Reference: compute_matrix.cu:21-257 (area of a sphere inside a lattice
// box), :505-562 (table layout and scaling).
#include "gd_internal.h"

#include <cmath>
#include <cstdio>

namespace gd {
namespace {

constexpr double kErr = 1.0e-10;  // velocity.h:37
constexpr double kHalfPi = 1.57079632679489661923;
constexpr double kPi = 3.14159265358979323846;

// |g| for lattice offset (gi, gj, gk): float components, float sum of squares
// summed u, v, w in that order, float square root (compute_matrix.cu:517-553).
__device__ __forceinline__ float relative_speed(float du, float dv, float dw, int gi, int gj, int gk)
{
    const float gu = du * (float)gi, gv = dv * (float)gj, gw = dw * (float)gk;
    float s = gu * gu;
    s = s + gv * gv;
    s = s + gw * gw;
    return sqrtf(s);
}

// Antiderivative in the height p of one azimuth bound of a box face on the
// unit sphere (kind 1: phi <= acos(A/rho), 2: phi >= acos(A/rho),
// 3: phi >= asin(A/rho), 4: phi <= asin(A/rho); rho = sqrt(1 - p^2)), with the
// limits the reference takes when A, p or 1 - A^2 - p^2 is within 1e-10 of a
// singular value (compute_matrix.cu:21-108).
__device__ double azimuth_primitive(int kind, double p, double A)
{
    const double q = 1. - A * A - p * p;
    const bool p_small = (p < kErr) && (p > -kErr);
    const bool q_small = (q < kErr) && (q > -kErr);
    const bool q_regular = (q >= kErr) && (p >= kErr);
    if (kind <= 2) {
        if (kind == 1 && (A < kErr) && (A > -kErr)) return kHalfPi * p;
        if (kind == 2 && A > (1 - kErr)) return 0.;
        if (p_small) return kHalfPi * A;
        if (q_small) return kHalfPi;
        if (q_regular && (kind == 2 || A >= kErr)) {
            const double s = sqrt(q);
            return p * atan(s / A) + A * atan(s / p) + atan(A * p / s);
        }
        return 0.;
    }
    if (kind == 3 && A < kErr) return 0.;
    if (kind == 4 && A > (1. - kErr)) return kHalfPi * p;
    if (p_small) return -kHalfPi * A;
    if (q_small) return kHalfPi * (p - 1.);
    if (q_regular) {
        const double s = sqrt(q);
        return kHalfPi * p - p * atan(s / A) - A * atan(s / p) - atan(A * p / s);
    }
    return 0.;
}

// Area of the sphere |x| = g inside box n (faces d(n-1) .. d(n+1) per axis,
// lower face clamped at 0 on the n = 0 layer), over g^2.  Integral over the
// height of the open azimuth interval: each of the four side-face bounds is
// active on a fixed range between the heights h0..h3 at which the sphere
// crosses the vertical box edges, and contributes F(end) - F(start) on the
// part of that range inside [z_lo, z_hi]; accumulated in the fixed order
// (v <= v_hi, u >= u_lo, u <= u_hi, v >= v_lo) (compute_matrix.cu:110-257).
__device__ double box_sphere_area(double du, double dv, double dw, int in, int jn, int kn, double g)
{
    const double u_lo = in > 0 ? du * (in - 1) : 0., u_hi = du * (in + 1);
    const double v_lo = jn > 0 ? dv * (jn - 1) : 0., v_hi = dv * (jn + 1);
    const double w_lo = kn > 0 ? dw * (kn - 1) : 0., w_hi = dw * (kn + 1);
    const double g2 = g * g;
    const double uu_lo = u_lo * u_lo, uu_hi = u_hi * u_hi;
    const double vv_lo = v_lo * v_lo, vv_hi = v_hi * v_hi;
    const double ww_lo = w_lo * w_lo, ww_hi = w_hi * w_hi;
    if (!(uu_lo + vv_lo + ww_lo < g2 && uu_hi + vv_hi + ww_hi > g2)) return 0.;
    const double phi_max = in > 1 ? atan(sqrt(g2 / uu_lo - 1.)) : kHalfPi;
    const double phi_min = jn > 1 ? kHalfPi - atan(sqrt(g2 / vv_lo - 1.)) : 0;
    if (!(phi_max > phi_min)) return 0.;
    double h[4];
    const double r2[4] = {uu_hi + vv_hi, uu_lo + vv_hi, uu_lo + vv_lo, uu_hi + vv_lo};
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const double t = 1. - r2[e] / g2;
        h[e] = t < 0 ? 0. : sqrt(t);
    }
    const double z_lo = w_lo / g;
    const double z_hi = w_hi / g > 1. ? 1. : w_hi / g;
    const int kinds[4] = {4, 1, 2, 3};
    const double As[4] = {v_hi / g, u_lo / g, u_hi / g, v_lo / g};
    const double from[4] = {h[0], h[1], h[0], h[3]};
    const double to[4] = {h[1], h[2], h[3], h[2]};
    double area = 0.;
#pragma unroll
    for (int b = 0; b < 4; b++) {
        if (!(z_lo <= to[b] && z_hi > from[b])) continue;
        const double end = z_hi <= to[b] ? z_hi : to[b];
        const double start = z_lo <= from[b] ? from[b] : z_lo;
        const double fe = azimuth_primitive(kinds[b], end, As[b]);
        const double fs = azimuth_primitive(kinds[b], start, As[b]);
        if (b < 2) {
            area = area + fe;
            area = area - fs;
        } else {
            area = area - fe;
            area = area + fs;
        }
    }
    return area;
}

// One thread per table entry; the linear index is the reference layout
// (((in1*nx + gi)*(hy*hz) + jn1*hz + kn1)*nyz + gj*nz + gk).
__global__ void dense_a_kernel(Dims d, float *__restrict__ a)
{
    const int64_t total = (int64_t)d.hx * d.nx * d.hy * d.hz * d.nyz;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = idx;
        const int gk = (int)(r % d.nz); r /= d.nz;
        const int gj = (int)(r % d.ny); r /= d.ny;
        const int kn1 = (int)(r % d.hz); r /= d.hz;
        const int jn1 = (int)(r % d.hy); r /= d.hy;
        const int gi = (int)(r % d.nx); r /= d.nx;
        const int in1 = (int)r;
        const int in = (gi & 1) | (in1 << 1);
        const int jn = (gj & 1) | (jn1 << 1);
        const int kn = (gk & 1) | (kn1 << 1);
        const double g1 = (double)relative_speed(d.du, d.dv, d.dw, gi, gj, gk);
        const double A = box_sphere_area((double)d.du, (double)d.dv, (double)d.dw, in, jn, kn, g1);
        a[idx] = (A < kErr) ? 0.0f : (float)(A * 2.0 * g1 * (double)d.d3v);
    }
}

// b[gi*nyz + gj*nz + gk] = 4 pi |g| d3v (compute_matrix.cu:519-530).
__global__ void dense_b_kernel(Dims d, float *__restrict__ b)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= d.nxyz) return;
    const int gk = idx % d.nz, gj = (idx / d.nz) % d.ny, gi = idx / d.nyz;
    const float g = relative_speed(d.du, d.dv, d.dw, gi, gj, gk);
    b[idx] = (float)(4.0 * kPi * (double)g * (double)d.d3v);
}

// Row |g| of the compact table: the nonzero a entries over (in1, jn1, kn1),
// in that lexicographic order, each stored with the byte offset of n's pair
// product in the gain kernel's P_s array (cb cells per class row).  Pass 1
// counts, pass 2 fills.
__global__ void weight_rows_kernel(Dims d, int cb, const float *__restrict__ a, const int *__restrict__ off,
                                   int *__restrict__ counts, WEntry *__restrict__ out)
{
    const int gbox = blockIdx.x * blockDim.x + threadIdx.x;
    if (gbox >= d.nxyz) return;
    const int gk = gbox % d.nz, gj = (gbox / d.nz) % d.ny, gi = gbox / d.nyz;
    int cnt = 0;
    int64_t pos = off ? off[gbox] : 0;
    for (int in1 = 0; in1 < d.hx; in1++)
        for (int jn1 = 0; jn1 < d.hy; jn1++)
            for (int kn1 = 0; kn1 < d.hz; kn1++) {
                const int64_t idx =
                    ((int64_t)(in1 * d.nx + gi) * (d.hy * d.hz) + jn1 * d.hz + kn1) * d.nyz +
                    gj * d.nz + gk;
                const float wv = a[idx];
                if (wv == 0.0f) continue;
                if (out) {
                    const int nc = (in1 * d.hy + jn1) * d.hz + kn1;
                    out[pos].off = (uint32_t)nc * (uint32_t)cb * 4u;
                    out[pos].w = wv;
                    pos++;
                }
                cnt++;
            }
    if (counts) counts[gbox] = cnt;
}

}  // namespace

int launch_dense_tables(const Dims &d, float *b, float *a, cudaStream_t st)
{
    if (b) {
        dense_b_kernel<<<(d.nxyz + 255) / 256, 256, 0, st>>>(d, b);
        GD_CUDA(cudaGetLastError());
    }
    if (a) {
        const int64_t total = (int64_t)d.hx * d.nx * d.hy * d.hz * d.nyz;
        int64_t blocks = (total + 255) / 256;
        if (blocks > 1 << 20) blocks = 1 << 20;
        dense_a_kernel<<<(unsigned)blocks, 256, 0, st>>>(d, a);
        GD_CUDA(cudaGetLastError());
    }
    return GD_OK;
}

int build_weight_rows(Context &c, const float *a_dense, cudaStream_t st)
{
    const Dims &d = c.d;
    int *d_counts = nullptr;
    GD_CUDA(cudaMalloc(&d_counts, sizeof(int) * d.nxyz));
    weight_rows_kernel<<<(d.nxyz + 127) / 128, 128, 0, st>>>(d, c.gain_cb, a_dense, nullptr, d_counts, nullptr);
    cudaError_t e = cudaGetLastError();
    std::vector<int> counts(d.nxyz);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts.data(), d_counts, sizeof(int) * d.nxyz,
                                              cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(d_counts);
        return cuda_error(e, "weight row count");
    }
    std::vector<int> off(d.nxyz + 1);
    int64_t total = 0;
    for (int g = 0; g < d.nxyz; g++) {
        off[g] = (int)total;
        total += counts[g];
    }
    off[d.nxyz] = (int)total;
    if (total >= (int64_t)1 << 31) {
        cudaFree(d_counts);
        return set_error(GD_ERR_UNSUPPORTED, "weight table has more than 2^31 nonzero entries");
    }
    c.n_entries = total;
    e = cudaMalloc(&c.d_list_off, sizeof(int) * (d.nxyz + 1));
    if (e == cudaSuccess) e = cudaMalloc(&c.d_list, sizeof(WEntry) * (total + 1));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c.d_list_off, off.data(), sizeof(int) * (d.nxyz + 1),
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        weight_rows_kernel<<<(d.nxyz + 127) / 128, 128, 0, st>>>(d, c.gain_cb, a_dense, c.d_list_off, nullptr,
                                                                 c.d_list);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_counts);
    if (e != cudaSuccess) return cuda_error(e, "weight row fill");
    return GD_OK;
}

}  // namespace gd
