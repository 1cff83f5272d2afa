// gd_loss.cu -- loss frequency nu_i = sum_j b(|i - j|) f_j (sm_103a).
//
// Reference: evolve_direct_colisions, collision_integral.cu:32-72 (full-box
// partner loop; f is zero outside the sphere so only in-sphere partners
// contribute).  Lane = cell, each warp keeps kRows outputs in registers and
// streams the partners once for all of them; b and the node coordinates sit
// in shared memory.  The partner order is the compact node order for every
// output, so the FP32 sums are reproducible bit for bit.  The reference sums
// all partners in one FP32 chain; here each block of kBlock partners is
// summed in its own chain and the block sums are added with compensated
// (Kahan) summation, which keeps the frequency within a few FP32 ulp of the
// FP64 sum (one chain over the ~3600 partners of a 20^3 grid drifts to
// ~2e-6): the loss multiplies f in Q = I - f nu, where near equilibrium I
// and f nu agree to 1e-3, so its rounding shows up a thousandfold in Q.
#include "gd_internal.h"

#include <algorithm>

namespace gd {
namespace {

constexpr int kRows = 8;
constexpr int kWarps = 8;
constexpr int kBlock = 64;  // partners per partial chain

__global__ void __launch_bounds__(kWarps * 32) loss_kernel(Dims d, const float *__restrict__ f, int ld,
                                                           int ncells, const float *__restrict__ b,
                                                           const uint32_t *__restrict__ nodes,
                                                           float *__restrict__ nu)
{
    extern __shared__ __align__(16) unsigned char smem[];
    float *bs = reinterpret_cast<float *>(smem);
    uint32_t *ns = reinterpret_cast<uint32_t *>(smem + (((size_t)d.nxyz * 4 + 15) & ~(size_t)15));
    for (int t = threadIdx.x; t < d.nxyz; t += blockDim.x) bs[t] = b[t];
    for (int t = threadIdx.x; t < d.n_pnt; t += blockDim.x) ns[t] = nodes[t];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cell = blockIdx.x * 32 + lane;
    const bool live = cell < ncells;
    const float *fcol = f + (live ? cell : 0);
    const int row0 = (blockIdx.y * kWarps + warp) * kRows;
    if (row0 >= d.n_pnt) return;
    int ox[kRows], oy[kRows], oz[kRows];
#pragma unroll
    for (int r = 0; r < kRows; r++) {
        const int node = min(row0 + r, d.n_pnt - 1);
        const uint32_t p = ns[node];
        ox[r] = p & 1023;
        oy[r] = (p >> 10) & 1023;
        oz[r] = p >> 20;
    }
    float acc[kRows], comp[kRows];
#pragma unroll
    for (int r = 0; r < kRows; r++) acc[r] = comp[r] = 0.f;
    for (int j0 = 0; j0 < d.n_pnt; j0 += kBlock) {
        float part[kRows];
#pragma unroll
        for (int r = 0; r < kRows; r++) part[r] = 0.f;
        const int j1 = min(j0 + kBlock, d.n_pnt);
        for (int j = j0; j < j1; j++) {
            const uint32_t p = ns[j];
            const int jx = p & 1023, jy = (p >> 10) & 1023, jz = p >> 20;
            const float fj = live ? __ldg(fcol + (size_t)j * ld) : 0.f;
#pragma unroll
            for (int r = 0; r < kRows; r++) {
                const int idx = abs(ox[r] - jx) * d.nyz + abs(oy[r] - jy) * d.nz + abs(oz[r] - jz);
                part[r] = __fmaf_rn(bs[idx], fj, part[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < kRows; r++) {
            const float y = __fsub_rn(part[r], comp[r]);
            const float t = __fadd_rn(acc[r], y);
            comp[r] = __fsub_rn(__fsub_rn(t, acc[r]), y);
            acc[r] = t;
        }
    }
    if (!live) return;
#pragma unroll
    for (int r = 0; r < kRows; r++)
        if (row0 + r < d.n_pnt) nu[(size_t)(row0 + r) * ld + cell] = acc[r];
}

}  // namespace

int run_loss(Context &c, const float *f, int ncells, int ld, float *nu, cudaStream_t st)
{
    const Dims &d = c.d;
    const size_t smem = (((size_t)d.nxyz * 4 + 15) & ~(size_t)15) + (size_t)d.n_pnt * 4;
    GD_CUDA(cudaFuncSetAttribute(loss_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((ncells + 31) / 32, (d.n_pnt + kWarps * kRows - 1) / (kWarps * kRows));
    loss_kernel<<<grid, kWarps * 32, smem, st>>>(d, f, ld, ncells, c.d_b, c.d_nodes, nu);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

}  // namespace gd
