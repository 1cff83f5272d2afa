// gd_mlp.cu -- BF16 training and inference kernels of the collision surrogate.
//
// Network (per cell; x is the cell's distribution over the compact nodes):
//   h0 = W0 x + b0                      encoder      n_in  -> 256
//   h1 = GELU(W1 h0 + b1)               MLP          256   -> 512
//   h2 = GELU(W2 h1 + b2)                            512   -> 512
//   z  = W3 h2 + b3 + h0                (residual)   512   -> 256
//   y  = W4 z + b4                      decoder      256   -> n_out
// Every matrix product is C = A B^T on the tcgen05 tensor cores (BF16
// operands staged by TMA, FP32 accumulation in tensor memory) with the bias,
// GELU, GELU derivative or residual applied in the epilogue.  Weights are FP32
// masters with BF16 copies; Adam updates the masters.  Batch rows are cells;
// the public entry points take and return the library's [node][cell] layout.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_tc.cuh"

namespace gd {
namespace {

using namespace tc;
using bf16 = __nv_bfloat16;

constexpr int GM = 128, GN = 256, GK = 64, GS = 4;
constexpr uint32_t kA = GM * GK * 2, kB = GN * GK * 2, kStageBytes = kA + kB;
constexpr uint32_t kGIdesc = umma_idesc_bf16(GM, GN);
constexpr int kGThreads = 192;
constexpr size_t kGemmSmem = GS * kStageBytes + 1024;

enum { EPI_NONE = 0, EPI_GELU = 1, EPI_DGELU = 2 };

struct GemmArgs {
    int M, N, K;
    const float *bias;  // [N] or null
    const float *add;   // [M][ld32] added after the bias, or null
    const float *aux;   // EPI_DGELU: pre-activation [M][ld32]
    float *pre_out;     // EPI_GELU: pre-activation out [M][ld32], or null
    float *c32;         // [M][ld32] or null
    bf16 *c16;          // [M][ld16] or null
    int ld32, ld16;
    int *err;
    // failure-detection test hook: > 0 makes every CTA wait this many polls on
    // a barrier that nothing arrives at (before any copy or MMA is issued),
    // record the time-out, free its tensor memory and return
    int stall_polls;
};

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x)
{
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

template <int EPI>
__device__ __forceinline__ void epilogue_value(const GemmArgs &p, size_t o32, int n, float &x)
{
    if (p.bias) x += __ldg(p.bias + n);
    if (p.add) x += p.add[o32];
    if (EPI == EPI_GELU) {
        if (p.pre_out) p.pre_out[o32] = x;
        x = gelu(x);
    } else if (EPI == EPI_DGELU) {
        x *= gelu_grad(p.aux[o32]);
    }
}

// C[M][N] = sum_k A[m][k] B[n][k] (A: M x K, B: N x K, both K-major BF16),
// one 128 x 256 tile per CTA; warp 0 issues TMA, warp 1 the MMAs, warps 2..5
// read the accumulator (row m = thread) and apply the epilogue.
template <int EPI>
__global__ void __launch_bounds__(kGThreads, 1)
    gemm_nt_kernel(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, GemmArgs p)
{
    extern __shared__ __align__(1024) unsigned char dsmem[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t full_bar[GS], empty_bar[GS], acc_bar, stall_bar;
    __shared__ uint32_t tmem_holder;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * GM, n0 = blockIdx.y * GN;
    const int num_k = p.K / GK;

    if (threadIdx.x == 0) abort_flag = *(volatile int *)p.err;
    __syncthreads();
    if (abort_flag) return;
    if (threadIdx.x == 0) {
        for (int s = 0; s < GS; s++) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        mbar_init(smem_u32(&acc_bar), 1);
        mbar_init(smem_u32(&stall_bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(GN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_holder;

    if (p.stall_polls > 0) {
        // test hook: a bounded wait that must run out (stall_bar never
        // completes a phase); nothing has been issued yet, so the CTA can go
        // straight to the common exit below, which frees the tensor memory
        if (threadIdx.x == 32) mbar_wait_limit(smem_u32(&stall_bar), 0u, p.err, (uint32_t)p.stall_polls);
        __syncthreads();
        if (threadIdx.x == 0) abort_flag = *(volatile int *)p.err;
        __syncthreads();
    }

    if (abort_flag) {
        // every thread skips the work alike and meets the barrier below
    } else if (warp == 0) {
        if (lane == 0) {
            for (int k = 0; k < num_k; k++) {
                const int s = k % GS;
                const uint32_t ph = (uint32_t)(k / GS) & 1u;
                if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, p.err)) break;
                unsigned char *st = base + (size_t)s * kStageBytes;
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, kStageBytes);
                tma_load_2d(smem_u32(st), &tA, k * GK, m0, fb);
                tma_load_2d(smem_u32(st + kA), &tB, k * GK, n0, fb);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            bool ok = true;
            for (int k = 0; k < num_k; k++) {
                const int s = k % GS;
                const uint32_t ph = (uint32_t)(k / GS) & 1u;
                if (!mbar_wait(smem_u32(&full_bar[s]), ph, p.err)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t st = smem_u32(base + (size_t)s * kStageBytes);
#pragma unroll
                for (int kk = 0; kk < GK / 16; kk++) {
                    const uint32_t off = (uint32_t)kk * 32u;
                    umma_bf16(tmem, umma_desc(st + off), umma_desc(st + kA + off), kGIdesc, (k > 0 || kk > 0) ? 1u : 0u);
                }
                umma_commit(smem_u32(&empty_bar[s]));
            }
            if (ok) umma_commit(smem_u32(&acc_bar));
        }
    } else {
        const int quad = warp & 3;
        const int m = m0 + quad * 32 + lane;
        bool ok = true;
        if (lane == 0) ok = mbar_wait(smem_u32(&acc_bar), 0u, p.err);
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16);
            for (int c0 = 0; c0 < GN; c0 += 32) {
                float v[32];
                tmem_ld32(taddr + (uint32_t)c0, v);
                if (m >= p.M || n0 + c0 >= p.N) continue;
                const size_t r32 = (size_t)m * p.ld32, r16 = (size_t)m * p.ld16;
                if (n0 + c0 + 32 <= p.N) {
                    // full 32-column chunk: 16-byte FP32 and 8-byte BF16 stores
                    // (ld32, ld16 are multiples of 4 and n0 + c0 of 32)
#pragma unroll
                    for (int j = 0; j < 32; j += 4) {
                        const int n = n0 + c0 + j;
                        float x[4] = {v[j], v[j + 1], v[j + 2], v[j + 3]};
#pragma unroll
                        for (int q = 0; q < 4; q++) epilogue_value<EPI>(p, r32 + n + q, n + q, x[q]);
                        if (p.c32) *reinterpret_cast<float4 *>(p.c32 + r32 + n) = make_float4(x[0], x[1], x[2], x[3]);
                        if (p.c16) {
                            __nv_bfloat162 lo = __floats2bfloat162_rn(x[0], x[1]);
                            __nv_bfloat162 hi = __floats2bfloat162_rn(x[2], x[3]);
                            uint2 pk;
                            pk.x = *reinterpret_cast<uint32_t *>(&lo);
                            pk.y = *reinterpret_cast<uint32_t *>(&hi);
                            *reinterpret_cast<uint2 *>(p.c16 + r16 + n) = pk;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j++) {
                        const int n = n0 + c0 + j;
                        if (n < p.N) {
                            float x = v[j];
                            epilogue_value<EPI>(p, r32 + n, n, x);
                            if (p.c32) p.c32[r32 + n] = x;
                            if (p.c16) p.c16[r16 + n] = __float2bfloat16_rn(x);
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(GN) : "memory");
    }
}

// C[M][N] = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T (FP32) for K-major BF16
// operands: the FP32-equivalent product of two BF16 hi/lo splits, in one
// launch.  The tensor cores' FP32 accumulation loses bits over long sums, so
// the K range runs in chunks of kchunk 64-column steps: each chunk goes into
// one of two tensor-memory accumulators, and the epilogue adds the chunks, in
// chunk order, into FP32 sums it holds in registers (one row and 128 columns
// per thread).  One 128 x 128 tile per CTA; warp 0 issues TMA, warp 1 the
// MMAs (three per 16-column K step), warps 2..5 the epilogue.  Every wait is
// bounded.
constexpr int XM = 128, XN = 128, XS = 3;
constexpr uint32_t kXA = XM * GK * 2, kXB = XN * GK * 2, kXStage = 2 * kXA + 2 * kXB;  // 64 KB
constexpr uint32_t kXIdesc = umma_idesc_bf16(XM, XN);
constexpr size_t kX3Smem = XS * kXStage + 1024;

struct Gemm3Args {
    int M, N, K, kchunk;  // K and kchunk in elements (multiples of 64)
    float *c;
    int ldc;
    int *err;
    int stall_polls;  // failure-detection test hook, as in GemmArgs
};

__global__ void __launch_bounds__(kGThreads, 1)
    gemm3_nt_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                    const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, Gemm3Args p)
{
    extern __shared__ __align__(1024) unsigned char dsmem[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t full_bar[XS], empty_bar[XS], accf_bar[2], acce_bar[2], stall_bar;
    __shared__ uint32_t tmem_holder;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * XM, n0 = blockIdx.y * XN;
    const int num_k = p.K / GK, kcs = p.kchunk / GK;
    const int nchunks = (num_k + kcs - 1) / kcs;

    if (threadIdx.x == 0) abort_flag = *(volatile int *)p.err;
    __syncthreads();
    if (abort_flag) return;
    if (threadIdx.x == 0) {
        for (int s = 0; s < XS; s++) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&accf_bar[b]), 1);
            mbar_init(smem_u32(&acce_bar[b]), 4);  // the four epilogue warps
        }
        mbar_init(smem_u32(&stall_bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(2 * XN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_holder;

    if (p.stall_polls > 0) {
        // test hook: a bounded wait that must run out before anything is issued
        if (threadIdx.x == 32) mbar_wait_limit(smem_u32(&stall_bar), 0u, p.err, (uint32_t)p.stall_polls);
        __syncthreads();
        if (threadIdx.x == 0) abort_flag = *(volatile int *)p.err;
        __syncthreads();
    }

    if (abort_flag) {
        // every thread skips the work alike and meets the barrier below
    } else if (warp == 0) {
        if (lane == 0) {
            for (int k = 0; k < num_k; k++) {
                const int s = k % XS;
                const uint32_t ph = (uint32_t)(k / XS) & 1u;
                if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, p.err)) break;
                unsigned char *st = base + (size_t)s * kXStage;
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, kXStage);
                tma_load_2d(smem_u32(st), &tAh, k * GK, m0, fb);
                tma_load_2d(smem_u32(st + kXA), &tAl, k * GK, m0, fb);
                tma_load_2d(smem_u32(st + 2 * kXA), &tBh, k * GK, n0, fb);
                tma_load_2d(smem_u32(st + 2 * kXA + kXB), &tBl, k * GK, n0, fb);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            bool ok = true;
            int k = 0;
            for (int c = 0; ok && c < nchunks; c++) {
                const int buf = c & 1;
                if (!mbar_wait(smem_u32(&acce_bar[buf]), ((uint32_t)(c >> 1) & 1u) ^ 1u, p.err)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d_tmem = tmem + (uint32_t)(buf * XN);
                const int kend = min(num_k, k + kcs);
                for (const int kbeg = k; k < kend; k++) {
                    const int s = k % XS;
                    if (!mbar_wait(smem_u32(&full_bar[s]), (uint32_t)(k / XS) & 1u, p.err)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t st = smem_u32(base + (size_t)s * kXStage);
                    const uint32_t aH = st, aL = st + kXA, bH = st + 2 * kXA, bL = st + 2 * kXA + kXB;
#pragma unroll
                    for (int kk = 0; kk < GK / 16; kk++) {
                        const uint32_t off = (uint32_t)kk * 32u;
                        umma_bf16(d_tmem, umma_desc(aH + off), umma_desc(bH + off), kXIdesc,
                                  (k > kbeg || kk > 0) ? 1u : 0u);
                        umma_bf16(d_tmem, umma_desc(aH + off), umma_desc(bL + off), kXIdesc, 1u);
                        umma_bf16(d_tmem, umma_desc(aL + off), umma_desc(bH + off), kXIdesc, 1u);
                    }
                    umma_commit(smem_u32(&empty_bar[s]));
                }
                if (ok) umma_commit(smem_u32(&accf_bar[buf]));
            }
        }
    } else {
        const int quad = warp & 3;
        const int m = m0 + quad * 32 + lane;
        float sum[XN];
#pragma unroll
        for (int j = 0; j < XN; j++) sum[j] = 0.f;
        bool ok = true;
        for (int c = 0; ok && c < nchunks; c++) {
            const int buf = c & 1;
            bool w = true;
            if (lane == 0) w = mbar_wait(smem_u32(&accf_bar[buf]), (uint32_t)(c >> 1) & 1u, p.err);
            if (__shfl_sync(0xffffffffu, w ? 1 : 0, 0) == 0) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * XN);
#pragma unroll
            for (int c0 = 0; c0 < XN; c0 += 32) {
                float v[32];
                tmem_ld32(taddr + (uint32_t)c0, v);
#pragma unroll
                for (int j = 0; j < 32; j++) sum[c0 + j] += v[j];
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&acce_bar[buf]));
        }
        if (ok && m < p.M) {
            float *row = p.c + (size_t)m * p.ldc;
#pragma unroll
            for (int j = 0; j < XN; j += 4) {
                const int n = n0 + j;
                if (n + 4 <= p.N) {
                    *reinterpret_cast<float4 *>(row + n) = make_float4(sum[j], sum[j + 1], sum[j + 2], sum[j + 3]);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (n + q < p.N) row[n + q] = sum[j + q];
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * XN) : "memory");
    }
}

// out[c][r] = in[r][c] for BF16 [R][C] (row strides ldi, ldo)
__global__ void transpose_bf16_kernel(const bf16 *__restrict__ in, int R, int Cc, int ldi, bf16 *__restrict__ out,
                                      int ldo)
{
    __shared__ bf16 tile[32][34];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        tile[y][threadIdx.x] = (r < R && c < Cc) ? in[(size_t)r * ldi + c] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (c < Cc && r < R) out[(size_t)c * ldo + r] = tile[threadIdx.x][y];
    }
}

// FP32 [R][C] (ld ldi) -> BF16 [R][C_pad] (ld ldo), zero columns C..C_pad
__global__ void to_bf16_kernel(const float *__restrict__ in, int R, int Cc, int ldi, int C_pad, bf16 *__restrict__ out,
                               int ldo)
{
    const int64_t total = (int64_t)R * C_pad;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / C_pad), c = (int)(t % C_pad);
        out[(size_t)r * ldo + c] = __float2bfloat16_rn(c < Cc ? in[(size_t)r * ldi + c] : 0.f);
    }
}

// Per-cell scale: mean of x over the n nodes (fixed order), or 1.
__global__ void cell_scale_kernel(const float *__restrict__ x, int n, int ld, int B, int use_mean,
                                  float *__restrict__ scale)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B) return;
    if (!use_mean) {
        scale[r] = 1.f;
        return;
    }
    float s = 0.f;
    for (int i = 0; i < n; i++) s += x[(size_t)i * ld + r];
    scale[r] = s / (float)n;
}

__device__ __forceinline__ float inv_or_zero(float s) { return s != 0.f ? 1.f / s : 0.f; }

// node-major FP32 x[i][r] (ld) -> cell-major BF16 xb[r][i] * gain / scale[r] (pad to n_p)
__global__ void gather_in_kernel(const float *__restrict__ x, int n, int ld, int B, const float *__restrict__ scale,
                                 float gain, bf16 *__restrict__ xb, int n_p)
{
    __shared__ float tile[32][33];
    const int i0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int i = i0 + y, r = r0 + threadIdx.x;
        tile[y][threadIdx.x] = (i < n && r < B) ? x[(size_t)i * ld + r] : 0.f;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, i = i0 + threadIdx.x;
        if (r < B && i < n_p) xb[(size_t)r * n_p + i] = __float2bfloat16_rn(tile[threadIdx.x][y] * (inv_or_zero(scale[r]) * gain));
    }
}

// node-major FP32 t[i][r] -> cell-major FP32 tt[r][i] * inv_gain / scale[r]^2 (the
// scale only when pw; pad to n_p)
__global__ void gather_target_kernel(const float *__restrict__ t, int n, int ld, int B, const float *__restrict__ scale,
                                     int pw, float inv_gain, float *__restrict__ tt, int n_p)
{
    __shared__ float tile[32][33];
    const int i0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int i = i0 + y, r = r0 + threadIdx.x;
        tile[y][threadIdx.x] = (i < n && r < B) ? t[(size_t)i * ld + r] : 0.f;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, i = i0 + threadIdx.x;
        if (r < B && i < n_p) {
            const float s = (pw ? inv_or_zero(scale[r] * scale[r]) : 1.f) * inv_gain;
            tt[(size_t)r * n_p + i] = tile[threadIdx.x][y] * s;
        }
    }
}

// cell-major FP32 y[r][i] (ld n_p) -> node-major out[i][r] * gain * scale[r]^2 (the scale
// only when pw)
__global__ void scatter_out_kernel(const float *__restrict__ y, int n_p, int n, int B, const float *__restrict__ scale,
                                   int pw, float gain, float *__restrict__ out, int ld)
{
    __shared__ float tile[32][33];
    const int i0 = blockIdx.y * 32, r0 = blockIdx.x * 32;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int r = r0 + yy, i = i0 + threadIdx.x;
        tile[yy][threadIdx.x] = (r < B && i < n) ? y[(size_t)r * n_p + i] : 0.f;
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int i = i0 + yy, r = r0 + threadIdx.x;
        if (i < n && r < B) {
            const float s = (pw ? scale[r] * scale[r] : 1.f) * gain;
            out[(size_t)i * ld + r] = tile[threadIdx.x][yy] * s;
        }
    }
}

// Loss denominators per cell: sum_i d[i][r]^2 (scaled like the targets) for the
// relative losses, or n for the mean squared error.
__global__ void row_den_kernel(const float *__restrict__ d, int n, int ld, int B, const float *__restrict__ scale,
                               int pw, float inv_gain, int mse, float *__restrict__ den)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= B) return;
    if (mse) {
        den[r] = (float)n;
        return;
    }
    float s = 0.f;
    for (int i = 0; i < n; i++) {
        const float v = d[(size_t)i * ld + r];
        s += v * v;
    }
    float sc = (pw ? inv_or_zero(scale[r] * scale[r]) : 1.f) * inv_gain;
    den[r] = s * sc * sc;
}

// den[r] <- mean over the batch of den (fixed order), for the batch-relative loss
__global__ void batch_mean_den_kernel(float *__restrict__ den, int B)
{
    __shared__ double s[256];
    double a = 0.0;
    for (int i = threadIdx.x; i < B; i += blockDim.x) a += den[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    const float m = (float)(s[0] / B);
    __syncthreads();
    for (int i = threadIdx.x; i < B; i += blockDim.x) den[i] = m;
}

// column sums out[n] = sum_r d[r][n], r < R (fixed order)
__global__ void colsum_kernel(const float *__restrict__ d, int R, int N, int ld, float *__restrict__ out)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int r = 0; r < R; r++) s += d[(size_t)r * ld + n];
    out[n] = s;
}

// e_r = sum_n (y - t)^2 / den_r; dy = 2 (y - t) / den_r / B.  One block per row.
__global__ void loss_grad_kernel(const float *__restrict__ y, const float *__restrict__ t, int ld, int N, int B,
                                 const float *__restrict__ den, float *__restrict__ dy, bf16 *__restrict__ dyb,
                                 float *__restrict__ row_err)
{
    __shared__ float s_e[256];
    const int r = blockIdx.x;
    const float dr = fmaxf(den[r], 1e-30f);
    float e = 0.f;
    for (int n = threadIdx.x; n < ld; n += blockDim.x) {
        float g = 0.f;
        if (n < N) {
            const float d = y[(size_t)r * ld + n] - t[(size_t)r * ld + n];
            e += d * d;
            g = 2.f * d / dr / (float)B;
        }
        dy[(size_t)r * ld + n] = g;
        dyb[(size_t)r * ld + n] = __float2bfloat16_rn(g);
    }
    s_e[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) s_e[threadIdx.x] += s_e[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) row_err[r] = s_e[0] / dr;
}

__global__ void mean_kernel(const float *__restrict__ v, int n, float *__restrict__ out)
{
    __shared__ double s[256];
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += v[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = (float)(s[0] / n);
}

// Adam (decoupled weight decay) on an FP32 master tensor; writes the BF16 copy.
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, bf16 *__restrict__ wb, int64_t n, float lr, float b1, float b2,
                            float c1, float c2, float eps, float wd)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float upd = (mi / c1) / (sqrtf(vi / c2) + eps) + wd * w[i];
        const float wn = w[i] - lr * upd;
        w[i] = wn;
        if (wb) wb[i] = __float2bfloat16_rn(wn);
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder()
{
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// 2-D map over a K-major BF16 matrix [rows][K] (row stride K), box 64 x box_rows
int make_map(CUtensorMap *m, const bf16 *ptr, int rows, int K, int box_rows)
{
    EncodeTiled fn = encoder();
    if (!fn) return set_error(GD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t str[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {GK, (cuuint32_t)box_rows}, es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(ptr), dims, str, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GD_ERR_CUDA, "tensor map encoding failed (" + std::to_string((int)r) + ")");
    return GD_OK;
}

// C = A B^T with A [M][K], B [N][K] (BF16, row stride K), K % 64 == 0;
// output strides ld32, ld16 multiples of 4.
int gemm_nt(int epi, const bf16 *A, const bf16 *B, const GemmArgs &a, cudaStream_t st)
{
    if (a.K % GK || a.K <= 0 || a.M <= 0 || a.N <= 0 || (a.ld32 & 3) || (a.ld16 & 3))
        return set_error(GD_ERR_INVALID_ARG, "GEMM shape: K a multiple of 64, strides multiples of 4");
    CUtensorMap tA, tB;
    int rc = make_map(&tA, A, a.M, a.K, GM);
    if (!rc) rc = make_map(&tB, B, a.N, a.K, GN);
    if (rc) return rc;
    dim3 grid((a.M + GM - 1) / GM, (a.N + GN - 1) / GN);
    switch (epi) {
#define GD_GEMM_CASE(E)                                                                                          \
    case E:                                                                                                      \
        GD_CUDA(cudaFuncSetAttribute(gemm_nt_kernel<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem)); \
        gemm_nt_kernel<E><<<grid, kGThreads, kGemmSmem, st>>>(tA, tB, a);                                        \
        break;
        GD_GEMM_CASE(EPI_NONE)
        GD_GEMM_CASE(EPI_GELU)
        GD_GEMM_CASE(EPI_DGELU)
#undef GD_GEMM_CASE
    default:
        return set_error(GD_ERR_INVALID_ARG, "unknown GEMM epilogue");
    }
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

int transpose(const bf16 *in, int R, int Cc, int ldi, bf16 *out, int ldo, cudaStream_t st)
{
    dim3 b(32, 8), g((Cc + 31) / 32, (R + 31) / 32);
    transpose_bf16_kernel<<<g, b, 0, st>>>(in, R, Cc, ldi, out, ldo);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

int pad64(int n) { return (n + 63) / 64 * 64; }

}  // namespace

// C[M][N] (FP32, row stride ldc) = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T for
// K-major BF16 [M][K] and [N][K] operands, in one launch, the tensor cores
// summing at most k_chunk products per FP32 accumulation (the chunks added in
// FP32 in chunk order); the collision-matrix path computes the loss with it.
int gemm_bf16x3_nt_f32(const void *Ah, const void *Al, int M, const void *Bh, const void *Bl, int N, int K, float *C,
                       int ldc, int *err, cudaStream_t st, int stall_polls, int k_chunk)
{
    if (K % GK || K <= 0 || M <= 0 || N <= 0 || (ldc & 3) || k_chunk <= 0 || k_chunk % GK ||
        (reinterpret_cast<uintptr_t>(C) & 15))
        return set_error(GD_ERR_INVALID_ARG, "GEMM shape: K and the chunk multiples of 64, ldc a multiple of 4");
    CUtensorMap tAh, tAl, tBh, tBl;
    int rc = make_map(&tAh, static_cast<const bf16 *>(Ah), M, K, XM);
    if (!rc) rc = make_map(&tAl, static_cast<const bf16 *>(Al), M, K, XM);
    if (!rc) rc = make_map(&tBh, static_cast<const bf16 *>(Bh), N, K, XN);
    if (!rc) rc = make_map(&tBl, static_cast<const bf16 *>(Bl), N, K, XN);
    if (rc) return rc;
    Gemm3Args a{M, N, K, k_chunk, C, ldc, err, stall_polls};
    dim3 grid((M + XM - 1) / XM, (N + XN - 1) / XN);
    GD_CUDA(cudaFuncSetAttribute(gemm3_nt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kX3Smem));
    gemm3_nt_kernel<<<grid, kGThreads, kX3Smem, st>>>(tAh, tAl, tBh, tBl, a);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

}  // namespace gd

using gd::bf16;

struct gd_mlp {
    struct Layer {
        int out = 0, in = 0;  // padded
        float *w = nullptr, *b = nullptr, *gw = nullptr, *gb = nullptr;
        float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
        bf16 *wb = nullptr, *wt = nullptr;  // BF16 copy [out][in] and its transpose [in][out]
    };
    int n_in = 0, n_out = 0, n_in_p = 0, n_out_p = 0, cap = 0, flags = 0;
    int device = 0;
    float in_gain = 1.f, out_gain = 1.f;  // global input / output normalisation
    Layer L[5];
    int64_t step = 0;
    int stall_next = 0;  // gd_mlp_inject_timeout: polls for the next forward's first GEMM
    // activations, [cap][features]
    bf16 *xb = nullptr, *h0b = nullptr, *h1b = nullptr, *h2b = nullptr, *zb = nullptr;
    float *h0 = nullptr, *a1 = nullptr, *a2 = nullptr, *y = nullptr, *tt = nullptr;
    float *dy = nullptr, *dz = nullptr, *da2 = nullptr, *da1 = nullptr, *dh0 = nullptr;
    bf16 *dyb = nullptr, *dzb = nullptr, *da2b = nullptr, *da1b = nullptr, *dh0b = nullptr;
    bf16 *tmp1 = nullptr, *tmp2 = nullptr;  // transposes [features][cap]
    float *scale = nullptr, *den = nullptr, *row_err = nullptr;
    int *err = nullptr;
    std::vector<void *> allocs;
};

namespace {

int mlp_alloc(gd_mlp *h, void **p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return gd::cuda_error(e, "surrogate allocation");
    h->allocs.push_back(*p);
    return GD_OK;
}

template <typename T>
int alloc_n(gd_mlp *h, T **p, size_t n)
{
    return mlp_alloc(h, reinterpret_cast<void **>(p), n * sizeof(T));
}

void layer_dims(const gd_mlp *h, int k, int *out, int *in)
{
    const int dims[5][2] = {{256, h->n_in_p}, {512, 256}, {512, 512}, {256, 512}, {h->n_out_p, 256}};
    *out = dims[k][0];
    *in = dims[k][1];
}

int refresh_bf16(gd_mlp *h, cudaStream_t st)
{
    for (int k = 0; k < 5; k++) {
        gd_mlp::Layer &l = h->L[k];
        const int64_t n = (int64_t)l.out * l.in;
        gd::to_bf16_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(l.w, l.out, l.in, l.in, l.in,
                                                                                           l.wb, l.in);
        GD_CUDA(cudaGetLastError());
        if (k > 0) {
            int rc = gd::transpose(l.wb, l.out, l.in, l.in, l.wt, l.out, st);
            if (rc) return rc;
        }
    }
    return GD_OK;
}

gd::GemmArgs args(int M, int N, int K, int *err)
{
    gd::GemmArgs a{};
    a.M = M;
    a.N = N;
    a.K = K;
    a.err = err;
    return a;
}

// network input: per-cell scales and the BF16 cell-major copy of x
int load_input(gd_mlp *h, const float *x, int ldx, int B, cudaStream_t st)
{
    gd::cell_scale_kernel<<<(B + 127) / 128, 128, 0, st>>>(x, h->n_in, ldx, B, h->flags & GD_MLP_SCALE_INPUT,
                                                           h->scale);
    dim3 blk(32, 8), grd((B + 31) / 32, h->n_in_p / 32);
    gd::gather_in_kernel<<<grd, blk, 0, st>>>(x, h->n_in, ldx, B, h->scale, h->in_gain, h->xb, h->n_in_p);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

// forward on rows [0, B) of h->xb; y (FP32, [B][n_out_p]) into h->y
int forward(gd_mlp *h, int B, cudaStream_t st)
{
    using namespace gd;
    int rc;
    GemmArgs a = args(B, 256, h->n_in_p, h->err);
    a.stall_polls = h->stall_next;  // a pending time-out injection fires here, once
    h->stall_next = 0;
    a.bias = h->L[0].b;
    a.c32 = h->h0;
    a.ld32 = 256;
    a.c16 = h->h0b;
    a.ld16 = 256;
    if ((rc = gemm_nt(EPI_NONE, h->xb, h->L[0].wb, a, st))) return rc;
    a = args(B, 512, 256, h->err);
    a.bias = h->L[1].b;
    a.pre_out = h->a1;
    a.ld32 = 512;
    a.c16 = h->h1b;
    a.ld16 = 512;
    if ((rc = gemm_nt(EPI_GELU, h->h0b, h->L[1].wb, a, st))) return rc;
    a = args(B, 512, 512, h->err);
    a.bias = h->L[2].b;
    a.pre_out = h->a2;
    a.ld32 = 512;
    a.c16 = h->h2b;
    a.ld16 = 512;
    if ((rc = gemm_nt(EPI_GELU, h->h1b, h->L[2].wb, a, st))) return rc;
    a = args(B, 256, 512, h->err);
    a.bias = h->L[3].b;
    a.add = h->h0;
    a.ld32 = 256;
    a.c16 = h->zb;
    a.ld16 = 256;
    if ((rc = gemm_nt(EPI_NONE, h->h2b, h->L[3].wb, a, st))) return rc;
    a = args(B, h->n_out_p, 256, h->err);
    a.bias = h->L[4].b;
    a.c32 = h->y;
    a.ld32 = h->n_out_p;
    return gemm_nt(EPI_NONE, h->zb, h->L[4].wb, a, st);
}

int backward(gd_mlp *h, int B, cudaStream_t st)
{
    using namespace gd;
    int rc;
    auto grad_w = [&](int k, const bf16 *dY, int nout, const bf16 *X, int nin) -> int {
        // dW[o][i] = sum_b dY[b][o] X[b][i]: A = dY^T [nout][B], B = X^T [nin][B]
        int r = transpose(dY, B, nout, nout, h->tmp1, B, st);
        if (!r) r = transpose(X, B, nin, nin, h->tmp2, B, st);
        if (r) return r;
        GemmArgs a = args(nout, nin, B, h->err);
        a.c32 = h->L[k].gw;
        a.ld32 = nin;
        return gemm_nt(EPI_NONE, h->tmp1, h->tmp2, a, st);
    };
    auto grad_b = [&](int k, const float *dY, int n) -> int {
        colsum_kernel<<<(n + 127) / 128, 128, 0, st>>>(dY, B, n, n, h->L[k].gb);
        GD_CUDA(cudaGetLastError());
        return GD_OK;
    };
    // y = W4 z + b4
    if ((rc = grad_w(4, h->dyb, h->n_out_p, h->zb, 256)) || (rc = grad_b(4, h->dy, h->n_out_p))) return rc;
    GemmArgs a = args(B, 256, h->n_out_p, h->err);
    a.c32 = h->dz;
    a.ld32 = 256;
    a.c16 = h->dzb;
    a.ld16 = 256;
    if ((rc = gemm_nt(EPI_NONE, h->dyb, h->L[4].wt, a, st))) return rc;
    // z = W3 h2 + b3 + h0
    if ((rc = grad_w(3, h->dzb, 256, h->h2b, 512)) || (rc = grad_b(3, h->dz, 256))) return rc;
    a = args(B, 512, 256, h->err);
    a.aux = h->a2;
    a.c32 = h->da2;
    a.ld32 = 512;
    a.c16 = h->da2b;
    a.ld16 = 512;
    if ((rc = gemm_nt(EPI_DGELU, h->dzb, h->L[3].wt, a, st))) return rc;
    // h2 = GELU(W2 h1 + b2)
    if ((rc = grad_w(2, h->da2b, 512, h->h1b, 512)) || (rc = grad_b(2, h->da2, 512))) return rc;
    a = args(B, 512, 512, h->err);
    a.aux = h->a1;
    a.c32 = h->da1;
    a.ld32 = 512;
    a.c16 = h->da1b;
    a.ld16 = 512;
    if ((rc = gemm_nt(EPI_DGELU, h->da2b, h->L[2].wt, a, st))) return rc;
    // h1 = GELU(W1 h0 + b1); dh0 also receives dz through the residual
    if ((rc = grad_w(1, h->da1b, 512, h->h0b, 256)) || (rc = grad_b(1, h->da1, 512))) return rc;
    a = args(B, 256, 512, h->err);
    a.add = h->dz;
    a.c32 = h->dh0;
    a.ld32 = 256;
    a.c16 = h->dh0b;
    a.ld16 = 256;
    if ((rc = gemm_nt(EPI_NONE, h->da1b, h->L[1].wt, a, st))) return rc;
    // h0 = W0 x + b0
    if ((rc = grad_w(0, h->dh0b, 256, h->xb, h->n_in_p)) || (rc = grad_b(0, h->dh0, 256))) return rc;
    return GD_OK;
}

// loss and output gradient for targets t (loss denominators from tden, or t)
int loss_grad(gd_mlp *h, const float *t, int ldt, const float *tden, int ldd, int B, cudaStream_t st)
{
    const int pw = (h->flags & GD_MLP_SCALE_OUTPUT) ? 1 : 0;
    const int mse = (h->flags & GD_MLP_LOSS_MSE) ? 1 : 0;
    dim3 blk(32, 8), grd((B + 31) / 32, h->n_out_p / 32);
    const float inv_gain = 1.f / h->out_gain;
    gd::gather_target_kernel<<<grd, blk, 0, st>>>(t, h->n_out, ldt, B, h->scale, pw, inv_gain, h->tt, h->n_out_p);
    gd::row_den_kernel<<<(B + 127) / 128, 128, 0, st>>>(tden ? tden : t, h->n_out, tden ? ldd : ldt, B, h->scale, pw,
                                                        inv_gain, mse, h->den);
    if (!mse && (h->flags & GD_MLP_LOSS_BATCH)) gd::batch_mean_den_kernel<<<1, 256, 0, st>>>(h->den, B);
    gd::loss_grad_kernel<<<B, 256, 0, st>>>(h->y, h->tt, h->n_out_p, h->n_out, B, h->den, h->dy, h->dyb, h->row_err);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

int check_err(gd_mlp *h, cudaStream_t st)
{
    int flag = 0;
    GD_CUDA(cudaMemcpyAsync(&flag, h->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GD_CUDA(cudaStreamSynchronize(st));
    if (flag) {
        // clear the record so that later calls start clean
        GD_CUDA(cudaMemsetAsync(h->err, 0, sizeof(int), st));
        GD_CUDA(cudaStreamSynchronize(st));
        return gd::set_error(GD_ERR_CUDA, "surrogate GEMM: a pipeline wait timed out");
    }
    return GD_OK;
}

}  // namespace

extern "C" int gd_mlp_create(int n_in, int n_out, int batch_cap, int flags, uint64_t seed, gd_mlp **out)
{
    using namespace gd;
    if (!out) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (n_in < 1 || n_out < 1 || n_in > (1 << 16) || n_out > (1 << 16) || batch_cap < 64 || batch_cap % 64 ||
        (flags & ~(GD_MLP_SCALE_INPUT | GD_MLP_SCALE_OUTPUT | GD_MLP_LOSS_MSE | GD_MLP_LOSS_BATCH)))
        return set_error(GD_ERR_INVALID_ARG,
                         "need 1 <= n_in, n_out <= 65536, batch_cap a positive multiple of 64 and known flags");
    if ((flags & GD_MLP_SCALE_OUTPUT) && !(flags & GD_MLP_SCALE_INPUT))
        return set_error(GD_ERR_INVALID_ARG, "GD_MLP_SCALE_OUTPUT needs GD_MLP_SCALE_INPUT");
    {
        // parameters (FP32 master, gradient, two Adam moments, BF16 copy and
        // transpose) and activations, for the memory limit
        const double np = 256.0 * pad64(n_in) + 512.0 * 256 + 512.0 * 512 + 256.0 * 512 + 256.0 * pad64(n_out);
        const double acts = (double)batch_cap * (6.0 * pad64(n_in) + 14.0 * pad64(n_out) + 12000.0);
        const size_t limit = memory_limit();
        if (limit && np * 20.0 + acts > (double)limit)
            return set_error(GD_ERR_OUT_OF_MEMORY, "the surrogate network exceeds the library's memory limit");
    }
    gd_mlp *h = new gd_mlp();
    h->n_in = n_in;
    h->n_out = n_out;
    h->n_in_p = pad64(n_in);
    h->n_out_p = pad64(n_out);
    h->cap = batch_cap;
    h->flags = flags;
    cudaGetDevice(&h->device);
    int rc = GD_OK;
    // 64-bit LCG; uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) on the true inputs
    uint64_t state = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto uni = [&]() {
        state = state * 6364136223846793005ull + 1442695040888963407ull;
        return (float)(((state >> 11) + 0.5) * (1.0 / 9007199254740992.0));
    };
    for (int k = 0; k < 5 && !rc; k++) {
        gd_mlp::Layer &l = h->L[k];
        layer_dims(h, k, &l.out, &l.in);
        const size_t n = (size_t)l.out * l.in;
        if (!rc) rc = alloc_n(h, &l.w, n);
        if (!rc) rc = alloc_n(h, &l.gw, n);
        if (!rc) rc = alloc_n(h, &l.mw, n);
        if (!rc) rc = alloc_n(h, &l.vw, n);
        if (!rc) rc = alloc_n(h, &l.b, l.out);
        if (!rc) rc = alloc_n(h, &l.gb, l.out);
        if (!rc) rc = alloc_n(h, &l.mb, l.out);
        if (!rc) rc = alloc_n(h, &l.vb, l.out);
        if (!rc) rc = alloc_n(h, &l.wb, n);
        if (!rc) rc = alloc_n(h, &l.wt, n);
        if (rc) break;
        const int fan_in = k == 0 ? n_in : l.in;
        const float bound = 1.f / std::sqrt((float)fan_in);
        std::vector<float> w(n, 0.f);
        for (int o = 0; o < l.out; o++)
            for (int i = 0; i < l.in; i++) {
                const bool real = (k != 0 || i < n_in) && (k != 4 || o < n_out);
                const float r = (2.f * uni() - 1.f) * bound;
                w[(size_t)o * l.in + i] = real ? r : 0.f;
            }
        if (cudaMemcpy(l.w, w.data(), n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(l.b, 0, l.out * sizeof(float)) != cudaSuccess ||
            cudaMemset(l.mw, 0, n * sizeof(float)) != cudaSuccess ||
            cudaMemset(l.vw, 0, n * sizeof(float)) != cudaSuccess ||
            cudaMemset(l.mb, 0, l.out * sizeof(float)) != cudaSuccess ||
            cudaMemset(l.vb, 0, l.out * sizeof(float)) != cudaSuccess)
            rc = set_error(GD_ERR_CUDA, "surrogate weight upload");
    }
    const size_t c = h->cap;
    if (!rc) rc = alloc_n(h, &h->xb, c * h->n_in_p);
    if (!rc) rc = alloc_n(h, &h->h0b, c * 256);
    if (!rc) rc = alloc_n(h, &h->h1b, c * 512);
    if (!rc) rc = alloc_n(h, &h->h2b, c * 512);
    if (!rc) rc = alloc_n(h, &h->zb, c * 256);
    if (!rc) rc = alloc_n(h, &h->h0, c * 256);
    if (!rc) rc = alloc_n(h, &h->a1, c * 512);
    if (!rc) rc = alloc_n(h, &h->a2, c * 512);
    if (!rc) rc = alloc_n(h, &h->y, c * h->n_out_p);
    if (!rc) rc = alloc_n(h, &h->tt, c * h->n_out_p);
    if (!rc) rc = alloc_n(h, &h->dy, c * h->n_out_p);
    if (!rc) rc = alloc_n(h, &h->dyb, c * h->n_out_p);
    if (!rc) rc = alloc_n(h, &h->dz, c * 256);
    if (!rc) rc = alloc_n(h, &h->dzb, c * 256);
    if (!rc) rc = alloc_n(h, &h->da2, c * 512);
    if (!rc) rc = alloc_n(h, &h->da2b, c * 512);
    if (!rc) rc = alloc_n(h, &h->da1, c * 512);
    if (!rc) rc = alloc_n(h, &h->da1b, c * 512);
    if (!rc) rc = alloc_n(h, &h->dh0, c * 256);
    if (!rc) rc = alloc_n(h, &h->dh0b, c * 256);
    const size_t widest = (size_t)std::max(h->n_in_p, std::max(h->n_out_p, 512));
    if (!rc) rc = alloc_n(h, &h->tmp1, c * widest);
    if (!rc) rc = alloc_n(h, &h->tmp2, c * widest);
    if (!rc) rc = alloc_n(h, &h->scale, c);
    if (!rc) rc = alloc_n(h, &h->den, c);
    if (!rc) rc = alloc_n(h, &h->row_err, c);
    if (!rc) rc = alloc_n(h, &h->err, 1);
    if (!rc && cudaMemset(h->err, 0, sizeof(int)) != cudaSuccess) rc = set_error(GD_ERR_CUDA, "memset");
    if (!rc) rc = refresh_bf16(h, nullptr);
    if (!rc && cudaDeviceSynchronize() != cudaSuccess) rc = set_error(GD_ERR_CUDA, "surrogate set-up");
    if (rc) {
        for (void *p : h->allocs) cudaFree(p);
        delete h;
        return rc;
    }
    *out = h;
    return GD_OK;
}

extern "C" int gd_mlp_set_io_scale(gd_mlp *h, float in_gain, float out_gain)
{
    if (!h) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (!(in_gain > 0.f) || !(out_gain > 0.f) || !std::isfinite(in_gain) || !std::isfinite(out_gain))
        return gd::set_error(GD_ERR_INVALID_ARG, "input and output gains must be finite and > 0");
    h->in_gain = in_gain;
    h->out_gain = out_gain;
    return GD_OK;
}

extern "C" int gd_mlp_destroy(gd_mlp *h)
{
    if (!h) return GD_OK;
    gd::DeviceGuard ds(h->device);
    for (void *p : h->allocs) cudaFree(p);
    delete h;
    return GD_OK;
}

extern "C" int gd_mlp_info(const gd_mlp *h, gd_mlp_info_t *info)
{
    if (!h || !info) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    info->n_in = h->n_in;
    info->n_out = h->n_out;
    info->n_in_padded = h->n_in_p;
    info->n_out_padded = h->n_out_p;
    info->batch_cap = h->cap;
    info->flags = h->flags;
    info->steps = h->step;
    info->in_gain = h->in_gain;
    info->out_gain = h->out_gain;
    int64_t s = 0;
    double fl = 0.0;
    for (int k = 0; k < 5; k++) {
        s += (int64_t)h->L[k].out * h->L[k].in + h->L[k].out;
        fl += 2.0 * h->L[k].out * h->L[k].in;
    }
    info->num_params = s;
    info->forward_flop_per_cell = fl;
    return GD_OK;
}

extern "C" int gd_mlp_forward(gd_mlp *h, const float *x, int ldx, int batch, float *y, int ldy, gd_stream stream)
{
    using namespace gd;
    if (!h || !x || !y || batch < 1 || batch > h->cap || ldx < batch || ldy < batch)
        return set_error(GD_ERR_INVALID_ARG, "bad surrogate forward arguments (1 <= batch <= cap, ld >= batch)");
    gd::DeviceGuard ds(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = load_input(h, x, ldx, batch, st);
    if (!rc) rc = forward(h, batch, st);
    if (rc) return rc;
    dim3 blk(32, 8), grd((batch + 31) / 32, h->n_out_p / 32);
    scatter_out_kernel<<<grd, blk, 0, st>>>(h->y, h->n_out_p, h->n_out, batch, h->scale,
                                            (h->flags & GD_MLP_SCALE_OUTPUT) ? 1 : 0, h->out_gain, y, ldy);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

extern "C" int gd_mlp_train_step(gd_mlp *h, const float *x, int ldx, const float *t, int ldt, const float *tden,
                                 int ldd, int batch, float lr, float weight_decay, float *loss, gd_stream stream)
{
    using namespace gd;
    if (!h || !x || !t || batch < 64 || batch > h->cap || batch % 64 || ldx < batch || ldt < batch ||
        (tden && ldd < batch))
        return set_error(GD_ERR_INVALID_ARG, "bad surrogate training arguments (batch a multiple of 64, <= cap)");
    gd::DeviceGuard ds(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = load_input(h, x, ldx, batch, st);
    if (!rc) rc = forward(h, batch, st);
    if (!rc) rc = loss_grad(h, t, ldt, tden, ldd, batch, st);
    if (rc) return rc;
    if (loss) {
        mean_kernel<<<1, 256, 0, st>>>(h->row_err, batch, loss);
        GD_CUDA(cudaGetLastError());
    }
    if ((rc = backward(h, batch, st))) return rc;
    h->step++;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - (float)std::pow(0.9, (double)h->step), c2 = 1.f - (float)std::pow(0.999, (double)h->step);
    for (int k = 0; k < 5; k++) {
        gd_mlp::Layer &l = h->L[k];
        const int64_t nw = (int64_t)l.out * l.in;
        adam_kernel<<<(int)std::min<int64_t>((nw + 255) / 256, 4096), 256, 0, st>>>(l.w, l.gw, l.mw, l.vw, l.wb, nw, lr, b1,
                                                                                     b2, c1, c2, eps, weight_decay);
        adam_kernel<<<(l.out + 255) / 256, 256, 0, st>>>(l.b, l.gb, l.mb, l.vb, nullptr, l.out, lr, b1, b2, c1, c2, eps,
                                                         0.f);
        GD_CUDA(cudaGetLastError());
        if (k > 0 && (rc = transpose(l.wb, l.out, l.in, l.in, l.wt, l.out, st))) return rc;
    }
    return GD_OK;
}

extern "C" int gd_mlp_loss(gd_mlp *h, const float *x, int ldx, const float *t, int ldt, const float *tden, int ldd,
                           int batch, float *row_loss, gd_stream stream)
{
    using namespace gd;
    if (!h || !x || !t || !row_loss || batch < 1 || batch > h->cap || ldx < batch || ldt < batch ||
        (tden && ldd < batch))
        return set_error(GD_ERR_INVALID_ARG, "bad surrogate loss arguments");
    gd::DeviceGuard ds(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = load_input(h, x, ldx, batch, st);
    if (!rc) rc = forward(h, batch, st);
    if (!rc) rc = loss_grad(h, t, ldt, tden, ldd, batch, st);
    if (rc) return rc;
    GD_CUDA(cudaMemcpyAsync(row_loss, h->row_err, (size_t)batch * sizeof(float), cudaMemcpyDeviceToDevice, st));
    return GD_OK;
}

extern "C" int gd_mlp_check(gd_mlp *h, gd_stream stream)
{
    if (!h) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    gd::DeviceGuard ds(h->device);
    return check_err(h, (cudaStream_t)stream);
}

// FP32 parameter block: for each layer k = 0..4, W_k [out][in] then b_k [out],
// with n_in and n_out padded to multiples of 64 (padding entries are zero).
static int copy_params(gd_mlp *h, float *host, bool to_host, bool grads)
{
    gd::DeviceGuard ds(h->device);
    size_t off = 0;
    for (int k = 0; k < 5; k++) {
        gd_mlp::Layer &l = h->L[k];
        const size_t nw = (size_t)l.out * l.in;
        float *w = grads ? l.gw : l.w, *b = grads ? l.gb : l.b;
        cudaError_t e = to_host ? cudaMemcpy(host + off, w, nw * 4, cudaMemcpyDeviceToHost)
                                : cudaMemcpy(w, host + off, nw * 4, cudaMemcpyHostToDevice);
        off += nw;
        if (e == cudaSuccess)
            e = to_host ? cudaMemcpy(host + off, b, l.out * 4, cudaMemcpyDeviceToHost)
                        : cudaMemcpy(b, host + off, l.out * 4, cudaMemcpyHostToDevice);
        off += l.out;
        if (e != cudaSuccess) return gd::cuda_error(e, "surrogate parameter copy");
    }
    return GD_OK;
}

extern "C" int gd_mlp_get_params(gd_mlp *h, float *host)
{
    if (!h || !host) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    return copy_params(h, host, true, false);
}

extern "C" int gd_mlp_set_params(gd_mlp *h, const float *host)
{
    if (!h || !host) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    int rc = copy_params(h, const_cast<float *>(host), false, false);
    if (rc) return rc;
    gd::DeviceGuard ds(h->device);
    if ((rc = refresh_bf16(h, nullptr))) return rc;
    if (cudaDeviceSynchronize() != cudaSuccess) return gd::set_error(GD_ERR_CUDA, "surrogate parameter refresh");
    return GD_OK;
}

extern "C" int gd_mlp_get_grads(gd_mlp *h, float *host)
{
    if (!h || !host) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    return copy_params(h, host, true, true);
}

extern "C" int gd_mlp_inject_timeout(gd_mlp *h, int polls)
{
    using namespace gd;
    if (!h || polls < 1 || polls > (1 << 20))
        return set_error(GD_ERR_INVALID_ARG, "gd_mlp_inject_timeout: need a network and 1 <= polls <= 2^20");
    h->stall_next = polls;
    return GD_OK;
}
