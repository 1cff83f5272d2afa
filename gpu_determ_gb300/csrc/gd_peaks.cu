// gd_peaks.cu -- FP32 and FP64 fused multiply-add throughput of the device.
//
// The SIMT kernels of this library (the FP32 pair-product gain, the SIMT part
// of the pair kernel on the tensor cores, the FP64 projection) are measured
// against the FMA throughput of the GPU they run on, not against the BF16
// tensor-core peak.  This microbenchmark measures that throughput: every
// thread runs eight independent FMA chains (a = a * m + c, m slightly below
// one so the values stay bounded) unrolled 16 deep, on enough resident warps
// to cover the FMA latency, and the best of five timed launches (CUDA events)
// gives FLOP/s with 2 FLOP per FMA.  The reference measures nothing of the
// kind (its GpuTimer only times whole phases, gputimer.hpp:10-46).
#include <cuda_runtime.h>

#include <algorithm>

#include "gd_internal.h"

namespace gd {
namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;
constexpr int kPeakThreads = 256;

template <typename T>
__device__ __forceinline__ T fma_rn(T a, T b, T c);
template <>
__device__ __forceinline__ float fma_rn<float>(float a, float b, float c)
{
    return __fmaf_rn(a, b, c);
}
template <>
__device__ __forceinline__ double fma_rn<double>(double a, double b, double c)
{
    return __fma_rn(a, b, c);
}

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) fma_peak_kernel(T seed, int iters, T *sink)
{
    T a[kChains];
    const T m = seed * (T)0.999, c = seed * (T)1e-3;
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = seed + (T)(threadIdx.x + k);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < kUnroll; u++) {
#pragma unroll
            for (int k = 0; k < kChains; k++) a[k] = fma_rn<T>(a[k], m, c);
        }
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < kChains; k++) s += a[k];
    // never true for the seeds used (the chains converge to c / (1 - m) > 0),
    // but the compiler cannot know: the chains stay live
    if (s == (T)-1) sink[blockIdx.x] = s;
}

template <typename T>
int run_peak(int sms, int iters, double *flops)
{
    T *sink = nullptr;
    GD_CUDA(cudaMalloc(&sink, sizeof(T) * (size_t)sms * 8));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = GD_OK;
    const int blocks = sms * 8;  // 2048 resident threads per SM at 256-thread blocks
    double best = 0.0;
    do {
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            rc = set_error(GD_ERR_CUDA, "cudaEventCreate failed");
            break;
        }
        fma_peak_kernel<T><<<blocks, kPeakThreads>>>((T)1.0, iters, sink);  // warm-up
        for (int r = 0; r < 5 && rc == GD_OK; r++) {
            cudaEventRecord(e0);
            fma_peak_kernel<T><<<blocks, kPeakThreads>>>((T)1.0, iters, sink);
            cudaEventRecord(e1);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                rc = cuda_error(e, "fma_peak_kernel");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            const double flop = 2.0 * kChains * kUnroll * (double)iters * blocks * kPeakThreads;
            if (ms > 0.f) best = std::max(best, flop / (ms * 1e-3));
        }
    } while (0);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    *flops = best;
    return rc;
}

}  // namespace
}  // namespace gd

extern "C" int gd_fma_peak(int device, int precision, double *flops_per_s)
{
    using namespace gd;
    if (!flops_per_s || (precision != 32 && precision != 64))
        return set_error(GD_ERR_INVALID_ARG, "gd_fma_peak: precision is 32 or 64");
    DeviceGuard g(device);
    if (!g.ok) return set_error(GD_ERR_CUDA, "cudaSetDevice failed");
    int sms = 0;
    GD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    // about 30 ms per launch at the nominal rates (FP64 runs far slower)
    return precision == 32 ? run_peak<float>(sms, 40000, flops_per_s) : run_peak<double>(sms, 600, flops_per_s);
}
