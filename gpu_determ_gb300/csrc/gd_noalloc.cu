// gd_noalloc.cu -- gain term without any device allocation per call.
//
// gd_collision computes the gain with a partial-sum buffer that the context
// grows with cudaMalloc on the first call for a larger batch (and frees and
// synchronises the device when it grows).  Some callers cannot allow that:
// code that runs while a custom allocator or memory pool owns device
// memory, latency-critical loops that must not hit cudaMalloc's implicit
// synchronisation, or hosts that forbid allocation after start-up.  For them,
// gd_gain_noalloc runs the same gain kernel on a fixed scratch area that is
// part of the library image: a file-scope __device__ array of
// kNoAllocScratchBytes, which every GPU that loads this library holds until
// the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it; make
// that first call before any stream capture.  With lazy module loading (the
// CUDA default) that lookup is also what loads this library's device code on
// the device, and so reserves the 64 MiB array there: a caller that wants no
// allocation of any kind inside its hot loop makes one warm-up call at
// start-up.  Later calls only launch kernels and clear the partial sums with
// cudaMemsetAsync.
//
// The chunking of the s walk is the one gd_collision picks when it fits the
// array (at most kMaxChunks chunks); then the result is bitwise that of
// gd_collision's FP32 pair gain.  When it does not fit, fewer chunks are
// used, and the sums agree within FP32 rounding of the other order.
//
// All calls share the one array and it keeps the last call's contents; the
// partial sums are cleared at the start of every call.  Calls whose work
// overlaps on the GPU (different streams, or different host threads without
// ordering) race on the array and give wrong results: order them.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "gd_internal.h"


namespace gd {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB
constexpr int kMaxChunks = 64;
constexpr size_t kHeaderBytes = 512;  // chunk boundaries, then the partial sums
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_gain_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

struct ChunkBounds {
    int v[kMaxChunks + 1];
    int n;
};

__global__ void write_bounds_kernel(ChunkBounds b, int *dst)
{
    const int t = threadIdx.x;
    if (t <= b.n) dst[t] = b.v[t];
}

// Device address of g_gain_scratch on `dev` (which is current), looked up once.
int scratch_address(int dev, void **out)
{
    if (dev < 0 || dev >= kMaxDevices) return set_error(GD_ERR_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_gain_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_gain_scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GD_OK;
}

}  // namespace
}  // namespace gd

extern "C" int gd_gain_noalloc(gd_ctx *ctx, const float *f, int ncells, int ld, float *gain,
                               gd_stream stream)
{
    using namespace gd;
    if (!ctx || !f || !gain) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ncells < 1 || ld < ncells) return set_error(GD_ERR_INVALID_ARG, "need 1 <= ncells <= ld");
    Context &c = ctx->c;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != c.device && cudaSetDevice(c.device) != cudaSuccess)
        return set_error(GD_ERR_CUDA, "cudaSetDevice failed");
    int rc = GD_OK;
    do {
        int cb = 0, nblk = 0, want = 0;
        size_t smem = 0;
        if ((rc = gain_launch_shape(c, ncells, &cb, &smem, &nblk, &want))) break;
        const size_t per_chunk = (size_t)c.d.n_pnt * nblk * cb * sizeof(float);
        const size_t room = kNoAllocScratchBytes - kHeaderBytes;
        const int fit = (int)std::min<size_t>(room / per_chunk, kMaxChunks);
        if (fit < 1) {
            const size_t max_cells = room / ((size_t)c.d.n_pnt * sizeof(float)) / cb * cb;
            rc = set_error(GD_ERR_UNSUPPORTED,
                           "gd_gain_noalloc: " + std::to_string(ncells) + " cells need " +
                               std::to_string(per_chunk) + " bytes of partial sums; its fixed scratch holds " +
                               std::to_string(room) + " bytes (at most " + std::to_string(max_cells) +
                               " cells on this grid) -- split the batch or use gd_collision");
            break;
        }
        const int nchunks = std::min(want, fit);
        void *base = nullptr;
        if ((rc = scratch_address(c.device, &base))) break;
        int *d_bounds = static_cast<int *>(base);
        float *part = reinterpret_cast<float *>(static_cast<unsigned char *>(base) + kHeaderBytes);
        ChunkBounds b{};
        b.n = nchunks;
        gain_chunk_bounds(c, nchunks, b.v);
        cudaStream_t st = (cudaStream_t)stream;
        write_bounds_kernel<<<1, kMaxChunks + 1, 0, st>>>(b, d_bounds);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            rc = cuda_error(e, "write_bounds_kernel");
            break;
        }
        rc = launch_gain_pair(c, f, ncells, ld, gain, part, nchunks, d_bounds, cb, smem, st);
    } while (0);
    if (prev >= 0 && prev != c.device) cudaSetDevice(prev);
    return rc;
}
