// gd_layout.cu -- conversion between the reference's full-box layout
// f[(i*ny + j)*nz + k][cell] and the compact in-sphere layout the kernels use.
#include "gd_internal.h"

#include <algorithm>


namespace gd {
namespace {

// compact[p][c] = box[node(p)][c]
__global__ void box_to_compact_kernel(const uint32_t *__restrict__ nodes, int ny, int nz, int n_pnt,
                                      const float *__restrict__ box, int ld_box, int ncells,
                                      float *__restrict__ out, int ld)
{
    const int64_t total = (int64_t)n_pnt * ncells;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(t / ncells), c = (int)(t % ncells);
        const uint32_t q = nodes[p];
        const int bi = ((int)(q & 1023) * ny + (int)((q >> 10) & 1023)) * nz + (int)(q >> 20);
        out[(size_t)p * ld + c] = box[(size_t)bi * ld_box + c];
    }
}

// box[b][c] = compact[p(b)][c] inside the sphere, 0 outside
__global__ void compact_to_box_kernel(const int16_t *__restrict__ cmap, int nxyz,
                                      const float *__restrict__ in, int ld, int ncells,
                                      float *__restrict__ box, int ld_box)
{
    const int64_t total = (int64_t)nxyz * ncells;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(t / ncells), c = (int)(t % ncells);
        const int p = cmap[b];
        box[(size_t)b * ld_box + c] = p >= 0 ? in[(size_t)p * ld + c] : 0.f;
    }
}

}  // namespace
}  // namespace gd

extern "C" int gd_box_to_compact(gd_ctx *ctx, const float *box, int ncells, int ld_box, float *compact,
                                 int ld, gd_stream stream)
{
    using namespace gd;
    if (!ctx || !box || !compact) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ncells < 1 || ld_box < ncells || ld < ncells) return set_error(GD_ERR_INVALID_ARG, "bad ncells/ld");
    const Dims &d = ctx->c.d;
    const int64_t total = (int64_t)d.n_pnt * ncells;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 1 << 16);
    box_to_compact_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(ctx->c.d_nodes, d.ny, d.nz, d.n_pnt, box,
                                                                    ld_box, ncells, compact, ld);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

extern "C" int gd_compact_to_box(gd_ctx *ctx, const float *compact, int ncells, int ld, float *box,
                                 int ld_box, gd_stream stream)
{
    using namespace gd;
    if (!ctx || !box || !compact) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ncells < 1 || ld_box < ncells || ld < ncells) return set_error(GD_ERR_INVALID_ARG, "bad ncells/ld");
    const Dims &d = ctx->c.d;
    const int64_t total = (int64_t)d.nxyz * ncells;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 1 << 16);
    compact_to_box_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(ctx->c.d_cmap, d.nxyz, compact, ld, ncells,
                                                                    box, ld_box);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}
