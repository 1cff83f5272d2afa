// gd_gain.cu -- gain term of the hard-sphere collision integral (sm_103a).
//
// The reference sums, for each output node i, over partners i1 and
// post-collision offsets n (collision_integral.cu:75-188, host loop :637-648):
//   I_i = sum_{i1} sum_n w(|i - i1|, n) P(i + i1, n),
//   P(s, n) = f(lx,ly,lz) f(l1x,l1y,l1z) + f(lx,l1y,l1z) f(l1x,ly,lz)
//           + f(lx,ly,l1z) f(l1x,l1y,lz) + f(lx,l1y,lz)  f(l1x,ly,l1z),
//   l = (s + n)/2, l1 = (s - n)/2 per axis, n of the parity of s.
// The pair product P depends only on the pair sum s = i + i1 and on n, so this
// kernel walks s instead of i:
//   1. P_s[n] for every n of the class box B(D(s)), D_a = min(s_a, 2 n_a - 2 - s_a)
//      (exactly the n whose l, l1 stay in the box) -> shared memory,
//   2. C_s[g] = sum_n w(g, n) P_s[n] for every g in B(D(s)) (the |2i - s| of the
//      outputs that have a partner in the box),
//   3. C_s[g] is added to the outputs i = (s +- g)/2 (one per sign pattern).
// Each P is formed once per (s, n) and reused by every output on its collision
// shell instead of being regathered per (i, i1, n).
//
// Rows of the weight table that are bitwise identical (same parity class and
// same |g|) give identical C_s[g], so each such group is contracted once.
//
// Parallel layout: lane = cell (CB cells per row, 32/CB rows per warp), one
// CTA per (cell block, chunk of s).  A chunk owns its own partial output
// buffer; within one s all targets (s +- g)/2 are distinct and successive s
// are separated by barriers, so every partial sum receives its updates in s
// order.  A second kernel adds the chunk partials in chunk order.  Results are
// bitwise reproducible run to run.
#include "gd_internal.h"

#include <algorithm>
#include <cstdio>

namespace gd {
namespace {

constexpr int kThreads = 1024;

struct GainArgs {
    Dims d;
    const float *f;
    int ld, ncells, cells_pad;
    const int16_t *cmap;
    const int *grp_row_off;
    const WEntry *grp_rows;
    const int *D_item_off;
    const int4 *D_items;
    const uint32_t *D_members;
    const int *s_bounds;
    float *part;  // [chunk][n_pnt][cells_pad]
    int cmap_smem;  // 1: box -> compact map copied to shared memory; 0: read through L1 (selects the instance)
};

template <int CB, bool CMAP_SMEM>
__global__ void __launch_bounds__(kThreads, 1) gain_pair_kernel(GainArgs a)
{
    constexpr int G = 32 / CB;  // item rows per warp
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int row_next;
    const Dims &d = a.d;
    // P_s[class index][CB] first, then (when it fits) the box -> compact map;
    // otherwise the map is read from global memory through L1 (its lookups are
    // uniform across the cells of a lane group)
    float *P = reinterpret_cast<float *>(smem);
    int16_t *cmap_s = reinterpret_cast<int16_t *>(smem + (size_t)d.nclass * CB * sizeof(float));
    const int16_t *cmap = CMAP_SMEM ? cmap_s : a.cmap;

    if (CMAP_SMEM)
        for (int t = threadIdx.x; t < d.nxyz; t += blockDim.x) cmap_s[t] = a.cmap[t];
    for (int t = threadIdx.x; t < d.nclass * CB; t += blockDim.x) P[t] = 0.f;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int cl = lane % CB, grp = lane / CB;
    const int cell = blockIdx.x * CB + cl;
    const bool live = cell < a.ncells;
    const float *fcol = a.f + (live ? cell : 0);
    const int chunk = blockIdx.y;
    float *part = a.part + (size_t)chunk * d.n_pnt * a.cells_pad + blockIdx.x * CB + cl;
    const unsigned char *Pc = smem + cl * sizeof(float);
    const uint2 *rows = reinterpret_cast<const uint2 *>(a.grp_rows);
    const int item0 = warp * G + grp, istep = nwarps * G;
    // extents of the previous s's class box: P is zero outside it
    int pex = 0, pey = 0, pez = 0;
    __syncthreads();

    const int s_begin = a.s_bounds[chunk], s_end = a.s_bounds[chunk + 1];
    for (int sl = s_begin; sl < s_end; sl++) {
        const int sz = sl % d.sz, sy = (sl / d.sz) % d.sy, sx = sl / (d.sz * d.sy);
        const int Dx = min(sx, 2 * d.nx - 2 - sx), Dy = min(sy, 2 * d.ny - 2 - sy),
                  Dz = min(sz, 2 * d.nz - 2 - sz);
        const int ex = (Dx >> 1) + 1, ey = (Dy >> 1) + 1, ez = (Dz >> 1) + 1;
        const int px = sx & 1, py = sy & 1, pz = sz & 1;

        // 1. pair products P_s[n] on B(D(s)); zeros where only the previous
        //    s's box had values, so P_s is zero outside B(D(s)) and the rows
        //    can be summed without testing n against the box.  Work is split
        //    into z-runs (fixed n_x, n_y) so each run decodes its indices once.
        const int ux = max(ex, pex), uy = max(ey, pey), uz = max(ez, pez);
        const int nRuns = ux * uy;
        for (int r = item0; r < nRuns; r += istep) {
            const int a2 = r / uy, b2 = r - a2 * uy;
            float *Prun = P + (size_t)((a2 * d.hy + b2) * d.hz) * CB + cl;
            if (a2 >= ex || b2 >= ey) {
                for (int c2 = 0; c2 < uz; c2++) Prun[c2 * CB] = 0.f;
                continue;
            }
            const int nxv = 2 * a2 + px, nyv = 2 * b2 + py;
            const int X0 = ((sx + nxv) >> 1) * d.nyz, X1 = ((sx - nxv) >> 1) * d.nyz;
            const int Y0 = ((sy + nyv) >> 1) * d.nz, Y1 = ((sy - nyv) >> 1) * d.nz;
            const int A = X0 + Y0, B = X1 + Y1, Cc = X0 + Y1, Dd = X1 + Y0;
            const int ld = a.ld;
            for (int c2 = ez; c2 < uz; c2++) Prun[c2 * CB] = 0.f;
            // two pair products per iteration: 16 independent loads in flight
            for (int c2 = 0; c2 < ez; c2 += 2) {
                const bool two = c2 + 1 < ez;
                const int nz0 = 2 * c2 + pz;
                const int lz0 = (sz + nz0) >> 1, l1z0 = (sz - nz0) >> 1;
                const int lz1 = two ? lz0 + 1 : lz0, l1z1 = two ? l1z0 - 1 : l1z0;
                const int k0 = cmap[A + lz0], k1 = cmap[B + l1z0], k2 = cmap[Cc + l1z0], k3 = cmap[Dd + lz0];
                const int k4 = cmap[A + l1z0], k5 = cmap[B + lz0], k6 = cmap[Cc + lz0], k7 = cmap[Dd + l1z0];
                const int j0 = cmap[A + lz1], j1 = cmap[B + l1z1], j2 = cmap[Cc + l1z1], j3 = cmap[Dd + lz1];
                const int j4 = cmap[A + l1z1], j5 = cmap[B + lz1], j6 = cmap[Cc + lz1], j7 = cmap[Dd + l1z1];
#define GD_F(k) (((k) >= 0 && live) ? __ldg(fcol + (k) * ld) : 0.f)  // 32-bit offsets: n_pnt ld < 2^31
                const float f0 = GD_F(k0), f1 = GD_F(k1), f2 = GD_F(k2), f3 = GD_F(k3);
                const float f4 = GD_F(k4), f5 = GD_F(k5), f6 = GD_F(k6), f7 = GD_F(k7);
                const float h0 = GD_F(j0), h1 = GD_F(j1), h2 = GD_F(j2), h3 = GD_F(j3);
                const float h4 = GD_F(j4), h5 = GD_F(j5), h6 = GD_F(j6), h7 = GD_F(j7);
#undef GD_F
                Prun[c2 * CB] = __fmaf_rn(f0, f1, f2 * f3) + __fmaf_rn(f4, f5, f6 * f7);
                if (two) Prun[(c2 + 1) * CB] = __fmaf_rn(h0, h1, h2 * h3) + __fmaf_rn(h4, h5, h6 * h7);
            }
        }
        pex = ex;
        pey = ey;
        pez = ez;
        if (threadIdx.x == 0) row_next = 0;
        __syncthreads();

        // 2./3. contraction and scatter --------------------------------------
        // The work items of D(s) are the row groups with a member in B(D(s))
        // (rows of g's with equal |g| and parity are bitwise identical), each
        // with its members in B(D(s)).  A group's row is contracted with P_s
        // once; the sum goes to the targets (s +- g)/2 of every member g.
        // Items are handed out through a shared counter (a warp takes G at a
        // time, one per lane group).  Each sum is formed by one lane group in
        // entry order; within one s every target receives exactly one update
        // and successive s are separated by a barrier, so every partial sum is
        // updated in s order whichever warp does the work.
        const int Did = (Dx * d.ny + Dy) * d.nz + Dz;
        const int it0 = __ldg(a.D_item_off + Did), nIt = __ldg(a.D_item_off + Did + 1) - it0;
        for (;;) {
            int t0 = 0;
            if (lane == 0) t0 = atomicAdd(&row_next, G);
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            if (t0 >= nIt) break;
            const int t = t0 + grp;
            if (t >= nIt) continue;
            const int4 item = __ldg(a.D_items + it0 + t);
            const int e0 = __ldg(a.grp_row_off + item.x), e1 = __ldg(a.grp_row_off + item.x + 1);
            // rows are 8-entry padded and 16-byte aligned: two entries per
            // load, 16 entries per batch
            float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, acc3 = 0.f;
            const uint4 *rp = reinterpret_cast<const uint4 *>(rows + e0);
            const uint4 *rend = reinterpret_cast<const uint4 *>(rows + e1);
#define GD_MAC(acc, wv, ov) acc = __fmaf_rn(__uint_as_float(wv), *reinterpret_cast<const float *>(Pc + (ov)), acc)
            for (; rp + 8 <= rend; rp += 8) {
                uint4 r[8];
#pragma unroll
                for (int q = 0; q < 8; q++) r[q] = __ldg(rp + q);
#pragma unroll
                for (int q = 0; q < 8; q += 2) {
                    GD_MAC(acc0, r[q].y, r[q].x);
                    GD_MAC(acc1, r[q].w, r[q].z);
                    GD_MAC(acc2, r[q + 1].y, r[q + 1].x);
                    GD_MAC(acc3, r[q + 1].w, r[q + 1].z);
                }
            }
            if (rp < rend) {
                const uint4 r01 = __ldg(rp), r23 = __ldg(rp + 1), r45 = __ldg(rp + 2), r67 = __ldg(rp + 3);
                GD_MAC(acc0, r01.y, r01.x);
                GD_MAC(acc1, r01.w, r01.z);
                GD_MAC(acc2, r23.y, r23.x);
                GD_MAC(acc3, r23.w, r23.z);
                GD_MAC(acc0, r45.y, r45.x);
                GD_MAC(acc1, r45.w, r45.z);
                GD_MAC(acc2, r67.y, r67.x);
                GD_MAC(acc3, r67.w, r67.z);
            }
#undef GD_MAC
            const float acc = (acc0 + acc1) + (acc2 + acc3);
            if (!live) continue;
            // explicit load/add/store: global float reductions flush subnormal
            // values to zero, and corner-node contributions are subnormal
            for (int m = item.y; m < item.z; m++) {
                const uint32_t mm = __ldg(a.D_members + m);
                const int gx = 2 * (int)(mm & 31) + px, gy = 2 * (int)((mm >> 6) & 31) + py,
                          gz = 2 * (int)((mm >> 12) & 31) + pz;
                // per axis the two target coordinates (s - g)/2 and (s + g)/2
                const int X0 = ((sx - gx) >> 1) * d.nyz, X1 = X0 + gx * d.nyz;
                const int Y0 = ((sy - gy) >> 1) * d.nz, Y1 = Y0 + gy * d.nz;
                const int Z0 = (sz - gz) >> 1, Z1 = Z0 + gz;
                int tgt[8];
                float old[8];
#pragma unroll
                for (int sg = 0; sg < 8; sg++) {
                    const bool hx = sg & 1, hy = (sg >> 1) & 1, hz = (sg >> 2) & 1;
                    const bool dup = (hx && gx == 0) || (hy && gy == 0) || (hz && gz == 0);
                    tgt[sg] = dup ? -1 : cmap[(hx ? X1 : X0) + (hy ? Y1 : Y0) + (hz ? Z1 : Z0)];
                    old[sg] = tgt[sg] >= 0 ? part[tgt[sg] * a.cells_pad] : 0.f;
                }
#pragma unroll
                for (int sg = 0; sg < 8; sg++)
                    if (tgt[sg] >= 0) part[tgt[sg] * a.cells_pad] = old[sg] + acc;
            }
        }
        __syncthreads();
    }
}

// gain[node][c] = sum over chunks of the partials, in chunk order.
__global__ void gain_reduce_kernel(const float *__restrict__ part, int nchunks, int n_pnt,
                                   int cells_pad, int ncells, int ld, float *__restrict__ gain)
{
    const int64_t total = (int64_t)n_pnt * ncells;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int node = (int)(t / ncells), c = (int)(t % ncells);
        const float *p = part + (size_t)node * cells_pad + c;
        float s = 0.f;
        for (int k = 0; k < nchunks; k++) s += p[(size_t)k * n_pnt * cells_pad];
        gain[(size_t)node * ld + c] = s;
    }
}

size_t gain_smem_bytes(const Dims &d, int cb, bool cmap_smem)
{
    return (size_t)d.nclass * cb * sizeof(float) + (cmap_smem ? (size_t)((d.nxyz * 2 + 15) & ~15) : 0);
}

// Number of s-chunks for nblk cell blocks: at least gain_waves CTAs per SM
// (2 unless the autotuner chose otherwise), then the
// count (up to 64 chunks, or 512 when a few blocks must fill the GPU) whose
// CTA total fills the last wave best; ties go to fewer chunks.
int gain_chunk_count(const Context &c, int nblk)
{
    const int sms = std::max(1, c.sm_count);
    const int lo = std::max(1, (std::max(1, c.gain_waves) * sms + nblk - 1) / nblk);
    const int hi = std::max(lo, std::min(lo + 64, 512));
    int best = lo;
    double best_fill = -1.0;
    for (int k = lo; k <= hi; k++) {
        const int64_t ctas = (int64_t)nblk * k;
        const double fill = (double)ctas / (double)(((ctas + sms - 1) / sms) * sms);
        if (fill > best_fill + 1e-9) {
            best_fill = fill;
            best = k;
        }
        if (fill > 0.999) break;
    }
    return (int)std::min<int64_t>(best, c.d.ns);
}

}  // namespace

int gain_plan_cells(Context &c)
{
    int max_smem = 0;
    GD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    // widest cell block that fits: with the box -> compact map in shared memory
    // first, then with the map read through L1
    int cb = 32;
    bool cmap_smem = true;
    for (;;) {
        if (gain_smem_bytes(c.d, cb, true) <= (size_t)max_smem) break;
        if (gain_smem_bytes(c.d, cb, false) <= (size_t)max_smem) {
            cmap_smem = false;
            break;
        }
        if (cb == 4) return set_error(GD_ERR_UNSUPPORTED, "velocity grid too large for the gain kernel's shared memory");
        cb >>= 1;
    }
    if ((int64_t)c.d.nclass * cb * 4 >= ((int64_t)1 << 32))
        return set_error(GD_ERR_UNSUPPORTED, "pair-product array too large");
    c.gain_cb = cb;
    c.gain_cmap_smem = cmap_smem;
    c.gain_smem = gain_smem_bytes(c.d, cb, cmap_smem);
    return GD_OK;
}

// Device copy of the chunk boundaries for nchunks chunks, built and uploaded
// on first use (a synchronous copy: the first call of a new launch shape must
// not be inside a stream capture).
int gain_bounds_device(Context &c, int nchunks, const int **out)
{
    auto it = c.s_bounds_dev.find(nchunks);
    if (it == c.s_bounds_dev.end()) {
        std::vector<int> bounds(nchunks + 1);
        gain_chunk_bounds(c, nchunks, bounds.data());
        int *d = nullptr;
        GD_CUDA(cudaMalloc(&d, sizeof(int) * (nchunks + 1)));
        cudaError_t e = cudaMemcpy(d, bounds.data(), sizeof(int) * (nchunks + 1), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d);
            return cuda_error(e, "gain chunk bounds");
        }
        it = c.s_bounds_dev.emplace(nchunks, d).first;
    }
    *out = it->second;
    return GD_OK;
}

int run_gain(Context &c, const float *f, int ncells, int ld, float *gain, cudaStream_t st)
{
    const Dims &d = c.d;
    int cb = 0, nblk = 0, nchunks = 0;
    size_t smem = 0;
    int rc = gain_launch_shape(c, ncells, &cb, &smem, &nblk, &nchunks);
    if (rc) return rc;
    const int cells_pad = nblk * cb;
    // the partial buffer [chunk][node][cells] is bounded at 16 GiB
    while (nchunks > 1 && (size_t)nchunks * d.n_pnt * cells_pad * sizeof(float) > ((size_t)16 << 30)) nchunks--;
    // work-balanced chunk boundaries over the linear s order, cached per count
    const int *d_bounds = nullptr;
    if ((rc = gain_bounds_device(c, nchunks, &d_bounds))) return rc;
    if ((rc = ensure_scratch(c, (size_t)nchunks * d.n_pnt * cells_pad * sizeof(float)))) return rc;
    return launch_gain_pair(c, f, ncells, ld, gain, static_cast<float *>(c.scratch.ptr), nchunks, d_bounds, cb,
                            smem, st);
}

int reduce_gain_partials(Context &c, const float *part, int nchunks, int cells_pad, int ncells, int ld,
                         float *gain, cudaStream_t st)
{
    const int64_t outs = (int64_t)c.d.n_pnt * ncells;
    const int rblocks = (int)std::min<int64_t>((outs + 255) / 256, (int64_t)c.sm_count * 16);
    gain_reduce_kernel<<<std::max(rblocks, 1), 256, 0, st>>>(part, nchunks, c.d.n_pnt, cells_pad, ncells, ld,
                                                              gain);
    GD_CUDA(cudaGetLastError());
    return GD_OK;
}

// ---------------------------------------------------------------------------
// Launch pieces shared by run_gain above (partials in the context's scratch)
// and the allocation-free entry point in gd_noalloc.cu (partials in its
// fixed array): the launch shape, the chunk boundaries, and the one launch
// routine (clear the partials, gain kernel, chunk reduction).

// cells per lane row, shared memory, cell blocks and the s-chunk count
// (at least two CTAs per SM, whole waves preferred), before any bound on the
// partial buffer
int gain_launch_shape(Context &c, int ncells, int *cb_out, size_t *smem_out, int *nblk_out,
                      int *chunks_out)
{
    const int cb = c.gain_cb;
    const int nblk = (ncells + cb - 1) / cb;
    const int nchunks = gain_chunk_count(c, nblk);
    *cb_out = cb;
    *smem_out = c.gain_smem;
    *nblk_out = nblk;
    *chunks_out = nchunks;
    return GD_OK;
}

void gain_chunk_bounds(const Context &c, int nchunks, int *bounds)
{
    const int64_t total = c.s_work_prefix[c.d.ns];
    bounds[0] = 0;
    for (int k = 1; k < nchunks; k++) {
        const int64_t target = total * k / nchunks;
        bounds[k] = (int)(std::lower_bound(c.s_work_prefix.begin(), c.s_work_prefix.end(), target) -
                          c.s_work_prefix.begin());
        bounds[k] = std::max(bounds[k], bounds[k - 1]);
    }
    bounds[nchunks] = (int)c.d.ns;
}

int launch_gain_pair(Context &c, const float *f, int ncells, int ld, float *gain, float *part,
                     int nchunks, const int *d_bounds, int cb, size_t smem, cudaStream_t st)
{
    const Dims &d = c.d;
    const int nblk = (ncells + cb - 1) / cb;
    const int cells_pad = nblk * cb;
    // the kernel forms node x stride offsets in 32 bits
    if ((int64_t)d.n_pnt * std::max(ld, cells_pad) >= ((int64_t)1 << 31))
        return set_error(GD_ERR_UNSUPPORTED, "pair gain: n_pnt * ld must stay below 2^31");
    GD_CUDA(cudaMemsetAsync(part, 0, (size_t)nchunks * d.n_pnt * cells_pad * sizeof(float), st));
    GainArgs a{d, f, ld, ncells, cells_pad, c.d_cmap, c.d_grp_row_off, c.d_grp_rows, c.d_D_item_off,
               c.d_D_items, c.d_D_members, d_bounds, part, c.gain_cmap_smem ? 1 : 0};
    dim3 grid(nblk, nchunks);
    switch (cb) {
#define GD_GAIN_CASE(CBV)                                                                       \
    case CBV:                                                                                   \
        if (a.cmap_smem) {                                                                      \
            GD_CUDA(cudaFuncSetAttribute(gain_pair_kernel<CBV, true>,                           \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
            gain_pair_kernel<CBV, true><<<grid, kThreads, smem, st>>>(a);                       \
        } else {                                                                                \
            GD_CUDA(cudaFuncSetAttribute(gain_pair_kernel<CBV, false>,                          \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
            gain_pair_kernel<CBV, false><<<grid, kThreads, smem, st>>>(a);                      \
        }                                                                                       \
        break;
        GD_GAIN_CASE(32)
        GD_GAIN_CASE(16)
        GD_GAIN_CASE(8)
        GD_GAIN_CASE(4)
#undef GD_GAIN_CASE
    default:
        return set_error(GD_ERR_UNSUPPORTED, "gain kernel cell block");
    }
    GD_CUDA(cudaGetLastError());
    return reduce_gain_partials(c, part, nchunks, cells_pad, ncells, ld, gain, st);
}

}  // namespace gd
