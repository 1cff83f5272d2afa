// gd_pair_tc.cu -- gain in the pair-product formulation with its contraction
// on the tensor cores (sm_103a).
//
// The FP32 gain kernel (gd_gain.cu) walks the pair sums s = i + i1: for every
// s it forms the pair products P_s[n] on the class box B(D(s)), contracts them
// with the weight row of every row group present in B(D(s)),
//     C_s[m] = sum_{n in B(D)} W_D[m][n] P_s[n],
// and adds C_s[m] to the outputs (s +- g)/2 of each member g of group m
// (collision_integral.cu:75-188 summed in pair-product form).  Here the
// contraction is one GEMM per (s, 128 cells) on the tensor cores:
//     C^T [128 cells x M_D] = P_s^T [128 cells x K_D] . W_D^T [K_D x M_D],
// W_D holding D's group rows restricted to B(D) (K_D = |B(D)| class offsets in
// the order (x2 * ey + y2) * ez + z2, M_D groups in the order of D's work
// items), stored once per D in chunks of 64 offsets.  P and W are split into
// BF16 hi + lo and P_hi W_hi + P_hi W_lo + P_lo W_hi accumulates in FP32
// (relative error ~1e-6 against the FP32 kernel).  Boxes with more than 256
// groups run as several passes of at most 256 groups, each forming P again.
//
// One persistent CTA per SM takes (grid, 128-cell tile, chunk of the walk over
// s) units from a device list, warp-specialized:
//   warps 14..21 pair products of one 64-offset chunk for the 128 cells (thread
//                = cell, eight gathers of f per product, the FP32 products of
//                the FP32 kernel), split into BF16 hi/lo and written to shared
//                memory in the MMA's 128-byte-swizzled K-major layout; two
//                groups of four warps fill the two stages alternately;
//   warp 0       TMA loads of the chunk's weight rows (hi, lo), 16 rows a box;
//   warp 1       tcgen05.mma (M = 128 cells, N = groups padded to 16, K = 16)
//                into one of two TMEM accumulators per (s, pass);
//   warps 2..13  read C^T from TMEM (thread = cell; three warps per lane
//                quadrant taking every third block of 16 groups) and add each
//                group's sum, by fire-and-forget reductions, to the outputs
//                at its members' targets (s +- g)/2.
// The outputs accumulate in 64-bit fixed point: each cell has a power-of-two
// scale 2^k, set before the launch from a bound on its gain (max|f|^2 times
// the largest gain of f = 1), and a group's sum enters as round(C * 2^k).
// Integer addition is associative, so every unit of every s-chunk adds into
// one accumulator per grid, in whatever order the hardware runs them, and the
// result is still bitwise reproducible; no per-chunk partial buffers cross
// DRAM and no reduction pass is needed, only a conversion back to FP32.
// Every mbarrier wait is bounded (a time-out sets the error flag).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "gd_internal.h"
#include "gd_tc.cuh"

namespace gd {
namespace {

using namespace tc;

constexpr int PT_BM = 128;               // cells per CTA (MMA M, TMEM lanes)
constexpr int PT_KC = 64;                // class offsets per chunk (one 128-byte swizzle row of BF16)
constexpr int PT_NMAX = 256;             // groups per pass (MMA N, TMEM columns per accumulator)
constexpr uint32_t kPTile = PT_BM * PT_KC * 2;     // 16 KB: P part of one chunk
constexpr uint32_t kWTile = PT_NMAX * PT_KC * 2;   // 32 KB: W part of one chunk (up to 256 rows)
constexpr uint32_t kPtStage = 2 * kPTile + 2 * kWTile;  // P hi, P lo, W hi, W lo
constexpr int kPtStages = 2;
constexpr int kEpiWarps = 12;            // three per TMEM lane quadrant
constexpr int kProdWarps = 8;            // two groups of four
constexpr int kPtThreads = 32 * (2 + kEpiWarps + kProdWarps);

constexpr int kPtMaxGrids = 4;          // velocity grids one launch can serve
constexpr int kBadScale = -0x7fffffff;  // scale exponent of a cell with a non-finite f
constexpr int kAccBits = 60;            // |sum of contributions| * 2^k < 2^60

// One velocity grid's tables and arrays as the kernel reads them.
struct PtGrid {
    Dims d;
    const float *f;
    int ld, ncells, cells_pad;
    const int16_t *cmap;
    const int *D_item_off;
    const int4 *D_items;
    const uint32_t *D_members;
    const int *wrow;        // [nxyz] first weight row of each D
    const int *s_bounds;    // [chunks + 1] bounds of the walk's chunks
    unsigned long long *acc;  // [n_pnt][cells_pad] fixed-point gain (two's complement)
    const int *kcell;       // [cells_pad] scale exponent k of each cell
};

// A launch: up to kPtMaxGrids grids and the device list of work units
// {grid, 128-cell tile, chunk of the walk, 0} that the persistent CTAs pull, one at a
// time, from a device counter.
struct PtLaunch {
    PtGrid g[kPtMaxGrids];
    const int4 *units;
    int nunits;
    int *next;  // the next unit to hand out (zeroed before the launch)
    int *err;
};

// The weight tables' tensor maps per grid (hi and lo parts).
struct PtMaps {
    CUtensorMap wh[kPtMaxGrids], wl[kPtMaxGrids];
};

// One (s, pass) of the walk: its class box, groups and weight rows.
struct Unit {
    int sx, sy, sz, px, py, pz;
    int ex, ey, ez, K, nch;    // class box extents, offsets, 64-offset chunks
    int it0, mcnt, npad;       // first work item of this pass, groups, groups padded to 16
    int mpad;                  // all of D's groups padded to 16 (rows per chunk in the table)
    int wrow;                  // first table row of D
    int npass;
};

// The walk visits the pair sums class box by class box: position
// p = 8 D + r, D = (Dx ny + Dy) nz + Dz, holds the pair sum whose axis a is
// D_a (bit a of r clear) or its reflection 2 n_a - 2 - D_a (bit a set).  A
// reflection of D_a = n_a - 1 is that value itself, so such positions repeat
// an earlier one and are empty.  The (up to) eight pair sums of one D read the
// same weight rows one after another, so the rows come from DRAM about once
// per launch instead of once per pair sum.
__device__ __forceinline__ int walk_D(const Dims &d, int p, int &sx, int &sy, int &sz)
{
    const int Did = p >> 3, r = p & 7;
    const int Dz = Did % d.nz, Dy = (Did / d.nz) % d.ny, Dx = Did / d.nyz;
    if (((r & 1) && Dx == d.nx - 1) || ((r & 2) && Dy == d.ny - 1) || ((r & 4) && Dz == d.nz - 1)) return -1;
    sx = (r & 1) ? 2 * d.nx - 2 - Dx : Dx;
    sy = (r & 2) ? 2 * d.ny - 2 - Dy : Dy;
    sz = (r & 4) ? 2 * d.nz - 2 - Dz : Dz;
    return Did;
}

__device__ __forceinline__ void unit_of(const PtGrid &a, int sl, int q, Unit &u)
{
    const Dims &d = a.d;
    const int Did = walk_D(d, sl, u.sx, u.sy, u.sz);  // the caller skips empty positions
    const int Dz = Did % d.nz, Dy = (Did / d.nz) % d.ny, Dx = Did / d.nyz;
    u.ex = (Dx >> 1) + 1;
    u.ey = (Dy >> 1) + 1;
    u.ez = (Dz >> 1) + 1;
    u.px = u.sx & 1;
    u.py = u.sy & 1;
    u.pz = u.sz & 1;
    u.K = u.ex * u.ey * u.ez;
    u.nch = (u.K + PT_KC - 1) / PT_KC;
    const int i0 = __ldg(a.D_item_off + Did), m = __ldg(a.D_item_off + Did + 1) - i0;
    u.npass = (m + PT_NMAX - 1) / PT_NMAX;
    u.it0 = i0 + q * PT_NMAX;
    u.mcnt = min(PT_NMAX, m - q * PT_NMAX);
    u.npad = (u.mcnt + 15) & ~15;
    u.mpad = (m + 15) & ~15;
    u.wrow = __ldg(a.wrow + Did);
}

__device__ __forceinline__ int npass_of(const PtGrid &a, int sl)
{
    const Dims &d = a.d;
    int sx, sy, sz;
    const int Did = walk_D(d, sl, sx, sy, sz);
    if (Did < 0) return 0;
    const int m = __ldg(a.D_item_off + Did + 1) - __ldg(a.D_item_off + Did);
    return (m + PT_NMAX - 1) / PT_NMAX;
}

template <bool CMAP_SMEM>
__global__ void __launch_bounds__(kPtThreads, 1)
    pair_tc_kernel(const __grid_constant__ PtMaps maps, const __grid_constant__ PtLaunch L)
{
    extern __shared__ __align__(1024) unsigned char dsmem[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~static_cast<uintptr_t>(1023));
    int16_t *cmap_s = reinterpret_cast<int16_t *>(base + kPtStages * kPtStage);
    __shared__ __align__(8) uint64_t full_bar[kPtStages], empty_bar[kPtStages], accf_bar[2], acce_bar[2];
    __shared__ uint32_t tmem_base_holder;
    __shared__ int epi_fail;
    __shared__ int unit_slot, stop_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        epi_fail = 0;
        stop_flag = 0;
        for (int s = 0; s < kPtStages; s++) {
            mbar_init(smem_u32(&full_bar[s]), 4 + 1);  // four producer warps + the TMA arrival
            mbar_init(smem_u32(&empty_bar[s]), 1);      // the MMA commit
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&accf_bar[b]), 1);
            mbar_init(smem_u32(&acce_bar[b]), kEpiWarps);  // the epilogue warps
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (CMAP_SMEM)  // single-grid launches only: the box -> compact map of grid 0
        for (int t = threadIdx.x; t < L.g[0].d.nxyz; t += blockDim.x) cmap_s[t] = L.g[0].cmap[t];
    if (warp == 1) {
        tmem_alloc<1>(smem_u32(&tmem_base_holder), 2 * PT_NMAX);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_holder;

    // per-role state that runs on across units: pipeline counters (stage,
    // accumulator) and whether this thread's role is still healthy
    int ck = 0, uc = 0;
    bool ok = true;

    // Units are pulled one at a time from the device counter by thread 0 and
    // shared through unit_slot; every thread of the CTA meets the two barriers
    // of each round, so all roles work on the same unit and the pipeline
    // drains between units (units are long: a chunk of s for 128 cells).  A
    // role that gave up after a timed-out wait raises stop_flag, and the CTA
    // takes no further unit.
    for (;;) {
        if (threadIdx.x == 0) unit_slot = stop_flag ? L.nunits : atomicAdd(L.next, 1);
        __syncthreads();
        const int ui_ = unit_slot;
        if (ui_ >= L.nunits) break;
        const int4 un_ = L.units[ui_];
        const PtGrid &a = L.g[un_.x];
        const Dims &d = a.d;
        const int m_tile = un_.y, chunk = un_.z;
        const int s_begin = __ldg(a.s_bounds + chunk), s_end = __ldg(a.s_bounds + chunk + 1);

    if (warp == 0) {
        // ---- TMA: weight rows of every chunk --------------------------------------
        if (lane == 0 && ok) {
            {
            const CUtensorMap *tmWh = &maps.wh[un_.x], *tmWl = &maps.wl[un_.x];
            for (int sl = s_begin; ok && sl < s_end; sl++) {
                const int np = npass_of(a, sl);
                for (int q = 0; ok && q < np; q++) {
                    Unit u;
                    unit_of(a, sl, q, u);
                    for (int ch = 0; ch < u.nch; ch++, ck++) {
                        const int st = ck & 1;
                        if (!mbar_wait(smem_u32(&empty_bar[st]), ((uint32_t)(ck >> 1) & 1u) ^ 1u, L.err)) {
                            ok = false;
                            break;
                        }
                        unsigned char *sb = base + (size_t)st * kPtStage;
                        const uint32_t fb = smem_u32(&full_bar[st]);
                        mbar_expect_tx(fb, 2u * (uint32_t)u.npad * (PT_KC * 2));
                        const int row0 = u.wrow + ch * u.mpad + q * PT_NMAX;
                        for (int r = 0; r < u.npad; r += 16) {
                            tma_load_2d(smem_u32(sb + 2 * kPTile + r * (PT_KC * 2)), tmWh, 0, row0 + r, fb);
                            tma_load_2d(smem_u32(sb + 2 * kPTile + kWTile + r * (PT_KC * 2)), tmWl, 0, row0 + r,
                                        fb);
                        }
                    }
                }
            }
            }
        }
    } else if (warp == 1) {
        // ---- MMA ---------------------------------------------------------------------
        if (lane == 0 && ok) {
            {
            for (int sl = s_begin; ok && sl < s_end; sl++) {
                const int np = npass_of(a, sl);
                for (int q = 0; ok && q < np; q++, uc++) {
                    Unit u;
                    unit_of(a, sl, q, u);
                    const int buf = uc & 1;
                    if (!mbar_wait(smem_u32(&acce_bar[buf]), ((uint32_t)(uc >> 1) & 1u) ^ 1u, L.err)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t d_tmem = tmem + (uint32_t)(buf * PT_NMAX);
                    const uint32_t idesc = umma_idesc_bf16(PT_BM, u.npad);
                    for (int ch = 0; ch < u.nch; ch++, ck++) {
                        const int st = ck & 1;
                        if (!mbar_wait(smem_u32(&full_bar[st]), (uint32_t)(ck >> 1) & 1u, L.err)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t sb = smem_u32(base + (size_t)st * kPtStage);
                        const uint32_t pH = sb, pL = sb + kPTile, wH = sb + 2 * kPTile, wL = sb + 2 * kPTile + kWTile;
#pragma unroll
                        for (int kk = 0; kk < PT_KC / 16; kk++) {
                            const uint32_t off = (uint32_t)kk * 32u;
                            const uint32_t acc = (ch > 0 || kk > 0) ? 1u : 0u;
                            umma_bf16(d_tmem, umma_desc(pH + off), umma_desc(wH + off), idesc, acc);
                            umma_bf16(d_tmem, umma_desc(pH + off), umma_desc(wL + off), idesc, 1u);
                            umma_bf16(d_tmem, umma_desc(pL + off), umma_desc(wH + off), idesc, 1u);
                        }
                        umma_commit(smem_u32(&empty_bar[st]));
                    }
                    if (!ok) break;
                    umma_commit(smem_u32(&accf_bar[buf]));
                }
            }
            }
        }
    } else if (warp < 2 + kEpiWarps) {
        // ---- epilogue: thread = cell = TMEM lane (warp % 4 is the lane quadrant it
        // may read); the quadrant's warps take every third 16-group block -------
        const int quad = warp & 3;
        const int third = (warp - 2) >> 2;  // which of the quadrant's warps
        const int row = quad * 32 + lane;
        if (ok) {
        const int16_t *cmap = CMAP_SMEM ? cmap_s : a.cmap;
        const int cell = m_tile * PT_BM + row;
        const bool live = cell < a.ncells;
        // the unit's fields used in the scatter loop, held in registers (the
        // reductions' memory clobber would otherwise reload them each time)
        const int cells_pad = a.cells_pad, nyz = d.nyz, nz = d.nz;
        const int4 *D_items = a.D_items;
        const uint32_t *D_members = a.D_members;
        unsigned long long *acc = a.acc + cell;
        // the cell's fixed-point scale 2^k as two exact power-of-two factors
        const int kc = live ? __ldg(a.kcell + cell) : 0;
        const int k1 = kc == kBadScale ? 0 : kc / 2, k2 = kc == kBadScale ? 0 : kc - kc / 2;
        const float s1 = __int_as_float((127 + k1) << 23), s2 = __int_as_float((127 + k2) << 23);
        for (int sl = s_begin; ok && sl < s_end; sl++) {
            const int np = npass_of(a, sl);
            for (int q = 0; ok && q < np; q++, uc++) {
                Unit u;
                unit_of(a, sl, q, u);
                const int buf = uc & 1;
                if (lane == 0 && !mbar_wait(smem_u32(&accf_bar[buf]), (uint32_t)(uc >> 1) & 1u, L.err)) epi_fail = 1;
                // the epilogue warps take each unit together, so that the
                // decision to stop is taken after the barrier, by all of them
                // alike
                asm volatile("bar.sync 1, %0;" ::"n"(32 * kEpiWarps) : "memory");
                if (*(volatile int *)&epi_fail) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t taddr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * PT_NMAX);
                for (int m0 = third * 16; m0 < u.mcnt; m0 += 16 * (kEpiWarps / 4)) {
                    float v[16];
                    tmem_ld16(taddr + (uint32_t)m0, v);
                    if (!live) continue;
                    const int mend = min(16, u.mcnt - m0);
                    for (int t = 0; t < mend; t++) {
                        // the group's sum in the cell's fixed point; integer
                        // fire-and-forget reductions, whose order does not
                        // matter (contributions below 2^-k round away)
                        const long long qv = __float2ll_rn(__fmul_rn(__fmul_rn(v[t], s1), s2));
                        if (qv == 0) continue;
                        const int4 item = __ldg(D_items + u.it0 + m0 + t);
                        for (int mm = item.y; mm < item.z; mm++) {
                            const uint32_t pk = __ldg(D_members + mm);
                            const int gx = 2 * (int)(pk & 31) + u.px, gy = 2 * (int)((pk >> 6) & 31) + u.py,
                                      gz = 2 * (int)((pk >> 12) & 31) + u.pz;
                            const int X0 = ((u.sx - gx) >> 1) * nyz, X1 = X0 + gx * nyz;
                            const int Y0 = ((u.sy - gy) >> 1) * nz, Y1 = Y0 + gy * nz;
                            const int Z0 = (u.sz - gz) >> 1, Z1 = Z0 + gz;
#pragma unroll
                            for (int sg = 0; sg < 8; sg++) {
                                const bool hx = sg & 1, hy = (sg >> 1) & 1, hz = (sg >> 2) & 1;
                                const bool dup = (hx && gx == 0) || (hy && gy == 0) || (hz && gz == 0);
                                const int tg = dup ? -1 : cmap[(hx ? X1 : X0) + (hy ? Y1 : Y0) + (hz ? Z1 : Z0)];
                                if (tg >= 0)
                                    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(acc + tg * cells_pad),
                                                 "l"((unsigned long long)qv)
                                                 : "memory");
                            }
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&acce_bar[buf]));
            }
        }
        }
    } else {
        // ---- pair products ------------------------------------------------------------
        const int pw = warp - 2 - kEpiWarps;
        const int grp = pw >> 2;             // fills the stages of chunks ck with ck % 2 == grp
        const int row = (pw & 3) * 32 + lane;  // cell row of the P tile
        const uint32_t swz = (uint32_t)(row & 7);
        const uint32_t rowoff = (uint32_t)(row >> 3) * 1024u + (uint32_t)(row & 7) * 128u;
        if (ok) {
        const int16_t *cmap = CMAP_SMEM ? cmap_s : a.cmap;
        const int cell = m_tile * PT_BM + row;
        const bool live = cell < a.ncells;
        const float *fcol = a.f + (live ? cell : 0);
        const int ldf = a.ld, nyz = d.nyz, nz = d.nz;  // in registers for the gather loop
        for (int sl = s_begin; ok && sl < s_end; sl++) {
            const int np = npass_of(a, sl);
            for (int q = 0; ok && q < np; q++) {
                Unit u;
                unit_of(a, sl, q, u);
                for (int ch = 0; ch < u.nch; ch++, ck++) {
                    const int st = ck & 1;
                    if (st != grp) continue;
                    bool w = true;
                    if (lane == 0) w = mbar_wait(smem_u32(&empty_bar[st]), ((uint32_t)(ck >> 1) & 1u) ^ 1u, L.err);
                    if (__shfl_sync(0xffffffffu, w ? 1 : 0, 0) == 0) {
                        ok = false;
                        break;
                    }
                    unsigned char *pH = base + (size_t)st * kPtStage + rowoff;
                    unsigned char *pL = pH + kPTile;
                    // class offset k = ch * 64 + t decoded as (x2, y2, z2) with z2
                    // fastest; along a z-run only lz and l1z move, by +-1
                    int k = ch * PT_KC;
                    int z2 = k % u.ez, y2 = (k / u.ez) % u.ey, x2 = k / (u.ez * u.ey);
                    int A = 0, B = 0, Cc = 0, Dd = 0;
                    auto set_run = [&]() {
                        const int nxv = 2 * x2 + u.px, nyv = 2 * y2 + u.py;
                        const int X0 = ((u.sx + nxv) >> 1) * nyz, X1 = ((u.sx - nxv) >> 1) * nyz;
                        const int Y0 = ((u.sy + nyv) >> 1) * nz, Y1 = ((u.sy - nyv) >> 1) * nz;
                        A = X0 + Y0;
                        B = X1 + Y1;
                        Cc = X0 + Y1;
                        Dd = X1 + Y0;
                    };
                    if (k < u.K) set_run();
                    const int zc0 = (u.sz + u.pz) >> 1, zc1 = (u.sz - u.pz) >> 1;
#pragma unroll 1
                    for (int j = 0; j < PT_KC / 8; j++) {
                        float pv[8];
#pragma unroll
                        for (int t = 0; t < 8; t++) {
                            float p = 0.f;
                            if (k < u.K) {
                                const int lz = zc0 + z2, l1z = zc1 - z2;
                                const int k0 = cmap[A + lz], k1 = cmap[B + l1z], k2 = cmap[Cc + l1z], k3 = cmap[Dd + lz];
                                const int k4 = cmap[A + l1z], k5 = cmap[B + lz], k6 = cmap[Cc + lz], k7 = cmap[Dd + l1z];
#define GD_F(kk) (((kk) >= 0 && live) ? __ldg(fcol + (kk) * ldf) : 0.f)  // 32-bit offsets: n_pnt ld < 2^31
                                const float f0 = GD_F(k0), f1 = GD_F(k1), f2 = GD_F(k2), f3 = GD_F(k3);
                                const float f4 = GD_F(k4), f5 = GD_F(k5), f6 = GD_F(k6), f7 = GD_F(k7);
#undef GD_F
                                p = __fmaf_rn(f0, f1, f2 * f3) + __fmaf_rn(f4, f5, f6 * f7);
                            }
                            pv[t] = p;
                            k++;
                            if (++z2 == u.ez) {
                                z2 = 0;
                                if (++y2 == u.ey) {
                                    y2 = 0;
                                    x2++;
                                }
                                if (k < u.K) set_run();
                            }
                        }
                        // BF16 hi / lo of each pair of products, two per conversion
                        // (the first at the lower address; p - hi is exact in FP32)
                        uint32_t hw[4], lw[4];
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const __nv_bfloat162 h2 = __floats2bfloat162_rn(pv[2 * q], pv[2 * q + 1]);
                            const __nv_bfloat162 l2 = __floats2bfloat162_rn(pv[2 * q] - __low2float(h2),
                                                                            pv[2 * q + 1] - __high2float(h2));
                            hw[q] = *reinterpret_cast<const uint32_t *>(&h2);
                            lw[q] = *reinterpret_cast<const uint32_t *>(&l2);
                        }
                        const uint4 hv = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                        const uint4 lv = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                        // 16-byte chunk j of this row, 128-byte swizzle
                        const uint32_t co = (((uint32_t)j ^ swz) & 7u) * 16u;
                        *reinterpret_cast<uint4 *>(pH + co) = hv;
                        *reinterpret_cast<uint4 *>(pL + co) = lv;
                    }
                    // generic-proxy writes, read next by the tensor cores
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(&full_bar[st]));
                }
            }
        }
        }
    }
    if (!ok) stop_flag = 1;
    // the unit is done in every role before unit_slot is written again
    __syncthreads();
    }  // units
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tmem_dealloc<1>(tmem, 2 * PT_NMAX);
    }
}

}  // namespace

namespace {

// Scale exponent of every cell: k = kAccBits - e with bound = max|f|^2 * imax1
// < 2^e, imax1 the largest gain of f = 1 on this grid.  Every pair product
// obeys |P(f)| <= max|f|^2 P(1), so every output's sum of |contributions| is at
// most the bound (the BF16 split of P and W changes it by ~1e-5 relative), and
// the fixed-point sums stay below 2^60.  Block = 32 cells x 8 node strides.
__global__ void pt_scale_kernel(const float *__restrict__ f, int ld, int n_pnt, int ncells, int cells_pad,
                                double imax1, int *__restrict__ kcell)
{
    __shared__ float fmax_s[8][32];
    __shared__ int bad_s[8][32];
    const int cx = threadIdx.x, cy = threadIdx.y;
    const int cell = blockIdx.x * 32 + cx;
    float fm = 0.f;
    int bad = 0;
    if (cell < ncells)
        for (int p = cy; p < n_pnt; p += 8) {
            const float v = fabsf(__ldg(f + (size_t)p * ld + cell));
            if (!(v <= 3.402823466e38f)) bad = 1;  // NaN or infinity
            else fm = fmaxf(fm, v);
        }
    fmax_s[cy][cx] = fm;
    bad_s[cy][cx] = bad;
    __syncthreads();
    if (cy == 0 && cell < cells_pad) {
        for (int y = 1; y < 8; y++) {
            fm = fmaxf(fm, fmax_s[y][cx]);
            bad |= bad_s[y][cx];
        }
        int k = 0;
        if (bad) {
            k = kBadScale;
        } else if (fm > 0.f && cell < ncells) {
            int e = 0;
            frexp((double)fm * (double)fm * imax1, &e);
            k = min(240, max(-120, kAccBits - e));
        }
        kcell[cell] = k;
    }
}

// Fixed-point sums back to FP32: acc * 2^-k, rounded once (the power-of-two
// factors are exact while the result is normal); NaN for a non-finite f.
__global__ void pt_convert_kernel(const long long *__restrict__ acc, const int *__restrict__ kcell, int n_pnt,
                                  int cells_pad, int ncells, int ld, float *__restrict__ gain)
{
    const int64_t outs = (int64_t)n_pnt * ncells;
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < outs; o += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(o / ncells), cell = (int)(o - (int64_t)p * ncells);
        const int k = __ldg(kcell + cell);
        float g;
        if (k == kBadScale) {
            g = __int_as_float(0x7fc00000);
        } else {
            const int k1 = k / 2, k2 = k - k / 2;
            g = __fmul_rn(__fmul_rn(__ll2float_rn(__ldg(acc + (size_t)p * cells_pad + cell)),
                                    __int_as_float((127 - k1) << 23)),
                          __int_as_float((127 - k2) << 23));
        }
        gain[(size_t)p * ld + cell] = g;
    }
}

}  // namespace

// Weight table of the tensor-core pair path: for every D (box-indexed like g),
// its groups' rows restricted to B(D), in chunks of 64 class offsets: rows
// wrow[D] + ch * mpad(D) + m hold group m's weights at offsets ch * 64 .. +63
// (BF16 hi and lo, zero past K_D and for the padding groups).
struct PairTc {
    __nv_bfloat16 *wh = nullptr, *wl = nullptr;
    int *wrow = nullptr;
    int *err = nullptr;   // set by the kernel when a pipeline wait times out
    int *next = nullptr;  // unit counter of the launches led by this context
    int64_t rows = 0;
    int max_items = 0;
    double imax1 = 0.0;   // largest gain of f = 1 (sets the cells' fixed-point scales)
    std::vector<int64_t> walk_prefix;          // [8 nxyz + 1] cumulative work along the walk
    std::map<int, int *> bounds_dev;           // chunk bounds on the walk, per chunk count
};

namespace {

int64_t table_rows(const Dims &d, const std::vector<int> &item_off, std::vector<int> *wrow)
{
    int64_t rows = 0;
    if (wrow) wrow->assign(d.nxyz, 0);
    for (int Dx = 0; Dx < d.nx; Dx++)
        for (int Dy = 0; Dy < d.ny; Dy++)
            for (int Dz = 0; Dz < d.nz; Dz++) {
                const int Did = (Dx * d.ny + Dy) * d.nz + Dz;
                const int64_t K = (int64_t)((Dx >> 1) + 1) * ((Dy >> 1) + 1) * ((Dz >> 1) + 1);
                const int m = item_off[Did + 1] - item_off[Did];
                if (wrow) (*wrow)[Did] = (int)rows;
                rows += (K + PT_KC - 1) / PT_KC * (int64_t)((m + 15) & ~15);
            }
    return rows;
}

int download_item_offsets(const Context &c, std::vector<int> &item_off)
{
    item_off.resize(c.d.nxyz + 1);
    GD_CUDA(cudaMemcpy(item_off.data(), c.d_D_item_off, sizeof(int) * (c.d.nxyz + 1), cudaMemcpyDeviceToHost));
    return GD_OK;
}

}  // namespace

double pair_tc_bytes(const Context &c)
{
    std::vector<int> item_off;
    if (download_item_offsets(c, item_off)) return 1e300;
    return (double)table_rows(c.d, item_off, nullptr) * PT_KC * 2.0 * 2.0;
}

void pair_tc_free(Context &c)
{
    if (!c.pair_tc) return;
    cudaFree(c.pair_tc->wh);
    cudaFree(c.pair_tc->wl);
    cudaFree(c.pair_tc->wrow);
    cudaFree(c.pair_tc->err);
    cudaFree(c.pair_tc->next);
    for (auto &kv : c.pair_tc->bounds_dev) cudaFree(kv.second);
    delete c.pair_tc;
    c.pair_tc = nullptr;
}

int pair_tc_build(Context &c)
{
    if (c.pair_tc) return GD_OK;
    const Dims &d = c.d;
    std::vector<int> item_off, wrow;
    int rc = download_item_offsets(c, item_off);
    if (rc) return rc;
    const int64_t n_items = item_off[d.nxyz];
    std::vector<int4> items(n_items + 1);
    GD_CUDA(cudaMemcpy(items.data(), c.d_D_items, sizeof(int4) * n_items, cudaMemcpyDeviceToHost));
    const int64_t rows = table_rows(d, item_off, &wrow);
    if (rows >= ((int64_t)1 << 31)) return set_error(GD_ERR_UNSUPPORTED, "pair weight table too large");
    const size_t bytes = (size_t)rows * PT_KC * sizeof(__nv_bfloat16);
    const size_t lim = memory_limit();
    if (lim && 2 * bytes > lim) return set_error(GD_ERR_OUT_OF_MEMORY, "pair weight table exceeds the memory limit");
    PairTc *pt = new PairTc;
    pt->rows = rows;
    cudaError_t e1 = cudaMalloc(&pt->wh, bytes), e2 = cudaMalloc(&pt->wl, bytes),
                e3 = cudaMalloc(&pt->wrow, sizeof(int) * d.nxyz), e4 = cudaMalloc(&pt->err, sizeof(int)),
                e5 = cudaMalloc(&pt->next, sizeof(int));
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess || e5 != cudaSuccess) {
        cudaFree(pt->wh);
        cudaFree(pt->wl);
        cudaFree(pt->wrow);
        cudaFree(pt->err);
        cudaFree(pt->next);
        delete pt;
        cudaGetLastError();
        return set_error(GD_ERR_OUT_OF_MEMORY, "pair weight table allocation");
    }
    c.pair_tc = pt;  // a failure below frees it again
    if (cudaMemcpy(pt->wrow, wrow.data(), sizeof(int) * d.nxyz, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(pt->err, 0, sizeof(int)) != cudaSuccess) {
        pair_tc_free(c);
        return set_error(GD_ERR_CUDA, "pair weight table upload");
    }

    // dense rows of every group in the class-box layout (x2 * hy + y2) * hz + z2,
    // built D by D into a host slab of at most ~128 MB per part and uploaded
    // slab by slab (D's rows are contiguous and in D order)
    const uint32_t unit = (uint32_t)c.gain_cb * 4u;
    const int64_t slab_cap = std::max<int64_t>((int64_t)1 << 20, 1);
    std::vector<__nv_bfloat16> sh, sl;
    int64_t slab0 = 0, slab_rows = 0;
    auto flush = [&]() -> int {
        if (slab_rows == 0) return GD_OK;
        const size_t nb = (size_t)slab_rows * PT_KC * sizeof(__nv_bfloat16);
        GD_CUDA(cudaMemcpy(pt->wh + (size_t)slab0 * PT_KC, sh.data(), nb, cudaMemcpyHostToDevice));
        GD_CUDA(cudaMemcpy(pt->wl + (size_t)slab0 * PT_KC, sl.data(), nb, cudaMemcpyHostToDevice));
        slab0 += slab_rows;
        slab_rows = 0;
        return GD_OK;
    };
    int max_items = 0;
    for (int Dx = 0; Dx < d.nx; Dx++)
        for (int Dy = 0; Dy < d.ny; Dy++)
            for (int Dz = 0; Dz < d.nz; Dz++) {
                const int Did = (Dx * d.ny + Dy) * d.nz + Dz;
                const int ex = (Dx >> 1) + 1, ey = (Dy >> 1) + 1, ez = (Dz >> 1) + 1;
                const int i0 = item_off[Did], m = item_off[Did + 1] - i0, mpad = (m + 15) & ~15;
                const int64_t K = (int64_t)ex * ey * ez, rows_d = (K + PT_KC - 1) / PT_KC * mpad;
                max_items = std::max(max_items, m);
                if (slab_rows > 0 && slab_rows + rows_d > slab_cap && (rc = flush())) {
                    pair_tc_free(c);
                    return rc;
                }
                const size_t need = (size_t)(slab_rows + rows_d) * PT_KC;
                if (sh.size() < need) {
                    sh.resize(need);
                    sl.resize(need);
                }
                const size_t base = (size_t)slab_rows * PT_KC;
                std::fill(sh.begin() + base, sh.begin() + need, __float2bfloat16_rn(0.f));
                std::fill(sl.begin() + base, sl.begin() + need, __float2bfloat16_rn(0.f));
                for (int t = 0; t < m; t++) {
                    const int gidx = items[i0 + t].x;
                    for (int e = c.h_grp_row_off[gidx]; e < c.h_grp_row_off[gidx + 1]; e++) {
                        const WEntry we = c.h_grp_rows[e];
                        if (we.w == 0.0f) continue;  // row padding
                        const int nc = (int)(we.off / unit);
                        const int z2 = nc % d.hz, y2 = (nc / d.hz) % d.hy, x2 = nc / (d.hz * d.hy);
                        if (x2 >= ex || y2 >= ey || z2 >= ez) continue;  // P is zero outside B(D)
                        const int k = (x2 * ey + y2) * ez + z2;
                        const size_t at = base + ((size_t)(k / PT_KC) * mpad + t) * PT_KC + k % PT_KC;
                        const __nv_bfloat16 hi = __float2bfloat16_rn(we.w);
                        sh[at] = hi;
                        sl[at] = __float2bfloat16_rn(we.w - __bfloat162float(hi));
                    }
                }
                slab_rows += rows_d;
            }
    if (!(rc = flush()) && slab0 != rows) rc = set_error(GD_ERR_CUDA, "pair weight table: row count mismatch");
    if (rc) {
        pair_tc_free(c);
        return rc;
    }
    pt->max_items = max_items;
    // the largest gain of f = 1, by the FP32 pair kernel on one cell
    float *ones = nullptr, *g1 = nullptr;
    cudaError_t e = cudaMalloc(&ones, sizeof(float) * d.n_pnt);
    if (e == cudaSuccess) e = cudaMalloc(&g1, sizeof(float) * d.n_pnt);
    std::vector<float> h1(d.n_pnt, 1.0f);
    if (e == cudaSuccess) e = cudaMemcpy(ones, h1.data(), sizeof(float) * d.n_pnt, cudaMemcpyHostToDevice);
    rc = e == cudaSuccess ? run_gain(c, ones, 1, 1, g1, 0) : cuda_error(e, "pair weight table: unit gain");
    if (!rc && (e = cudaMemcpy(h1.data(), g1, sizeof(float) * d.n_pnt, cudaMemcpyDeviceToHost)) != cudaSuccess)
        rc = cuda_error(e, "pair weight table: unit gain");
    cudaFree(ones);
    cudaFree(g1);
    if (rc) {
        pair_tc_free(c);
        return rc;
    }
    double m1 = 0.0;
    for (float v : h1) m1 = std::max(m1, (double)v);
    if (!(m1 > 0.0 && m1 < 1e300)) {
        pair_tc_free(c);
        return set_error(GD_ERR_CUDA, "pair weight table: unit gain not finite");
    }
    pt->imax1 = m1;
    // work along the walk (class box by class box, the reflections of each
    // box's pair sum in turn; repeated reflections are empty)
    pt->walk_prefix.assign((size_t)8 * d.nxyz + 1, 0);
    int64_t acc = 0;
    for (int Did = 0; Did < d.nxyz; Did++) {
        const int Dz = Did % d.nz, Dy = (Did / d.nz) % d.ny, Dx = Did / d.nyz;
        for (int r = 0; r < 8; r++) {
            pt->walk_prefix[(size_t)8 * Did + r] = acc;
            if (((r & 1) && Dx == d.nx - 1) || ((r & 2) && Dy == d.ny - 1) || ((r & 4) && Dz == d.nz - 1)) continue;
            const int sx = (r & 1) ? 2 * d.nx - 2 - Dx : Dx, sy = (r & 2) ? 2 * d.ny - 2 - Dy : Dy,
                      sz = (r & 4) ? 2 * d.nz - 2 - Dz : Dz;
            const int64_t sl = ((int64_t)sx * d.sy + sy) * d.sz + sz;
            acc += c.s_work_prefix[sl + 1] - c.s_work_prefix[sl];
        }
    }
    pt->walk_prefix[(size_t)8 * d.nxyz] = acc;
    return GD_OK;
}

namespace {

// Work-balanced chunk bounds on the walk, uploaded once per chunk count.
int pt_bounds_device(Context &c, int nchunks, const int **out)
{
    PairTc &pt = *c.pair_tc;
    auto it = pt.bounds_dev.find(nchunks);
    if (it == pt.bounds_dev.end()) {
        const std::vector<int64_t> &pre = pt.walk_prefix;
        const int npos = (int)pre.size() - 1;
        std::vector<int> bounds(nchunks + 1);
        bounds[0] = 0;
        for (int k = 1; k < nchunks; k++) {
            const int64_t target = pre[npos] * k / nchunks;
            bounds[k] = std::max(bounds[k - 1], (int)(std::lower_bound(pre.begin(), pre.end(), target) - pre.begin()));
        }
        bounds[nchunks] = npos;
        int *dev = nullptr;
        GD_CUDA(cudaMalloc(&dev, sizeof(int) * (nchunks + 1)));
        cudaError_t e = cudaMemcpy(dev, bounds.data(), sizeof(int) * (nchunks + 1), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(dev);
            return cuda_error(e, "pair tensor-core chunk bounds");
        }
        it = pt.bounds_dev.emplace(nchunks, dev).first;
    }
    *out = it->second;
    return GD_OK;
}

}  // namespace

int pair_tc_take_timeout(Context &c, cudaStream_t st, bool *timed_out)
{
    *timed_out = false;
    if (!c.pair_tc) return GD_OK;
    int flag = 0;
    GD_CUDA(cudaMemcpyAsync(&flag, c.pair_tc->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GD_CUDA(cudaStreamSynchronize(st));
    *timed_out = flag != 0;
    if (flag) {
        GD_CUDA(cudaMemsetAsync(c.pair_tc->err, 0, sizeof(int), st));
        GD_CUDA(cudaStreamSynchronize(st));
    }
    return GD_OK;
}

namespace {

// Chunks of one grid's walk for ncells cells: about 32 waves of one CTA per
// SM.  The work estimate of a box is rough, and a chunk of the walk holds few
// boxes, so units of equal estimated work end unevenly; many short units keep
// the tail short (20^3, 4096 cells: 459 ms with 32 waves, 468 with 16, 481
// with 4; 24^3, 1024 cells: 379, 392, 454 ms).
int pt_chunks(const Context &c, int ncells)
{
    const int tiles = (ncells + PT_BM - 1) / PT_BM;
    const int sms = std::max(1, c.sm_count);
    return (int)std::min<int64_t>(std::max(1, (32 * sms + tiles - 1) / tiles), c.d.ns);
}

// Cell tiles whose units run together: the accumulators they share (8 bytes
// per node and cell) stay within ~32 MB, far inside L2
int pt_tile_group(const Context &c, int tiles)
{
    const size_t per_tile = (size_t)c.d.n_pnt * PT_BM * sizeof(long long);
    return std::max(1, std::min(tiles, (int)(((size_t)32 << 20) / per_tile)));
}

}  // namespace

// The pair-product gain with the contraction on the tensor cores for one or
// more grids (each with its own context, cells and output) in one launch:
// each grid's walk over s is split into work-balanced chunks, and every
// (grid, 128-cell tile, chunk) unit adds its group sums into the grid's
// fixed-point accumulator, so the results do not depend on how the units are
// spread over the CTAs and equal those of separate launches bit for bit.  The
// units are ordered by their work, largest first; within a grid by groups of
// cell tiles whose accumulators fit L2 together, chunk-major inside a group
// (tiles fastest, so that the CTAs in flight share weight rows in L2).  One
// persistent CTA per SM pulls them from a device counter as it finishes its
// previous unit.  The unit list is uploaded once per launch shape and cached
// on the first job's context (a replayed graph reads it without a host copy);
// a pipeline time-out is recorded on that context.  Before the launch a small
// kernel sets every cell's scale; after it the sums are converted to FP32.
int launch_pair_tc(const PtJob *jobs, int njobs, cudaStream_t st)
{
    if (njobs < 1 || njobs > kPtMaxGrids) return set_error(GD_ERR_UNSUPPORTED, "pair tensor-core launch: 1-4 grids");
    Context &c0 = *jobs[0].c;
    PtLaunch L{};
    PtMaps maps{};
    std::vector<int> chunks(njobs), cells_pad(njobs);
    std::vector<double> unit_cost(njobs);
    std::string key;
    size_t smem = (size_t)kPtStages * kPtStage + 1024;
    int max_smem = 0;
    GD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c0.device));
    for (int j = 0; j < njobs; j++) {
        Context &c = *jobs[j].c;
        if (!c.pair_tc) return set_error(GD_ERR_INVALID_ARG, "pair weight table not built");
        for (int k = 0; k < j; k++)
            if (jobs[k].c == jobs[j].c) return set_error(GD_ERR_UNSUPPORTED, "one launch serves distinct contexts");
        const Dims &d = c.d;
        const int tiles = (jobs[j].ncells + PT_BM - 1) / PT_BM;
        cells_pad[j] = tiles * PT_BM;
        // the kernel forms node x stride offsets in 32 bits (5 % faster than 64)
        if ((int64_t)d.n_pnt * std::max(jobs[j].ld, cells_pad[j]) >= ((int64_t)1 << 31))
            return set_error(GD_ERR_UNSUPPORTED, "pair tensor-core gain: n_pnt * ld must stay below 2^31");
        chunks[j] = pt_chunks(c, jobs[j].ncells);
        unit_cost[j] = (double)c.s_work_prefix[d.ns] / chunks[j];
        const int *d_bounds = nullptr;
        int rc = pt_bounds_device(c, chunks[j], &d_bounds);
        if (rc) return rc;
        const size_t acc_bytes = (size_t)d.n_pnt * cells_pad[j] * sizeof(long long);
        if ((rc = ensure_scratch(c, acc_bytes + sizeof(int) * cells_pad[j]))) return rc;
        auto *acc = static_cast<unsigned long long *>(c.scratch.ptr);
        int *kcell = reinterpret_cast<int *>(static_cast<char *>(c.scratch.ptr) + acc_bytes);
        GD_CUDA(cudaMemsetAsync(acc, 0, acc_bytes, st));
        pt_scale_kernel<<<tiles * (PT_BM / 32), dim3(32, 8), 0, st>>>(jobs[j].f, jobs[j].ld, d.n_pnt, jobs[j].ncells,
                                                                        cells_pad[j], c.pair_tc->imax1, kcell);
        GD_CUDA(cudaGetLastError());
        const uint64_t dims[2] = {(uint64_t)PT_KC, (uint64_t)std::max<int64_t>(c.pair_tc->rows, 16)};
        const uint64_t strides[1] = {(uint64_t)PT_KC * 2};
        const uint32_t box[2] = {PT_KC, 16};
        if ((rc = encode_bf16_sw128(&maps.wh[j], c.pair_tc->wh, 2, dims, strides, box))) return rc;
        if ((rc = encode_bf16_sw128(&maps.wl[j], c.pair_tc->wl, 2, dims, strides, box))) return rc;
        L.g[j] = PtGrid{d, jobs[j].f, jobs[j].ld, jobs[j].ncells, cells_pad[j], c.d_cmap, c.d_D_item_off,
                        c.d_D_items, c.d_D_members, c.pair_tc->wrow, d_bounds, acc, kcell};
        key += std::to_string(tiles) + "x" + std::to_string(chunks[j]) + "c" +
               std::to_string((long long)unit_cost[j]) + ";";
    }
    // a single grid keeps its box -> compact map in shared memory when it fits
    const size_t cmap_bytes = ((size_t)c0.d.nxyz * 2 + 15) & ~(size_t)15;
    const bool cmap_smem = njobs == 1 && smem + cmap_bytes + 512 <= (size_t)max_smem;
    if (cmap_smem) smem += cmap_bytes;
    if (smem > (size_t)max_smem) return set_error(GD_ERR_UNSUPPORTED, "pair tensor-core kernel: shared memory");

    auto it = c0.pt_units_dev.find(key);
    if (it == c0.pt_units_dev.end()) {
        std::vector<int> order(njobs);
        for (int j = 0; j < njobs; j++) order[j] = j;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return unit_cost[a] > unit_cost[b]; });
        std::vector<int4> units;
        for (int j : order) {
            const int tiles = cells_pad[j] / PT_BM, grp = pt_tile_group(*jobs[j].c, tiles);
            for (int t0 = 0; t0 < tiles; t0 += grp)
                for (int ch = 0; ch < chunks[j]; ch++)
                    for (int t = t0; t < std::min(tiles, t0 + grp); t++) units.push_back(make_int4(j, t, ch, 0));
        }
        int4 *dev = nullptr;
        GD_CUDA(cudaMalloc(&dev, sizeof(int4) * units.size()));
        cudaError_t e = cudaMemcpy(dev, units.data(), sizeof(int4) * units.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(dev);
            return cuda_error(e, "pair tensor-core unit list");
        }
        it = c0.pt_units_dev.emplace(key, std::make_pair(dev, (int)units.size())).first;
    }
    L.units = it->second.first;
    L.nunits = it->second.second;
    L.err = c0.pair_tc->err;
    L.next = c0.pair_tc->next;
    GD_CUDA(cudaMemsetAsync(L.next, 0, sizeof(int), st));
    const int ctas = std::min(L.nunits, std::max(1, c0.sm_count));
    if (cmap_smem) {
        GD_CUDA(cudaFuncSetAttribute(pair_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        pair_tc_kernel<true><<<ctas, kPtThreads, smem, st>>>(maps, L);
    } else {
        GD_CUDA(cudaFuncSetAttribute(pair_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        pair_tc_kernel<false><<<ctas, kPtThreads, smem, st>>>(maps, L);
    }
    GD_CUDA(cudaGetLastError());
    // the kernel records a pipeline time-out instead of hanging; the call only
    // enqueues work, and gd_ctx_check reports the record
    for (int j = 0; j < njobs; j++) {
        const Context &c = *jobs[j].c;
        const int64_t outs = (int64_t)c.d.n_pnt * jobs[j].ncells;
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((outs + 255) / 256, (int64_t)c.sm_count * 16));
        pt_convert_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const long long *>(L.g[j].acc), L.g[j].kcell,
                                                  c.d.n_pnt, cells_pad[j], jobs[j].ncells, jobs[j].ld, jobs[j].gain);
        GD_CUDA(cudaGetLastError());
    }
    return GD_OK;
}

int run_pair_tc(Context &c, const float *f, int ncells, int ld, float *gain, cudaStream_t st)
{
    const PtJob job{&c, f, ncells, ld, gain};
    return launch_pair_tc(&job, 1, st);
}

}  // namespace gd

extern "C" int gd_pair_tc_table(gd_ctx *ctx, int64_t *rows, int *wrow, uint16_t *wh, uint16_t *wl)
{
    using namespace gd;
    if (!ctx || !rows) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    Context &c = ctx->c;
    if (!c.pair_tc) return set_error(GD_ERR_UNSUPPORTED, "the pair tensor-core weight table is not built");
    DeviceGuard g(c.device);
    *rows = c.pair_tc->rows;
    if (wrow) GD_CUDA(cudaMemcpy(wrow, c.pair_tc->wrow, sizeof(int) * c.d.nxyz, cudaMemcpyDeviceToHost));
    const size_t bytes = (size_t)c.pair_tc->rows * PT_KC * sizeof(__nv_bfloat16);
    if (wh) GD_CUDA(cudaMemcpy(wh, c.pair_tc->wh, bytes, cudaMemcpyDeviceToHost));
    if (wl) GD_CUDA(cudaMemcpy(wl, c.pair_tc->wl, bytes, cudaMemcpyDeviceToHost));
    return GD_OK;
}
