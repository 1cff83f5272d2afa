// gd_cmatrix.cu -- collision-matrix form of the gain on the tensor cores (sm_103a).
//
// The gain is a bilinear form in f: I_i = sum_{a,b} G_i[a][b] f_a f_b.  With
// s = a + b, d = a - b (lattice offsets) the reference's enumeration
// (collision_integral.cu:75-188: partner i1 = s - i, post-collision offset
// n = |d|, four sign patterns) gives the symmetric matrix
//   G_i[a][b] = m(d) * w(|2i - s|, |d|) * [s - i in the box],
//   m(d) = (d_x == 0 ? 1 : 1/2) * (d_y == 0 ? 2 : 1) * (d_z == 0 ? 2 : 1),
// with w the analytic weight table (compute_matrix.cu:505-562).  G is stored
// in BF16 (optionally as hi + lo parts) as the 256 x 64 tiles of its block
// upper triangle that hold a nonzero entry, with the nodes in a Hilbert-curve
// matrix order, and only for one node per orbit of the lattice's reflections
// (node R(i) uses G_i with f reflected by R).
//
// Contraction: for output node i and 128 cells c,
//   D[c][b] = sum_a F[c][a] G_i[a][b]   (tcgen05.mma, BF16 x BF16 -> FP32 in TMEM)
//   I[i][c] = sum_b D[c][b] f[b][c]      (epilogue, FP32)
// One CTA per (128-cell tile, i), by default two CTAs per cluster running each
// MMA as a CTA pair (M = 256 cells); one launch may serve several grids.  Warp 0 issues TMA loads of F (cells x
// 64 a) and of G_i (256 b x 64 a, or this CTA's half of it) into a ring of
// shared-memory stages (128-byte swizzle); warp 1 issues the MMAs (N = 256,
// K = 16) into one of two TMEM accumulators, or relays its CTA's landed
// stages to the pair's issuing CTA; warps 2..9 read the finished accumulator
// with tcgen05.ld and fold it into the per-cell sums while the next one is
// being filled.  Every mbarrier wait is bounded: on time-out the CTA records
// an error and stops issuing work instead of waiting forever.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_tc.cuh"


namespace gd {
namespace {

constexpr int BM = 128;  // cells per tile (MMA M, TMEM lanes)
constexpr int BN = 256;  // b per accumulator tile (MMA N, TMEM columns)
constexpr int BK = 64;   // a per stage (128 bytes of BF16: one swizzle row)
constexpr int kSlices = BK / 16;  // MMA K steps per tile, skipped one by one when all zero
constexpr int kEpiWarps = 8;  // two per TMEM lane quadrant, 128 accumulator columns each
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kTileA = BM * BK * 2;  // 16 KB
constexpr uint32_t kTileB = BN * BK * 2;  // 32 KB
using namespace tc;

// Ring of shared-memory stages (192 KB) for NPASS passes and CL CTAs per
// MMA.  A stage holds cm_tiles_per_stage consecutive stored tiles of one
// b-tile group, each tile its F tile(s) and this CTA's rows of its G
// tile(s).  One-pass CTA pairs put two tiles in a stage: their stream was
// bound by the handshakes per stage (full/empty barriers, relay), not by the
// bytes, and two tiles per stage (three stages) run at the tensor pipe's rate
// where one tile (six stages) reached 86 % of it; one CTA per MMA keeps one
// tile per stage (its 48 KB tiles would leave only two stages).
__host__ __device__ constexpr int cm_tiles_per_stage(int npass, int cl) { return npass == 1 && cl == 2 ? 2 : 1; }
__host__ __device__ constexpr uint32_t cm_tile_bytes(int npass, int cl)
{
    return (npass == 1 ? 1u : 2u) * (kTileA + kTileB / (uint32_t)cl);
}
__host__ __device__ constexpr uint32_t cm_stage_bytes(int npass, int cl)
{
    return (uint32_t)cm_tiles_per_stage(npass, cl) * cm_tile_bytes(npass, cl);
}
__host__ __device__ constexpr int cm_stages(int npass, int cl) { return (int)((192u << 10) / cm_stage_bytes(npass, cl)); }

// Stored tiles in the stage that starts at list entry j of a node's cnt
// tiles: two when allowed and entry j + 1 belongs to the same b-tile group.
// A stored tile's list entry: mask << 28 | n << 16 | k, with n its 256-row
// b-tile, k its 64-column a-tile and bit kk of mask set when columns
// 16 kk .. 16 kk + 15 hold a nonzero entry (the MMAs of all-zero 16-column
// slices are skipped).
__device__ __forceinline__ uint32_t tile_n(uint32_t e) { return (e >> 16) & 0xfffu; }
__device__ __forceinline__ uint32_t tile_k(uint32_t e) { return e & 0xffffu; }
__device__ __forceinline__ uint32_t tile_mask(uint32_t e) { return e >> 28; }

__device__ __forceinline__ int stage_len(const uint32_t *tiles, int j, int cnt, int tps)
{
    if (tps == 1 || j + 1 >= cnt) return 1;
    return tile_n(__ldg(tiles + j)) == tile_n(__ldg(tiles + j + 1)) ? 2 : 1;
}

// The tensor cores' FP32 accumulation loses precision over long sums (the
// collision-matrix gain against FP64 at 20^3: median relative error 2.5e-6
// with whole b-tile runs of ~25 tiles per accumulation, 6.4e-7 with at most
// four): in BF16x3 mode by default at most four 64-column tiles (256
// products per entry) go into one accumulation, the epilogue adding the runs
// in FP32 with compensation (2 % of the gain launch).  One BF16 pass is
// limited by the rounding of its operands (~3e-4), not by the accumulation,
// so it keeps whole b-tile runs (unlimited chain).  The tensor-core loss
// always sums K in chunks of kLossChunk columns per launch.
constexpr int kDefaultChainBf16x3 = 4;
constexpr int kChainUnlimited = 1 << 30;
constexpr int kLossChunk = 256;

struct CmParams {
    int ns;       // in-sphere nodes
    int ns_k;     // padded node count (multiple of BK)
    int ncells, ld;
    const float *f;  // [8][ns_k][ldf] FP32 distribution in matrix order, per reflection (epilogue)
    int ldf;
    float *gain;     // [ns][ld]
    int *err;        // set to 1 when a wait times out
    const int *node_off;     // [orbits + 1] each orbit representative's range of stored tiles
    const uint32_t *tiles;   // stored tiles (mask << 28 | n << 16 | k), n-major then k per representative
    const int *orbit;        // [ns] node -> representative's slot << 3 | reflection
    const int *order;        // [ns] the nodes in launch order (reflection-major)
    int m_tiles;             // cell tiles, padded to whole clusters
    int chain;               // most stored tiles summed in one tensor-memory accumulation (even)
};

// One launch serves up to kCmMaxGrids velocity grids (each with its own
// matrices, f and gain): blockIdx.y in [ystart[j], ystart[j + 1]) is node
// blockIdx.y - ystart[j] (in launch order) of grid j, blockIdx.x its cell
// tile (CTAs past the grid's m_tiles leave at once, pairs together).
constexpr int kCmMaxGrids = 4;
struct CmLaunch {
    CmParams g[kCmMaxGrids];
    int ystart[kCmMaxGrids + 1];
    int ngrids;
};
// the grids' tensor maps: f (hi, lo; one copy per reflection) and G (hi, lo)
struct CmMaps {
    CUtensorMap fh[kCmMaxGrids], fl[kCmMaxGrids], gh[kCmMaxGrids], gl[kCmMaxGrids];
};

// G_i is symmetric in (a, b), so only its block upper triangle is stored and
// contracted: entries with a < b doubled, the diagonal kept, a > b zero.  The
// b-tile n (rows b in [n BN, (n+1) BN)) then needs the a-tiles up to the end
// of its own b range.
__host__ __device__ __forceinline__ int k_end(int n, int num_k)
{
    const int e = ((n + 1) * BN + BK - 1) / BK;
    return e < num_k ? e : num_k;
}

// NPASS = 1: D = F_hi G_hi.  NPASS = 3: D = F_hi G_hi + F_hi G_lo + F_lo G_hi.
// CL = 2: a CTA pair (cluster of two) holding adjacent cell tiles of the same
// node runs each tile as one pair MMA (tcgen05 cta_group::2, M = 256 cells):
// each CTA loads its own F tile and half of the G tile (BN / 2 rows), the even
// CTA issues the MMAs, and each CTA's tensor memory receives its own cells'
// rows.  A CTA then brings 32 KB per tile into its shared memory instead of
// 48 KB, and a G tile crosses L2 once per pair.
template <int NPASS, int CL, bool MULTI>
__global__ void __launch_bounds__(kThreads, 1)
    cmatrix_gain_kernel(const __grid_constant__ CmMaps maps, const __grid_constant__ CmLaunch L)
{
    // MULTI: several grids in the launch (the fused batch); a single grid
    // reads its parameters at constant offsets (selecting them by a runtime
    // index costs registers, and the kernel is at its register limit)
    int gj = 0;
    if (MULTI)
        while (gj + 1 < L.ngrids && (int)blockIdx.y >= L.ystart[gj + 1]) gj++;
    const CmParams &p = L.g[MULTI ? gj : 0];
    // cell tiles past this grid's extent (m_tiles is a multiple of CL, so the
    // two CTAs of a pair leave together, before any barrier)
    if ((int)blockIdx.x >= p.m_tiles) return;
    const int mj = MULTI ? gj : 0;
    const CUtensorMap &tmFh = maps.fh[mj], &tmFl = maps.fl[mj], &tmGh = maps.gh[mj], &tmGl = maps.gl[mj];
    constexpr int NPARTS = NPASS == 1 ? 1 : 2;
    constexpr bool PAIR = CL == 2;
    constexpr uint32_t kTileBc = kTileB / CL;  // this CTA's rows of a G tile
    constexpr int S = cm_stages(NPASS, CL);  // pipeline stages
    constexpr int TPS = cm_tiles_per_stage(NPASS, CL);
    constexpr uint32_t kTileSlot = cm_tile_bytes(NPASS, CL);
    constexpr uint32_t kStage = cm_stage_bytes(NPASS, CL);
    static_assert(kTileSlot == NPARTS * (kTileA + kTileBc) && S >= 2, "stage layout");
    constexpr uint32_t kIdescT = umma_idesc_bf16(BM * CL, BN);
    extern __shared__ __align__(1024) unsigned char dsmem[];
    // 1024-byte aligned tile area
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t full_bar[S], empty_bar[S], accf_bar[2], acce_bar[2];
    __shared__ uint32_t tmem_base_holder;
    __shared__ int abort_flag;
    __shared__ int epi_failed;
    __shared__ float half_sum[BM];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (!PAIR) {
        if (threadIdx.x == 0) abort_flag = *(volatile int *)p.err;
        __syncthreads();
        if (abort_flag) return;  // an earlier CTA timed out: do no work
    } else {
        // paired CTAs never leave early: both must reach the cluster barriers
        if (threadIdx.x == 0) abort_flag = 0;
    }
    if (threadIdx.x == 0) epi_failed = 0;
    const uint32_t crank = PAIR ? cluster_rank() : 0u;
    const bool leader = crank == 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            // the even CTA's full barrier also takes the odd CTA's relay arrival
            mbar_init(smem_u32(&full_bar[s]), (PAIR && leader) ? 2 : 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);  // the MMA commit
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&accf_bar[b]), 1);
            mbar_init(smem_u32(&acce_bar[b]), CL * kEpiWarps);  // every epilogue warp of the pair
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        tmem_alloc<CL>(smem_u32(&tmem_base_holder), 2 * BN);
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    if (PAIR) cluster_sync();  // the peer's barriers exist before any arrival or commit reaches them
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_holder;

    // one CTA per (cell tile, node); a pair holds adjacent cell tiles of one node.
    // Node i = R(i0) for the representative i0 of its orbit under the lattice's
    // reflections: G_i[a][b] = G_i0[R a][R b], so I_i(f) = I_i0(f o R), and the
    // CTA contracts i0's stored tiles with the copy of f reflected by R.
    const int m_tile = blockIdx.x, node = __ldg(p.order + (blockIdx.y - (MULTI ? L.ystart[gj] : 0)));
    const int ob = __ldg(p.orbit + node), rep = ob >> 3, refl = ob & 7;
    const int l0 = __ldg(p.node_off + rep), cnt = __ldg(p.node_off + rep + 1) - l0;

    if (warp == 0) {
        // ---- TMA producer (both CTAs; each fills its own stages) ---------------
        if (lane == 0) {
            const uint32_t *tl = p.tiles + l0;
            int it = 0;
            for (int j = 0; j < cnt; it++) {
                const int s = it % S;
                const uint32_t ph = (uint32_t)(it / S) & 1u;
                if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, p.err)) {
                    abort_flag = 1;
                    break;
                }
                if (*(volatile int *)&abort_flag) break;
                const int len = stage_len(tl, j, cnt, TPS);
                unsigned char *st = base + (size_t)s * kStage;
                const uint32_t fb = smem_u32(&full_bar[s]);
                mbar_expect_tx(fb, (uint32_t)len * kTileSlot);
                for (int t = 0; t < len; t++) {
                    // F: this CTA's cells; G: stored tile l0 + j + t ([slot][BN rows][BK]),
                    // this CTA's BN / CL rows of it
                    const int k = (int)tile_k(__ldg(tl + j + t));
                    unsigned char *ts = st + (size_t)t * kTileSlot;
                    tma_load_3d(smem_u32(ts), &tmFh, k * BK, m_tile * BM, refl, fb);
                    tma_load_3d(smem_u32(ts + kTileA), &tmGh, 0, (int)crank * (BN / CL), l0 + j + t, fb);
                    if (NPARTS == 2) {
                        tma_load_3d(smem_u32(ts + kTileA + kTileBc), &tmFl, k * BK, m_tile * BM, refl, fb);
                        tma_load_3d(smem_u32(ts + 2 * kTileA + kTileBc), &tmGl, 0, (int)crank * (BN / CL),
                                    l0 + j + t, fb);
                    }
                }
                j += len;
            }
            if (PAIR) {
                // tail, bounded like every wait: the copies of the last stages have
                // landed, and the pair MMAs that read them have completed (their
                // commits have arrived here), before this CTA may leave the pair;
                // after a time-out the waits give up at once
                const int j0 = it > S ? it - S : 0;
                for (int j = j0; j < it; j++)
                    if (!mbar_wait(smem_u32(&full_bar[j % S]), (uint32_t)(j / S) & 1u, p.err)) break;
                for (int j = j0; j < it; j++)
                    if (!mbar_wait(smem_u32(&empty_bar[j % S]), (uint32_t)(j / S) & 1u, p.err)) break;
            }
        }
    } else if (warp == 1 && PAIR && !leader) {
        // ---- relay (odd CTA): its stage s has landed -> arrive on the even CTA's
        // full barrier, so the pair MMA reads both halves only when both are in
        if (lane == 0) {
            const uint32_t *tl = p.tiles + l0;
            for (int j = 0, it = 0; j < cnt; it++) {
                const int s = it % S;
                if (!mbar_wait(smem_u32(&full_bar[s]), (uint32_t)(it / S) & 1u, p.err)) break;
                mbar_arrive_cluster(mapa_cluster(smem_u32(&full_bar[s]), 0));
                j += stage_len(tl, j, cnt, TPS);
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer (one CTA, or the even CTA of a pair) --------------------
        if (lane == 0) {
            bool ok = true;
            int it = 0, grp = 0;  // stage counter; groups of tiles sharing one b-tile n
            int j = 0;
            while (ok && j < cnt) {
                const uint32_t n = tile_n(__ldg(p.tiles + l0 + j));
                const int buf = grp & 1;
                const uint32_t use = (uint32_t)(grp >> 1);
                if (!mbar_wait(smem_u32(&acce_bar[buf]), (use & 1u) ^ 1u, p.err)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d_tmem = tmem + (uint32_t)(buf * BN);
                bool first = true;
                const int jg = j;  // an accumulation: tiles of one b-tile, at most p.chain of them
                while (j < cnt && tile_n(__ldg(p.tiles + l0 + j)) == n && j - jg < p.chain) {
                    const int s = it % S;
                    const uint32_t ph = (uint32_t)(it / S) & 1u;
                    // the stage's tile entries, read before the wait so that
                    // their latency hides behind it
                    const int len = stage_len(p.tiles + l0, j, cnt, TPS);
                    const uint32_t masks = tile_mask(__ldg(p.tiles + l0 + j)) |
                                           (len > 1 ? tile_mask(__ldg(p.tiles + l0 + j + 1)) << 4 : 0u);
                    if (!mbar_wait(smem_u32(&full_bar[s]), ph, p.err)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    for (int t = 0; t < len; t++) {
                        const uint32_t ts = smem_u32(base + (size_t)s * kStage + (size_t)t * kTileSlot);
                        const uint32_t aH = ts, bH = ts + kTileA;
                        const uint32_t aL = ts + kTileA + kTileBc, bL = ts + 2 * kTileA + kTileBc;
                        // one BF16 pass issues whole tiles: its stream is bound by the
                        // handshakes per stage, and skipping slices there cost time
                        // (88 against 96 ms at 20^3); BF16x3 skips the all-zero ones
                        const uint32_t mask = NPASS == 1 ? 0xfu : (masks >> (4 * t)) & 0xfu;
#pragma unroll
                        for (int kk = 0; kk < BK / 16; kk++) {
                            if (!((mask >> kk) & 1u)) continue;  // an all-zero slice of G
                            const uint32_t off = (uint32_t)kk * 32u;  // 16 BF16 along K
                            const uint32_t acc = first ? 0u : 1u;
                            first = false;
                            if (PAIR) {
                                umma_bf16_pair(d_tmem, umma_desc(aH + off), umma_desc(bH + off), kIdescT, acc);
                                if (NPASS == 3) {
                                    umma_bf16_pair(d_tmem, umma_desc(aH + off), umma_desc(bL + off), kIdescT, 1u);
                                    umma_bf16_pair(d_tmem, umma_desc(aL + off), umma_desc(bH + off), kIdescT, 1u);
                                }
                            } else {
                                umma_bf16(d_tmem, umma_desc(aH + off), umma_desc(bH + off), kIdescT, acc);
                                if (NPASS == 3) {
                                    umma_bf16(d_tmem, umma_desc(aH + off), umma_desc(bL + off), kIdescT, 1u);
                                    umma_bf16(d_tmem, umma_desc(aL + off), umma_desc(bH + off), kIdescT, 1u);
                                }
                            }
                        }
                    }
                    // the stage is free in both CTAs once these MMAs have read it
                    if (PAIR)
                        umma_commit_pair_mc(smem_u32(&empty_bar[s]), (uint16_t)3u);
                    else
                        umma_commit(smem_u32(&empty_bar[s]));
                    j += len;
                    it++;
                }
                if (!ok) break;
                if (PAIR)
                    umma_commit_pair_mc(smem_u32(&accf_bar[buf]), (uint16_t)3u);
                else
                    umma_commit(smem_u32(&accf_bar[buf]));
                grp++;
            }
            if (!ok) abort_flag = 1;
        }
    } else if (warp >= 2) {
        // ---- epilogue: warps 2..9; warp % 4 is the TMEM lane quadrant it may
        // read, (warp - 2) / 4 the half of the accumulator columns it takes ---
        const int quad = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = quad * 32 + lane;
        int grp = 0;
        bool failed = false;
        const int cell = m_tile * BM + row;
        const bool live = cell < p.ncells;
        // the gain of this cell (this half's columns): each accumulation's
        // 128 products D[c][b] f_b are summed in four interleaved partials,
        // and the accumulations' sums are added with compensated (Kahan)
        // summation, so the rounding of one long FP32 chain of thousands of
        // terms does not limit the result
        float sum = 0.f, comp = 0.f;
        // f[b][cell] for this warp's 128 b of a group; rows b >= ns of G are
        // zero, so T[b] = 0 there and clamping b keeps every load in bounds
        // without a branch.  A group's values are requested as soon as the
        // previous group is folded, so they arrive while its MMAs run.
        const float *fcell = p.f + (size_t)refl * p.ns_k * p.ldf + (live ? cell : 0);
        float fv[BN / 2];
        auto load_f = [&](int b0) {
#pragma unroll
            for (int q = 0; q < BN / 2; q++) fv[q] = __ldg(fcell + (size_t)min(b0 + q, p.ns - 1) * p.ldf);
        };
        int j = 0;
        int n = cnt > 0 ? (int)tile_n(__ldg(p.tiles + l0)) : 0;
        if (live && cnt > 0) load_f(n * BN + half * (BN / 2));
        for (; j < cnt; grp++) {
            // b-tiles without stored tiles contribute nothing and are skipped;
            // a b-tile's run of tiles comes in accumulations of at most p.chain
            const int jg = j;
            while (j < cnt && (int)tile_n(__ldg(p.tiles + l0 + j)) == n && j - jg < p.chain) j++;
            const int n_next = j < cnt ? (int)tile_n(__ldg(p.tiles + l0 + j)) : -1;
            const int buf = grp & 1;
            const uint32_t use = (uint32_t)(grp >> 1);
            bool ok = true;
            if (lane == 0) ok = mbar_wait(smem_u32(&accf_bar[buf]), use & 1u, p.err);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) {
                failed = true;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t taddr =
                tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * BN) + (uint32_t)(half * (BN / 2));
            float ps[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int c0 = 0; c0 < BN / 2; c0 += 16) {
                float v[16];
                tmem_ld16(taddr + (uint32_t)c0, v);
                if (live) {
#pragma unroll
                    for (int q = 0; q < 16; q++) ps[q & 3] = __fmaf_rn(v[q], fv[c0 + q], ps[q & 3]);
                }
            }
            {
                const float part = __fadd_rn(__fadd_rn(ps[0], ps[1]), __fadd_rn(ps[2], ps[3]));
                const float y = __fsub_rn(part, comp);
                const float t = __fadd_rn(sum, y);
                comp = __fsub_rn(__fsub_rn(t, sum), y);
                sum = t;
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            // report the drained accumulator to the MMA issuer's CTA
            if (lane == 0) {
                if (PAIR)
                    mbar_arrive_cluster(mapa_cluster(smem_u32(&acce_bar[buf]), 0));
                else
                    mbar_arrive(smem_u32(&acce_bar[buf]));
            }
            // the next accumulation of the same b-tile reuses fv
            if (live && n_next >= 0 && n_next != n) load_f(n_next * BN + half * (BN / 2));
            n = n_next;
        }
        // the two column halves of a cell are added in a fixed order
        if (failed) epi_failed = 1;
        if (half == 1) half_sum[row] = sum;
        asm volatile("bar.sync 1, %0;" ::"n"(32 * kEpiWarps) : "memory");
        if (half == 0 && live && !epi_failed) p.gain[(size_t)node * p.ld + cell] = sum + half_sum[row];
    }
    __syncthreads();
    if (PAIR) cluster_sync();  // no remote write or arrival can reach this CTA after it leaves
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tmem_dealloc<CL>(tmem, 2 * BN);
    }
}

// G_i in tiles of BN rows (b) x BK columns (a): tile t of the block upper
// triangle is (n, k) = tile_nk[t], stored at [i][t][b - n BN][a - k BK];
// hi = bf16(v), lo = bf16(v - hi), v = u(a, b) m(d) w(|2i - s|, |d|) [s - i in
// box] with u = 2 above the diagonal (a < b), 1 on it, 0 below (G_i is
// symmetric, so the triangle carries the whole bilinear form).  Zero for
// padding rows and columns.
//
// Two passes: with nz set, only mark the triangle tiles holding a nonzero
// entry (every writer stores 1); otherwise write each entry into the stored
// slot slot_of[i * tiles + t] of its tile (tiles that are all zero have no slot).
__global__ void assemble_g_kernel(Dims d, int nout, int tiles, const int2 *__restrict__ tile_nk,
                                  const uint32_t *__restrict__ nodes, const uint32_t *__restrict__ mnodes,
                                  const float *__restrict__ w_dense,
                                  uint8_t *__restrict__ nz, const int *__restrict__ slot_of,
                                  __nv_bfloat16 *__restrict__ gh, __nv_bfloat16 *__restrict__ gl)
{
    const int64_t rows = (int64_t)nout * tiles * BN;  // (i, t, b) rows of BK entries, i < nout
    constexpr int vec = BK / 8;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < rows * vec;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = q / vec;
        const int rr = (int)(r % BN);
        const int64_t it = r / BN;
        const int t = (int)(it % tiles), i = (int)(it / tiles);
        const int slot = nz ? 0 : slot_of[it];
        if (slot < 0) continue;
        const int2 nk = tile_nk[t];
        const int b = nk.x * BN + rr;
        const int a0 = nk.y * BK + (int)(q % vec) * 8;
        __align__(16) __nv_bfloat16 hv[8], lv[8];
        const uint32_t qi = nodes[i];
        const int ix = qi & 1023, iy = (qi >> 10) & 1023, iz = qi >> 20;
        const bool bin = b < d.n_pnt;
        const uint32_t qb = bin ? mnodes[b] : 0u;
        const int bx = qb & 1023, by = (qb >> 10) & 1023, bz = qb >> 20;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int a = a0 + j;
            float v = 0.f;
            if (bin && a < d.n_pnt && a <= b) {
                const uint32_t qa = mnodes[a];
                const int ax = qa & 1023, ay = (qa >> 10) & 1023, az = qa >> 20;
                const int sx = ax + bx, sy = ay + by, sz = az + bz;
                const int jx = sx - ix, jy = sy - iy, jz = sz - iz;  // partner i1
                if (jx >= 0 && jx < d.nx && jy >= 0 && jy < d.ny && jz >= 0 && jz < d.nz) {
                    const int dx = abs(ax - bx), dy = abs(ay - by), dz = abs(az - bz);
                    const int gx = abs(2 * ix - sx), gy = abs(2 * iy - sy), gz = abs(2 * iz - sz);
                    const int64_t widx =
                        ((int64_t)((dx >> 1) * d.nx + gx) * (d.hy * d.hz) + (dy >> 1) * d.hz + (dz >> 1)) * d.nyz +
                        gy * d.nz + gz;
                    const float m = (dx == 0 ? 1.f : 0.5f) * (dy == 0 ? 2.f : 1.f) * (dz == 0 ? 2.f : 1.f);
                    const float g = m * w_dense[widx];
                    v = a < b ? 2.f * g : g;  // exact factor 2
                }
            }
            hv[j] = __float2bfloat16_rn(v);
            lv[j] = __float2bfloat16_rn(v - __bfloat162float(hv[j]));
        }
        if (nz) {  // one byte per 16-column slice of the tile
            bool any = false;
#pragma unroll
            for (int j = 0; j < 8; j++) any |= __bfloat162float(hv[j]) != 0.f;
            if (any) nz[it * (BK / 16) + (int)(q % vec) / 2] = 1;
            continue;
        }
        const size_t o = ((size_t)slot * BN + rr) * BK + (size_t)(q % vec) * 8;
        *reinterpret_cast<uint4 *>(gh + o) = *reinterpret_cast<const uint4 *>(hv);
        if (gl) *reinterpret_cast<uint4 *>(gl + o) = *reinterpret_cast<const uint4 *>(lv);
    }
}

// Loss matrix B[i][j] = b(|i - j|) (hi/lo BF16, j padded to ns_k with zeros),
// so that nu = B f is a GEMM: nu[i][c] = sum_j B[i][j] f[j][c].
__global__ void assemble_b_kernel(Dims d, int ns_k, const uint32_t *__restrict__ nodes,
                                  const uint32_t *__restrict__ mnodes, const float *__restrict__ b,
                                  __nv_bfloat16 *__restrict__ bh, __nv_bfloat16 *__restrict__ bl)
{
    const int64_t total = (int64_t)d.n_pnt * ns_k;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q / ns_k), j = (int)(q % ns_k);
        float v = 0.f;
        if (j < d.n_pnt) {
            const uint32_t pi = nodes[i], pj = mnodes[j];
            const int dx = abs((int)(pi & 1023) - (int)(pj & 1023));
            const int dy = abs((int)((pi >> 10) & 1023) - (int)((pj >> 10) & 1023));
            const int dz = abs((int)(pi >> 20) - (int)(pj >> 20));
            v = b[dx * d.nyz + dy * d.nz + dz];
        }
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        bh[q] = h;
        bl[q] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

// F[c][a] (BF16 hi/lo, a contiguous, padded to ns_k) from f (FP32, [node][c])
// in matrix order: column a holds node inv[a].  With fp set, also the FP32
// rows in matrix order, fp[a][c] (leading dimension ldf), for the epilogue.
__global__ void convert_f_kernel(const float *__restrict__ f, int ns, int ns_k, int ncells, int ld,
                                 const int *__restrict__ inv, __nv_bfloat16 *__restrict__ fh,
                                 __nv_bfloat16 *__restrict__ fl, float *__restrict__ fp, int ldf, int f_rows)
{
    __shared__ float tile[32][33];
    const int a0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    // blockIdx.z = R: the copy of f reflected by R (inv + R ns maps matrix
    // index -> node R(inv[m])), stacked R-major
    const int R = blockIdx.z;
    inv += (size_t)R * ns;
    fh += (size_t)R * f_rows * ns_k;
    if (fl) fl += (size_t)R * f_rows * ns_k;
    if (fp) fp += (size_t)R * ns_k * ldf;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int a = a0 + r, c = c0 + threadIdx.x;
        const float v = (a < ns && c < ncells) ? f[(size_t)__ldg(inv + a) * ld + c] : 0.f;
        tile[r][threadIdx.x] = v;
        if (fp && a < ns_k && c < ncells) fp[(size_t)a * ldf + c] = v;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int c = c0 + r, a = a0 + threadIdx.x;
        if (c < ncells && a < ns_k) {
            const float v = tile[threadIdx.x][r];
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            fh[(size_t)c * ns_k + a] = h;
            if (fl) fl[(size_t)c * ns_k + a] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int get_encoder(EncodeTiled *out)
{
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
            return set_error(GD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
        fn = reinterpret_cast<EncodeTiled>(p);
    }
    *out = fn;
    return GD_OK;
}

int encode(EncodeTiled fn, CUtensorMap *m, void *ptr, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
           const cuuint32_t *box)
{
    const cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, ptr, dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(GD_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GD_OK;
}

}  // namespace
}  // namespace gd

struct gd_cmatrix {
    gd_ctx *ctx = nullptr;
    int mode = 0;  // GD_CMATRIX_BF16 or GD_CMATRIX_BF16X3
    int ns = 0, ns_k = 0;
    int tiles = 0;       // BN x BK tiles of one node's block upper triangle
    int cluster = 2;     // CTAs per MMA: 2 (CTA-pair MMA, M = 256 cells; the default) or 1
    // matrices are stored for one representative per orbit of the nodes under
    // the reflections of the lattice (x -> nx - 1 - x per symmetric axis)
    int nreps = 0;       // orbit representatives (ns / 8 on a lattice symmetric in all three axes)
    int nrefl = 1;       // reflections of f kept on the device: 8, or 1 without a symmetric axis
    int *orbit = nullptr;  // [ns] rep slot << 3 | reflection bits (bit a: axis a mirrored)
    int *order = nullptr;  // [ns] the gain kernel's launch order (reflection-major)
    int64_t slots = 0;   // stored (not all-zero) tiles over the representatives
    int64_t slices = 0;  // 16-column slices with a nonzero entry issued per cell tile (all nodes)
    int64_t node_tiles = 0;  // stored tiles issued per cell tile (all nodes)
    int *node_off = nullptr;    // [nreps + 1] into list
    uint32_t *list = nullptr;   // stored tiles per representative, mask << 28 | n << 16 | k
    __nv_bfloat16 *gh = nullptr, *gl = nullptr;
    // f per reflection R, stacked R-major: [R][cell][matrix index] BF16 hi / lo
    // (f_cells rows per R) and [R][matrix index][cell] FP32 (epilogue)
    __nv_bfloat16 *fh = nullptr, *fl = nullptr;
    float *fp = nullptr;
    int f_cells = 0;
    // matrix order of the nodes: a 3-D Hilbert curve over the lattice, which
    // packs the nonzero entries of the G_i into fewer 256 x 64 tiles than
    // the compact (i, j, k) order; inv[R ns + m] is the node R(node at matrix
    // index m) (R = 0: the node itself), mnodes[m] its packed lattice
    // coordinates
    int *inv = nullptr;
    uint32_t *mnodes = nullptr;
    __nv_bfloat16 *bh = nullptr, *bl = nullptr;  // loss matrix [node][ns_k] BF16 hi / lo
    int *err = nullptr;
    int stall_next = 0;  // gd_ctx_inject_timeout: polls for the next tensor-core loss GEMM
    // stored tiles per tensor-memory accumulation of the gain (gd_cmatrix_set_chain)
    int chain = gd::kChainUnlimited;
    bool loss_only = false;  // the loss matrix alone (cmatrix_create_loss_only)
};

namespace gd {
int ensure_f(gd_cmatrix *h, int ncells);

// Axes along which the node set is symmetric (bit a: x_a -> n_a - 1 - x_a maps
// every in-sphere node to an in-sphere node).  The weights depend on |g|,
// |d| and whether s - i lies in the box, all invariant under these
// reflections, so G_R(i)[R a][R b] = G_i[a][b] exactly.
int lattice_reflections(const Context &c)
{
    const Dims &d = c.d;
    std::vector<char> in(d.nxyz, 0);
    for (int m = 0; m < d.n_pnt; m++) in[((size_t)c.ui[m] * d.ny + c.vi[m]) * d.nz + c.wi[m]] = 1;
    int axes = 0;
    const int n[3] = {d.nx, d.ny, d.nz};
    for (int a = 0; a < 3; a++) {
        if (n[a] & 1) continue;  // a middle plane would be its own mirror
        bool sym = true;
        for (int m = 0; sym && m < d.n_pnt; m++) {
            int x[3] = {c.ui[m], c.vi[m], c.wi[m]};
            x[a] = n[a] - 1 - x[a];
            sym = in[((size_t)x[0] * d.ny + x[1]) * d.nz + x[2]] != 0;
        }
        if (sym) axes |= 1 << a;
    }
    return axes;
}

// Index of (x, y, z) along a 3-D Hilbert curve through the 2^bits cube
// (Skilling's transpose algorithm: "Programming the Hilbert curve", AIP Conf.
// Proc. 707, 2004).
uint64_t hilbert_index(uint32_t x, uint32_t y, uint32_t z, int bits)
{
    uint32_t X[3] = {x, y, z};
    const uint32_t M = 1u << (bits - 1);
    for (uint32_t Q = M; Q > 1; Q >>= 1) {  // inverse undo excess work
        const uint32_t P = Q - 1;
        for (int i = 0; i < 3; i++) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    for (int i = 1; i < 3; i++) X[i] ^= X[i - 1];  // Gray encode
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    for (int i = 0; i < 3; i++) X[i] ^= t;
    uint64_t h = 0;  // interleave the transposed bits, most significant first
    for (int b = bits - 1; b >= 0; b--)
        for (int i = 0; i < 3; i++) h = (h << 1) | ((X[i] >> b) & 1u);
    return h;
}

// Side of the smallest power-of-two cube holding the lattice, as bits.
int hilbert_bits(const Dims &d)
{
    int bits = 1;
    while ((1 << bits) < std::max(d.nx, std::max(d.ny, d.nz))) bits++;
    return bits;
}

// The nodes' matrix order: sorted by their index along a Hilbert curve
// through the 2^bits cube, the lattice placed at (off, off, off) inside it.
// A run of consecutive matrix indices is then a compact block of nodes,
// which packs the orthogonality shells of each G_i ((a - i) . (b - i) near 0)
// into fewer 256 x 64 tiles than the compact (i, j, k) order (20^3, R = 4.8:
// 335-349 stored tiles per node, by offset, instead of 381).
void matrix_order(const Context &c, int off, std::vector<int> &inv, std::vector<uint32_t> &mnodes)
{
    const int ns = c.d.n_pnt;
    const int bits = hilbert_bits(c.d);
    std::vector<std::pair<uint64_t, int>> key(ns);
    for (int m = 0; m < ns; m++)
        key[m] = {hilbert_index((uint32_t)(c.ui[m] + off), (uint32_t)(c.vi[m] + off), (uint32_t)(c.wi[m] + off), bits),
                  m};
    std::sort(key.begin(), key.end());
    inv.resize(ns);
    mnodes.resize(ns);
    for (int m = 0; m < ns; m++) {
        const int node = key[m].second;
        inv[m] = node;
        mnodes[m] = (uint32_t)c.ui[node] | ((uint32_t)c.vi[node] << 10) | ((uint32_t)c.wi[node] << 20);
    }
}
}

namespace gd {

// The tensor-core loss alone (the loss matrix B in BF16 hi/lo, no collision
// matrices), for contexts whose gain runs on the pair kernel with its
// contraction on the tensor cores: nu = B f in one GEMM launch instead of the
// FP32 loss kernel (20^3, 4096 cells: ~0.3 against 22 ms).  The handle serves
// cmatrix_loss and the time-out records; it has no gain matrices.
int cmatrix_create_loss_only(gd_ctx *ctx, gd_cmatrix **out)
{
    *out = nullptr;
    Context &c = ctx->c;
    const Dims &d = c.d;
    int major = 0;
    GD_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c.device));
    if (major < 10) return set_error(GD_ERR_UNSUPPORTED, "the tensor-core loss needs tcgen05 (sm_100 family)");
    gd_cmatrix *h = new gd_cmatrix();
    h->ctx = ctx;
    h->mode = GD_CMATRIX_BF16X3;
    h->loss_only = true;
    h->ns = d.n_pnt;
    h->ns_k = (d.n_pnt + BK - 1) / BK * BK;
    std::vector<int> inv;
    std::vector<uint32_t> mnodes;
    matrix_order(c, 0, inv, mnodes);
    const size_t nb = (size_t)h->ns * h->ns_k;
    cudaError_t e = cudaMalloc(&h->inv, sizeof(int) * h->ns);
    if (e == cudaSuccess) e = cudaMalloc(&h->mnodes, sizeof(uint32_t) * h->ns);
    if (e == cudaSuccess) e = cudaMalloc(&h->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h->bh, nb * 2);
    if (e == cudaSuccess) e = cudaMalloc(&h->bl, nb * 2);
    if (e == cudaSuccess) e = cudaMemcpy(h->inv, inv.data(), sizeof(int) * h->ns, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(h->mnodes, mnodes.data(), sizeof(uint32_t) * h->ns, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->err, 0, sizeof(int));
    if (e == cudaSuccess) {
        assemble_b_kernel<<<(int)std::min<size_t>((nb + 255) / 256, (size_t)c.sm_count * 64), 256>>>(
            d, h->ns_k, c.d_nodes, h->mnodes, c.d_b, h->bh, h->bl);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        gd_cmatrix_destroy(h);
        return cuda_error(e, "tensor-core loss matrix");
    }
    *out = h;
    return GD_OK;
}

}  // namespace gd

extern "C" int gd_cmatrix_create(gd_ctx *ctx, int mode, gd_cmatrix **out)
{
    using namespace gd;
    if (!ctx || !out) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (mode != GD_CMATRIX_BF16 && mode != GD_CMATRIX_BF16X3) return set_error(GD_ERR_INVALID_ARG, "unknown mode");
    *out = nullptr;
    Context &c = ctx->c;
    const Dims &d = c.d;
    int major = 0;
    GD_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c.device));
    if (major < 10) return set_error(GD_ERR_UNSUPPORTED, "the collision-matrix path needs tcgen05 (sm_100 family)");
    gd_cmatrix *h = new gd_cmatrix();
    h->ctx = ctx;
    h->mode = mode;
    h->chain = mode == GD_CMATRIX_BF16X3 ? kDefaultChainBf16x3 : kChainUnlimited;
    h->ns = d.n_pnt;
    h->ns_k = (d.n_pnt + BK - 1) / BK * BK;
    const int num_n = (h->ns + BN - 1) / BN, num_k = h->ns_k / BK;
    std::vector<int2> tile_nk;
    for (int n = 0; n < num_n; n++)
        for (int k = 0; k < k_end(n, num_k); k++) tile_nk.push_back(make_int2(n, k));
    h->tiles = (int)tile_nk.size();
    // orbits of the nodes under the lattice's reflections: the representative
    // of node x mirrors every symmetric axis with x_a >= n_a / 2 (n_a is even,
    // so no node is its own mirror and every orbit has 2^axes nodes)
    const int axes = lattice_reflections(c);
    h->nrefl = axes ? 8 : 1;
    const int nax[3] = {d.nx, d.ny, d.nz};
    std::vector<int> box_map(d.nxyz, -1);
    for (int m = 0; m < h->ns; m++) box_map[((size_t)c.ui[m] * d.ny + c.vi[m]) * d.nz + c.wi[m]] = m;
    auto reflect = [&](int m, int R) {
        int x[3] = {c.ui[m], c.vi[m], c.wi[m]};
        for (int a = 0; a < 3; a++)
            if ((R >> a) & 1) x[a] = nax[a] - 1 - x[a];
        return box_map[((size_t)x[0] * d.ny + x[1]) * d.nz + x[2]];
    };
    std::vector<int> orbit(h->ns), rep_slot(h->ns, -1), order(h->ns);
    std::vector<uint32_t> rep_nodes;
    std::vector<int> orbit_size;
    for (int m = 0; m < h->ns; m++) {
        int R = 0;
        for (int a = 0; a < 3; a++) {
            const int xa = a == 0 ? c.ui[m] : a == 1 ? c.vi[m] : c.wi[m];
            if (((axes >> a) & 1) && 2 * xa >= nax[a]) R |= 1 << a;
        }
        const int r = reflect(m, R);
        if (rep_slot[r] < 0) {
            rep_slot[r] = (int)rep_nodes.size();
            rep_nodes.push_back((uint32_t)c.ui[r] | ((uint32_t)c.vi[r] << 10) | ((uint32_t)c.wi[r] << 20));
            orbit_size.push_back(0);
        }
        orbit[m] = rep_slot[r] << 3 | R;
        orbit_size[rep_slot[r]]++;
    }
    h->nreps = (int)rep_nodes.size();
    // launch order: reflection-major, so that the CTAs in flight read one
    // reflected copy of f (60 MB at 20^3 / 4096 cells, L2-resident) rather
    // than all eight; each representative's tiles are then read once per
    // reflection (orbit-major order ran 13 % slower: 233 against 207 ms)
    for (int m = 0; m < h->ns; m++) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return ((orbit[a] & 7) << 24 | orbit[a] >> 3) < ((orbit[b] & 7) << 24 | orbit[b] >> 3);
    });
    const size_t ntri = (size_t)h->nreps * h->tiles;  // triangle tiles over the representatives
    float *w = nullptr;
    int2 *d_tiles = nullptr;
    uint8_t *d_nz = nullptr;
    int *d_slot = nullptr;
    uint32_t *d_reps = nullptr;
    const size_t na = (size_t)d.hx * d.nx * d.hy * d.hz * d.nyz;
    const int64_t work = (int64_t)ntri * BN * (BK / 8);
    const int blocks = (int)std::min<int64_t>((work + 255) / 256, (int64_t)c.sm_count * 64);
    int rc = GD_OK;
    cudaError_t e = cudaMalloc(&h->inv, sizeof(int) * h->ns * h->nrefl);
    if (e == cudaSuccess) e = cudaMalloc(&h->mnodes, sizeof(uint32_t) * h->ns);
    if (e == cudaSuccess) e = cudaMalloc(&h->orbit, sizeof(int) * h->ns);
    if (e == cudaSuccess) e = cudaMalloc(&h->order, sizeof(int) * h->ns);
    if (e == cudaSuccess) e = cudaMalloc(&d_reps, sizeof(uint32_t) * h->nreps);
    if (e == cudaSuccess) e = cudaMemcpy(h->orbit, orbit.data(), sizeof(int) * h->ns, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->order, order.data(), sizeof(int) * h->ns, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_reps, rep_nodes.data(), sizeof(uint32_t) * h->nreps, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&h->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&w, na * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_tiles, sizeof(int2) * tile_nk.size());
    if (e == cudaSuccess) e = cudaMalloc(&d_nz, ntri * kSlices);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_tiles, tile_nk.data(), sizeof(int2) * tile_nk.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_error(e, "collision-matrix allocation");
    if (!rc) rc = launch_dense_tables(d, nullptr, w, nullptr);
    // the matrix order of the nodes: of the lattice's placements inside the
    // Hilbert cube, the one whose matrices store the fewest tiles, counted on
    // a sample of representatives (the same for every placement)
    std::vector<int> inv;
    std::vector<uint32_t> mnodes;
    if (!rc) {
        const int span = (1 << hilbert_bits(d)) - std::max(d.nx, std::max(d.ny, d.nz));
        const int nsample = std::min(h->nreps, 128);
        std::vector<uint32_t> sample(nsample);
        uint32_t *d_sample = nullptr;
        for (int k = 0; k < nsample; k++) sample[k] = rep_nodes[(size_t)k * h->nreps / nsample];
        e = cudaMalloc(&d_sample, sizeof(uint32_t) * nsample);
        if (e == cudaSuccess)
            e = cudaMemcpy(d_sample, sample.data(), sizeof(uint32_t) * nsample, cudaMemcpyHostToDevice);
        const size_t nsz = (size_t)nsample * h->tiles * kSlices;
        std::vector<uint8_t> snz(nsz);
        int64_t best = -1;
        for (int off = 0; e == cudaSuccess && off <= span; off++) {
            std::vector<int> inv_o;
            std::vector<uint32_t> mnodes_o;
            matrix_order(c, off, inv_o, mnodes_o);
            if (span > 0) {
                e = cudaMemcpy(h->mnodes, mnodes_o.data(), sizeof(uint32_t) * h->ns, cudaMemcpyHostToDevice);
                if (e == cudaSuccess) e = cudaMemset(d_nz, 0, nsz);
                if (e != cudaSuccess) break;
                const int sblocks =
                    (int)std::min<int64_t>(((int64_t)nsample * h->tiles * BN * (BK / 8) + 255) / 256,
                                           (int64_t)c.sm_count * 64);
                assemble_g_kernel<<<std::max(sblocks, 1), 256>>>(d, nsample, h->tiles, d_tiles, d_sample, h->mnodes, w,
                                                                 d_nz, nullptr, nullptr, nullptr);
                e = cudaGetLastError();
                if (e == cudaSuccess) e = cudaMemcpy(snz.data(), d_nz, nsz, cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) break;
            }
            int64_t stored = 0;  // MMA slices the sampled nodes' matrices issue
            for (uint8_t v : snz) stored += v;
            if (best < 0 || stored < best) {
                best = stored;
                inv.swap(inv_o);
                mnodes.swap(mnodes_o);
            }
        }
        cudaFree(d_sample);
        // inv per reflection R: the node R(inv[m]) at matrix index m
        std::vector<int> inv_r((size_t)h->ns * h->nrefl);
        for (int R = 0; R < h->nrefl; R++)
            for (int m = 0; m < h->ns; m++)
                inv_r[(size_t)R * h->ns + m] = (R & ~axes) ? inv[m] : reflect(inv[m], R);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->inv, inv_r.data(), sizeof(int) * inv_r.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->mnodes, mnodes.data(), sizeof(uint32_t) * h->ns, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(d_nz, 0, ntri * kSlices);
        if (e != cudaSuccess) rc = cuda_error(e, "collision-matrix node order");
    }
    // pass 1: which triangle tiles hold a nonzero entry
    std::vector<uint8_t> nz(ntri * kSlices);
    if (!rc) {
        assemble_g_kernel<<<blocks, 256>>>(d, h->nreps, h->tiles, d_tiles, d_reps, h->mnodes, w, d_nz, nullptr,
                                           nullptr, nullptr);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(nz.data(), d_nz, ntri * kSlices, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_error(e, "collision-matrix tile scan");
    }
    // per-representative lists of the stored tiles (n-major, k ascending) and
    // their slots; every node of an orbit issues its representative's slices
    std::vector<int> node_off(h->nreps + 1, 0), slot_of(ntri, -1);
    std::vector<uint32_t> list;
    if (!rc) {
        for (int i = 0; i < h->nreps; i++) {
            node_off[i] = (int)list.size();
            for (int t = 0; t < h->tiles; t++) {
                uint32_t mask = 0;
                for (int q = 0; q < kSlices; q++)
                    if (nz[((size_t)i * h->tiles + t) * kSlices + q]) mask |= 1u << q;
                if (mask) {
                    h->slices += (int64_t)__builtin_popcount(mask) * orbit_size[i];
                    h->node_tiles += orbit_size[i];
                    slot_of[(size_t)i * h->tiles + t] = (int)list.size();
                    list.push_back(mask << 28 | ((uint32_t)tile_nk[t].x << 16) | (uint32_t)tile_nk[t].y);
                }
            }
        }
        node_off[h->nreps] = (int)list.size();
        h->slots = (int64_t)list.size();
    }
    const size_t elems = (size_t)h->slots * BN * BK;
    if (!rc) {
        size_t free_b = 0, total_b = 0;
        e = cudaMemGetInfo(&free_b, &total_b);
        const size_t need = elems * 2 * (mode == GD_CMATRIX_BF16X3 ? 2 : 1);
        const size_t limit = memory_limit();
        if (e != cudaSuccess)
            rc = cuda_error(e, "cudaMemGetInfo");
        else if (limit && need > limit)
            rc = set_error(GD_ERR_OUT_OF_MEMORY, "collision matrices need " + std::to_string(need >> 20) +
                                                     " MiB; the library's memory limit is " +
                                                     std::to_string(limit >> 20) + " MiB");
        else if (need + ((size_t)1 << 30) > free_b)
            rc = set_error(GD_ERR_OUT_OF_MEMORY, "collision matrices need " + std::to_string(need >> 20) +
                                                     " MiB; free device memory is " + std::to_string(free_b >> 20) +
                                                     " MiB");
    }
    if (!rc) {
        e = cudaMalloc(&h->gh, std::max<size_t>(elems, 1) * 2);
        if (e == cudaSuccess && mode == GD_CMATRIX_BF16X3) e = cudaMalloc(&h->gl, std::max<size_t>(elems, 1) * 2);
        if (e == cudaSuccess) e = cudaMalloc(&h->node_off, sizeof(int) * node_off.size());
        if (e == cudaSuccess) e = cudaMalloc(&h->list, sizeof(uint32_t) * std::max<size_t>(list.size(), 1));
        if (e == cudaSuccess) e = cudaMalloc(&d_slot, sizeof(int) * ntri);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->node_off, node_off.data(), sizeof(int) * node_off.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && !list.empty())
            e = cudaMemcpy(h->list, list.data(), sizeof(uint32_t) * list.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_slot, slot_of.data(), sizeof(int) * ntri, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(e, "collision-matrix allocation");
    }
    // pass 2: the stored tiles, and the loss matrix
    if (!rc) {
        assemble_g_kernel<<<blocks, 256>>>(d, h->nreps, h->tiles, d_tiles, d_reps, h->mnodes, w, nullptr, d_slot,
                                           h->gh, h->gl);
        e = cudaGetLastError();
        const size_t nb = (size_t)h->ns * h->ns_k;
        if (e == cudaSuccess) e = cudaMalloc(&h->bh, nb * 2);
        if (e == cudaSuccess) e = cudaMalloc(&h->bl, nb * 2);
        if (e == cudaSuccess) {
            assemble_b_kernel<<<(int)std::min<size_t>((nb + 255) / 256, (size_t)c.sm_count * 64), 256>>>(
                d, h->ns_k, c.d_nodes, h->mnodes, c.d_b, h->bh, h->bl);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemset(h->err, 0, sizeof(int));
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = cuda_error(e, "collision-matrix assembly");
    }
    cudaFree(w);
    cudaFree(d_tiles);
    cudaFree(d_nz);
    cudaFree(d_slot);
    cudaFree(d_reps);
    if (rc) {
        cudaFree(h->bh);
        cudaFree(h->bl);
        cudaFree(h->gh);
        cudaFree(h->gl);
        cudaFree(h->node_off);
        cudaFree(h->list);
        cudaFree(h->err);
        cudaFree(h->inv);
        cudaFree(h->mnodes);
        cudaFree(h->orbit);
        cudaFree(h->order);
        delete h;
        return rc;
    }
    *out = h;
    return GD_OK;
}

extern "C" int gd_cmatrix_set_cluster(gd_cmatrix *h, int ctas)
{
    if (!h) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (ctas != 1 && ctas != 2) return gd::set_error(GD_ERR_INVALID_ARG, "cluster size must be 1 or 2");
    h->cluster = ctas;
    return GD_OK;
}

extern "C" int gd_cmatrix_set_chain(gd_cmatrix *h, int tiles)
{
    if (!h) return gd::set_error(GD_ERR_INVALID_ARG, "NULL argument");
    if (tiles < 0 || (tiles & 1)) return gd::set_error(GD_ERR_INVALID_ARG, "chain must be 0 or a positive even count");
    h->chain = tiles == 0 ? gd::kChainUnlimited : tiles;
    return GD_OK;
}

extern "C" int gd_cmatrix_destroy(gd_cmatrix *h)
{
    if (!h) return GD_OK;
    cudaFree(h->node_off);
    cudaFree(h->list);
    cudaFree(h->bh);
    cudaFree(h->bl);
    cudaFree(h->gh);
    cudaFree(h->gl);
    cudaFree(h->fh);
    cudaFree(h->fl);
    cudaFree(h->fp);
    cudaFree(h->err);
    cudaFree(h->inv);
    cudaFree(h->mnodes);
    cudaFree(h->orbit);
    cudaFree(h->order);
    delete h;
    return GD_OK;
}

namespace gd {

// The collision-matrix gain of one or more grids (at most kCmMaxGrids, one
// mode) in one launch: per grid the reflected copies of f, its tensor maps
// and parameters; the grids' nodes stacked along the grid's y extent.  Each
// grid's result equals its own launch's bit for bit (every CTA does the same
// work either way).
int launch_cmatrix(const CmJob *jobs, int njobs, cudaStream_t st)
{
    if (njobs < 1 || njobs > kCmMaxGrids) return set_error(GD_ERR_UNSUPPORTED, "collision-matrix launch: 1-4 grids");
    if (!jobs[0].cm) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    const bool split = jobs[0].cm->mode == GD_CMATRIX_BF16X3;
    // a CTA pair per MMA when every grid allows it (cluster 2, more than one cell tile)
    int cl = 2;
    int64_t total_nodes = 0;
    for (int j = 0; j < njobs; j++) {
        const CmJob &jb = jobs[j];
        if (!jb.cm || !jb.f || !jb.gain) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
        if (jb.ncells < 1 || jb.ld < jb.ncells) return set_error(GD_ERR_INVALID_ARG, "need 1 <= ncells <= ld");
        if (jb.cm->loss_only) return set_error(GD_ERR_UNSUPPORTED, "this handle holds no collision matrices");
        if ((jb.cm->mode == GD_CMATRIX_BF16X3) != split)
            return set_error(GD_ERR_UNSUPPORTED, "collision-matrix launch: one mode for every grid");
        for (int k = 0; k < j; k++)
            if (jobs[k].cm == jb.cm) return set_error(GD_ERR_UNSUPPORTED, "one launch serves distinct matrices");
        if (jb.cm->cluster != 2 || jb.ncells <= BM) cl = 1;
        total_nodes += jb.cm->ns;
    }
    if (total_nodes > 65535) return set_error(GD_ERR_UNSUPPORTED, "collision-matrix launch: too many nodes");
    EncodeTiled enc;
    int rc = get_encoder(&enc);
    if (rc) return rc;
    CmMaps maps{};
    CmLaunch L{};
    L.ngrids = njobs;
    int mx = 0;
    for (int j = 0; j < njobs; j++) {
        const CmJob &jb = jobs[j];
        gd_cmatrix *h = jb.cm;
        if ((rc = ensure_f(h, jb.ncells))) return rc;
        dim3 cb(32, 8), cg((h->ns_k + 31) / 32, (jb.ncells + 31) / 32, h->nrefl);
        convert_f_kernel<<<cg, cb, 0, st>>>(jb.f, h->ns, h->ns_k, jb.ncells, jb.ld, h->inv, h->fh,
                                            split ? h->fl : nullptr, h->fp, h->f_cells, h->f_cells);
        GD_CUDA(cudaGetLastError());
        // f per reflection: [R][cell][matrix index], f_cells rows per R (cells
        // past ncells read as zeros)
        const cuuint64_t fdims[3] = {(cuuint64_t)h->ns_k, (cuuint64_t)jb.ncells, (cuuint64_t)h->nrefl};
        const cuuint64_t fstr[2] = {(cuuint64_t)h->ns_k * 2, (cuuint64_t)h->f_cells * h->ns_k * 2};
        const cuuint32_t fbox[3] = {BK, BM, 1};
        const cuuint64_t gdims[3] = {(cuuint64_t)BK, (cuuint64_t)BN, (cuuint64_t)std::max<int64_t>(h->slots, 1)};
        const cuuint64_t gstr[2] = {(cuuint64_t)BK * 2, (cuuint64_t)BN * BK * 2};
        // with a CTA pair each CTA loads half of a G tile
        const cuuint32_t gbox[3] = {BK, (cuuint32_t)(BN / cl), 1};
        if ((rc = encode(enc, &maps.fh[j], h->fh, 3, fdims, fstr, fbox))) return rc;
        if ((rc = encode(enc, &maps.gh[j], h->gh, 3, gdims, gstr, gbox))) return rc;
        if (split) {
            if ((rc = encode(enc, &maps.fl[j], h->fl, 3, fdims, fstr, fbox))) return rc;
            if ((rc = encode(enc, &maps.gl[j], h->gl, 3, gdims, gstr, gbox))) return rc;
        } else {
            maps.fl[j] = maps.fh[j];
            maps.gl[j] = maps.gh[j];
        }
        // cell tiles padded to whole clusters: a tile past ncells reads zeros and stores nothing
        const int m_tiles = ((jb.ncells + BM - 1) / BM + cl - 1) / cl * cl;
        L.g[j] = CmParams{h->ns,     h->ns_k,     jb.ncells, jb.ld,    h->fp,    h->f_cells, jb.gain,
                          h->err,    h->node_off, h->list,   h->orbit, h->order, m_tiles,    h->chain};
        L.ystart[j + 1] = L.ystart[j] + h->ns;
        mx = std::max(mx, m_tiles);
    }
    // one CTA per (cell tile, node), cell tiles fastest so that the CTAs in flight
    // share a few nodes' matrix tiles in L2 (a persistent grid of one CTA per SM
    // taking the tiles round-robin measured 3-4 % slower at 20^3 / 4096 cells)
    dim3 grid((unsigned)mx, (unsigned)L.ystart[njobs]);
    const int npass = split ? 3 : 1;
    const size_t smem = (size_t)cm_stages(npass, cl) * cm_stage_bytes(npass, cl) + 1024;
    void (*kern)(const CmMaps, const CmLaunch) =
        njobs == 1 ? (split ? (cl == 2 ? cmatrix_gain_kernel<3, 2, false> : cmatrix_gain_kernel<3, 1, false>)
                            : (cl == 2 ? cmatrix_gain_kernel<1, 2, false> : cmatrix_gain_kernel<1, 1, false>))
                   : (split ? (cl == 2 ? cmatrix_gain_kernel<3, 2, true> : cmatrix_gain_kernel<3, 1, true>)
                            : (cl == 2 ? cmatrix_gain_kernel<1, 2, true> : cmatrix_gain_kernel<1, 1, true>));
    GD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GD_CUDA(cudaLaunchKernelEx(&cfg, kern, maps, L));
    GD_CUDA(cudaGetLastError());
    // the kernel records a pipeline time-out in each grid's err instead of
    // hanging; the call only enqueues work, and gd_cmatrix_check /
    // gd_ctx_check report it
    return GD_OK;
}

}  // namespace gd

extern "C" int gd_cmatrix_gain(gd_cmatrix *h, const float *f, int ncells, int ld, float *gain, gd_stream stream)
{
    using namespace gd;
    if (!h || !f || !gain) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    const CmJob job{h, f, ncells, ld, gain};
    return launch_cmatrix(&job, 1, (cudaStream_t)stream);
}

extern "C" int gd_ctx_inject_timeout(gd_ctx *ctx, int polls)
{
    using namespace gd;
    if (!ctx || polls < 1 || polls > (1 << 20))
        return set_error(GD_ERR_INVALID_ARG, "gd_ctx_inject_timeout: need a context and 1 <= polls <= 2^20");
    if (!ctx->c.cmatrix || ctx->c.gain_path == GD_GAIN_PAIR || ctx->c.gain_path == GD_GAIN_PAIR_TC)
        return set_error(GD_ERR_UNSUPPORTED, "gd_ctx_inject_timeout: the context's gain path has no tensor-core loss");
    ctx->c.cmatrix->stall_next = polls;
    return GD_OK;
}

namespace gd {
// Reads the collision-matrix time-out record on st (synchronising) and clears
// it; *timed_out receives whether it was set.
int cmatrix_take_timeout(gd_cmatrix *h, cudaStream_t st, bool *timed_out)
{
    int flag = 0;
    GD_CUDA(cudaMemcpyAsync(&flag, h->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GD_CUDA(cudaStreamSynchronize(st));
    *timed_out = flag != 0;
    if (flag) {
        GD_CUDA(cudaMemsetAsync(h->err, 0, sizeof(int), st));
        GD_CUDA(cudaStreamSynchronize(st));
    }
    return GD_OK;
}
}  // namespace gd

extern "C" int gd_cmatrix_check(gd_cmatrix *h, gd_stream stream)
{
    using namespace gd;
    if (!h) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    bool timed_out = false;
    const int rc = cmatrix_take_timeout(h, (cudaStream_t)stream, &timed_out);
    if (rc) return rc;
    if (timed_out) return set_error(GD_ERR_CUDA, "collision-matrix kernel: a pipeline wait timed out");
    return GD_OK;
}

namespace gd {
// BF16 hi and lo copies of f for up to ncells cells (grown on demand)
int ensure_f(gd_cmatrix *h, int ncells)
{
    if (h->f_cells >= ncells) return GD_OK;
    cudaFree(h->fh);
    cudaFree(h->fl);
    cudaFree(h->fp);
    h->fh = h->fl = nullptr;
    h->fp = nullptr;
    h->f_cells = 0;
    const size_t per = (size_t)ncells * h->ns_k * h->nrefl;  // one copy of f per reflection
    GD_CUDA(cudaMalloc(&h->fh, per * 2));
    GD_CUDA(cudaMalloc(&h->fl, per * 2));
    GD_CUDA(cudaMalloc(&h->fp, per * 4));
    h->f_cells = ncells;
    return GD_OK;
}

// nu = B f on the tensor cores, B_hi f_hi + B_hi f_lo + B_lo f_hi in one
// launch (the BF16 split keeps ~16 significant bits of both factors).
int cmatrix_loss(gd_cmatrix *h, const float *f, int ncells, int ld, float *nu, cudaStream_t st)
{
    if (!h->bh || (ld & 3) || (reinterpret_cast<uintptr_t>(nu) & 15)) return GD_ERR_UNSUPPORTED;
    int rc = ensure_f(h, ncells);
    if (rc) return rc;
    dim3 cb(32, 8), cg((h->ns_k + 31) / 32, (ncells + 31) / 32, 1);  // f itself (R = 0)
    convert_f_kernel<<<cg, cb, 0, st>>>(f, h->ns, h->ns_k, ncells, ld, h->inv, h->fh, h->fl, nullptr, 0, h->f_cells);
    GD_CUDA(cudaGetLastError());
    const int stall = h->stall_next;  // a pending time-out injection fires here, once
    h->stall_next = 0;
    // B_hi f_hi + B_hi f_lo + B_lo f_hi in one launch, at most kLossChunk
    // products per tensor-core FP32 accumulation, the chunks added in FP32
    return gemm_bf16x3_nt_f32(h->bh, h->bl, h->ns, h->fh, h->fl, ncells, h->ns_k, nu, ld, h->err, st, stall,
                              kLossChunk);
}

int64_t cmatrix_stored_tiles(const gd_cmatrix *cm) { return cm ? cm->slots : 0; }
int64_t cmatrix_issued_slices(const gd_cmatrix *cm) { return cm ? cm->slices : 0; }
int64_t cmatrix_node_tiles(const gd_cmatrix *cm) { return cm ? cm->node_tiles : 0; }

double cmatrix_bytes_bound(const Context &c, int mode)
{
    const int ns = c.d.n_pnt, ns_k = (ns + BK - 1) / BK * BK;
    const int num_n = (ns + BN - 1) / BN, num_k = ns_k / BK;
    int64_t tiles = 0;
    for (int n = 0; n < num_n; n++) tiles += k_end(n, num_k);
    // matrices of one representative per orbit of the reflections
    const int axes = lattice_reflections(c);
    const double reps = (double)ns / (double)(1 << __builtin_popcount(axes));
    return (double)tiles * reps * BN * BK * 2.0 * (mode == GD_CMATRIX_BF16X3 ? 2.0 : 1.0);
}

int encode_bf16_sw128(CUtensorMap *m, void *ptr, int rank, const uint64_t *dims, const uint64_t *strides,
                      const uint32_t *box)
{
    EncodeTiled fn = nullptr;
    int rc = get_encoder(&fn);
    if (rc) return rc;
    cuuint64_t dd[5], ss[4];
    cuuint32_t bb[5];
    for (int i = 0; i < rank; i++) {
        dd[i] = dims[i];
        bb[i] = box[i];
        if (i + 1 < rank) ss[i] = strides[i];
    }
    return encode(fn, m, ptr, rank, dd, ss, bb);
}

int run_loss_path(Context &c, const float *f, int ncells, int ld, float *nu, cudaStream_t st)
{
    if (c.gain_path != GD_GAIN_PAIR && c.cmatrix) {
        const int rc = cmatrix_loss(c.cmatrix, f, ncells, ld, nu, st);
        if (rc != GD_ERR_UNSUPPORTED) return rc;
    }
    return run_loss(c, f, ncells, ld, nu, st);
}

int run_gain_path(Context &c, const float *f, int ncells, int ld, float *gain, cudaStream_t st)
{
    if (c.gain_path == GD_GAIN_PAIR_TC && c.pair_tc) return run_pair_tc(c, f, ncells, ld, gain, st);
    if (c.gain_path == GD_GAIN_PAIR || !c.cmatrix) return run_gain(c, f, ncells, ld, gain, st);
    return gd_cmatrix_gain(c.cmatrix, f, ncells, ld, gain, st);
}
}  // namespace gd
