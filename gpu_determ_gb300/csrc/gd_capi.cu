// gd_capi.cu -- the extern "C" boundary (include/gpu_determ.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "gd_internal.h"

namespace gd {

namespace {
thread_local std::string g_last_error;
std::atomic<size_t> g_memory_limit{0};

int check_spec(const gd_grid_spec *s)
{
    if (!s) return set_error(GD_ERR_INVALID_ARG, "grid spec is NULL");
    const int n[3] = {s->nx, s->ny, s->nz};
    for (int a = 0; a < 3; a++) {
        if (n[a] < 2 || (n[a] & 1)) return set_error(GD_ERR_INVALID_ARG, "grid sizes must be even and >= 2");
        if (n[a] > 62) return set_error(GD_ERR_UNSUPPORTED, "grid sizes above 62 per axis are not supported");
        if (!(s->vmax[a] > s->vmin[a]) || !std::isfinite(s->vmin[a]) || !std::isfinite(s->vmax[a]))
            return set_error(GD_ERR_INVALID_ARG, "velocity bounds must be finite with vmin < vmax");
    }
    if (!std::isfinite(s->R)) return set_error(GD_ERR_INVALID_ARG, "sphere radius must be finite");
    return GD_OK;
}

int check_batch(const gd_ctx *ctx, const void *f, int ncells, int ld)
{
    if (!ctx) return set_error(GD_ERR_INVALID_ARG, "context is NULL");
    if (!f) return set_error(GD_ERR_INVALID_ARG, "distribution pointer is NULL");
    if (ncells < 1) return set_error(GD_ERR_INVALID_ARG, "ncells must be >= 1");
    if (ld < ncells) return set_error(GD_ERR_INVALID_ARG, "ld must be >= ncells");
    if ((int64_t)ld * ctx->c.d.n_pnt > ((int64_t)1 << 40))
        return set_error(GD_ERR_UNSUPPORTED, "batch too large");
    return GD_OK;
}

// Per-s work in linear s order (pair products, grouped weight-row visits,
// scatter) and the exact operation counts reported by gd_ctx_info.  Work
// depends on s only through D(s); each D stands for
// prod_a (D_a == n_a - 1 ? 1 : 2) pair sums s.
int build_s_schedule(Context &c, const std::vector<int> &gid_of_gbox)
{
    const Dims &d = c.d;
    std::vector<int64_t> work_by_D(d.nxyz, 0);
    std::vector<int> stamp(c.n_groups, -1);
    std::vector<int> item_off(d.nxyz + 1, 0);
    std::vector<int4> items;
    std::vector<uint32_t> members;
    std::vector<std::vector<uint32_t>> bucket(c.n_groups);
    std::vector<int> present;
    const uint32_t unit = (uint32_t)c.gain_cb * 4u;
    int64_t pairs = 0, terms = 0;
    for (int Dx = 0; Dx < d.nx; Dx++)
        for (int Dy = 0; Dy < d.ny; Dy++)
            for (int Dz = 0; Dz < d.nz; Dz++) {
                const int Did = (Dx * d.ny + Dy) * d.nz + Dz;
                const int mult = (Dx == d.nx - 1 ? 1 : 2) * (Dy == d.ny - 1 ? 1 : 2) * (Dz == d.nz - 1 ? 1 : 2);
                const int dx2 = Dx >> 1, dy2 = Dy >> 1, dz2 = Dz >> 1;
                int64_t nB = 0, visits = 0, used = 0;
                item_off[Did] = (int)items.size();
                present.clear();
                for (int gx = Dx & 1; gx <= Dx; gx += 2)
                    for (int gy = Dy & 1; gy <= Dy; gy += 2)
                        for (int gz = Dz & 1; gz <= Dz; gz += 2) {
                            nB++;
                            const int k = gid_of_gbox[(gx * d.ny + gy) * d.nz + gz];
                            bucket[k].push_back(half_pack(gx >> 1, gy >> 1, gz >> 1));
                            if (stamp[k] == Did) continue;
                            stamp[k] = Did;
                            present.push_back(k);
                            visits += c.h_grp_row_off[k + 1] - c.h_grp_row_off[k];
                            for (int e = c.h_grp_row_off[k]; e < c.h_grp_row_off[k + 1]; e++) {
                                if (c.h_grp_rows[e].w == 0.0f) continue;  // row padding
                                const int nc = (int)(c.h_grp_rows[e].off / unit);
                                const int z2 = nc % d.hz, y2 = (nc / d.hz) % d.hy, x2 = nc / (d.hz * d.hy);
                                used += x2 <= dx2 && y2 <= dy2 && z2 <= dz2;
                            }
                        }
                for (int k : present) {
                    const int mb = (int)members.size();
                    members.insert(members.end(), bucket[k].begin(), bucket[k].end());
                    items.push_back(make_int4(k, mb, (int)members.size(), 0));
                    bucket[k].clear();
                }
                work_by_D[Did] = 12 * nB + visits;
                pairs += nB * mult;
                terms += used * mult;
            }
    c.s_work_prefix.assign(d.ns + 1, 0);
    int64_t acc = 0;
    for (int sx = 0; sx < d.sx; sx++)
        for (int sy = 0; sy < d.sy; sy++)
            for (int sz = 0; sz < d.sz; sz++) {
                const int64_t sl = ((int64_t)sx * d.sy + sy) * d.sz + sz;
                const int Dx = std::min(sx, 2 * d.nx - 2 - sx), Dy = std::min(sy, 2 * d.ny - 2 - sy),
                          Dz = std::min(sz, 2 * d.nz - 2 - sz);
                c.s_work_prefix[sl] = acc;
                acc += work_by_D[(Dx * d.ny + Dy) * d.nz + Dz];
            }
    c.s_work_prefix[d.ns] = acc;
    c.pair_products = pairs;
    c.contraction_terms = terms;
    item_off[d.nxyz] = (int)items.size();
    GD_CUDA(cudaMalloc(&c.d_D_item_off, sizeof(int) * (d.nxyz + 1)));
    GD_CUDA(cudaMalloc(&c.d_D_items, sizeof(int4) * (items.size() + 1)));
    GD_CUDA(cudaMalloc(&c.d_D_members, sizeof(uint32_t) * (members.size() + 1)));
    GD_CUDA(cudaMemcpy(c.d_D_item_off, item_off.data(), sizeof(int) * (d.nxyz + 1), cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_D_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_D_members, members.data(), sizeof(uint32_t) * members.size(), cudaMemcpyHostToDevice));
    return GD_OK;
}

}  // namespace

size_t memory_limit() { return g_memory_limit.load(); }

// Group the per-|g| weight rows: rows with the same parity class and
// byte-identical (offset, weight) entries are one group.  Groups are ordered
// by parity class, then by first appearance in box order of g.
int build_row_groups(Context &c)
{
    const Dims &d = c.d;
    std::vector<int> off(d.nxyz + 1);
    std::vector<WEntry> rows(c.n_entries + 1);
    GD_CUDA(cudaMemcpy(off.data(), c.d_list_off, sizeof(int) * (d.nxyz + 1), cudaMemcpyDeviceToHost));
    GD_CUDA(cudaMemcpy(rows.data(), c.d_list, sizeof(WEntry) * c.n_entries, cudaMemcpyDeviceToHost));
    struct Group {
        int gbox0;  // first member (box index of g), row source
        std::vector<uint32_t> members;
    };
    std::vector<std::vector<Group>> by_class(8);
    std::vector<std::pair<int, int>> gref(d.nxyz);  // (class, index within class)
    std::vector<std::unordered_map<uint64_t, std::vector<int>>> index(8);
    auto same_row = [&](int a, int b) {
        const int la = off[a + 1] - off[a], lb = off[b + 1] - off[b];
        return la == lb && std::memcmp(&rows[off[a]], &rows[off[b]], sizeof(WEntry) * la) == 0;
    };
    for (int gx = 0; gx < d.nx; gx++)
        for (int gy = 0; gy < d.ny; gy++)
            for (int gz = 0; gz < d.nz; gz++) {
                const int gbox = (gx * d.ny + gy) * d.nz + gz;
                const int p = (gx & 1) | ((gy & 1) << 1) | ((gz & 1) << 2);
                uint64_t h = 1469598103934665603ull;  // FNV-1a over the row bytes
                const unsigned char *bytes = reinterpret_cast<const unsigned char *>(&rows[off[gbox]]);
                for (size_t t = 0; t < sizeof(WEntry) * (size_t)(off[gbox + 1] - off[gbox]); t++)
                    h = (h ^ bytes[t]) * 1099511628211ull;
                int found = -1;
                for (int k : index[p][h])
                    if (same_row(by_class[p][k].gbox0, gbox)) {
                        found = k;
                        break;
                    }
                if (found < 0) {
                    found = (int)by_class[p].size();
                    by_class[p].push_back(Group{gbox, {}});
                    index[p][h].push_back(found);
                }
                by_class[p][found].members.push_back(half_pack(gx >> 1, gy >> 1, gz >> 1));
                gref[gbox] = {p, found};
            }
    c.h_grp_row_off.assign(1, 0);
    c.h_grp_mem_off.assign(1, 0);
    c.h_grp_rows.clear();
    c.h_grp_members.clear();
    std::vector<int> base(9, 0);
    for (int p = 0; p < 8; p++) {
        base[p] = (int)c.h_grp_row_off.size() - 1;
        c.class_grp_off[p] = base[p];
        for (const Group &g : by_class[p]) {
            // rows are padded with zero-weight entries (offset 0) to a multiple
            // of 8, so the kernel reads them in aligned 16-byte pairs with no tail
            c.h_grp_rows.insert(c.h_grp_rows.end(), rows.begin() + off[g.gbox0], rows.begin() + off[g.gbox0 + 1]);
            while (c.h_grp_rows.size() % 8) c.h_grp_rows.push_back(WEntry{0u, 0.0f});
            c.h_grp_row_off.push_back((int)c.h_grp_rows.size());
            c.h_grp_members.insert(c.h_grp_members.end(), g.members.begin(), g.members.end());
            c.h_grp_mem_off.push_back((int)c.h_grp_members.size());
        }
    }
    c.n_groups = (int)c.h_grp_row_off.size() - 1;
    c.class_grp_off[8] = c.n_groups;
    c.n_grp_entries = (int64_t)c.h_grp_rows.size();
    std::vector<int> gid(d.nxyz);
    for (int gbox = 0; gbox < d.nxyz; gbox++) gid[gbox] = base[gref[gbox].first] + gref[gbox].second;
    GD_CUDA(cudaMalloc(&c.d_grp_row_off, sizeof(int) * (c.n_groups + 1)));
    GD_CUDA(cudaMalloc(&c.d_grp_rows, sizeof(WEntry) * (c.n_grp_entries + 1)));
    GD_CUDA(cudaMalloc(&c.d_grp_mem_off, sizeof(int) * (c.n_groups + 1)));
    GD_CUDA(cudaMalloc(&c.d_grp_members, sizeof(uint32_t) * c.h_grp_members.size()));
    GD_CUDA(cudaMemcpy(c.d_grp_row_off, c.h_grp_row_off.data(), sizeof(int) * (c.n_groups + 1), cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_grp_rows, c.h_grp_rows.data(), sizeof(WEntry) * c.n_grp_entries, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_grp_mem_off, c.h_grp_mem_off.data(), sizeof(int) * (c.n_groups + 1), cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_grp_members, c.h_grp_members.data(), sizeof(uint32_t) * c.h_grp_members.size(),
                       cudaMemcpyHostToDevice));
    return build_s_schedule(c, gid);
}

// gd_step's buffers: nu, gain (FP32) and Q (FP64) for every one the caller
// does not provide (NULL), context-owned and grown on demand (the growth
// synchronises st; no allocation per step once sized).
int step_buffers(Context &c, int ld, cudaStream_t st, float **nu, float **gain, double **q)
{
    if (*nu && *gain && *q) return GD_OK;
    const size_t n = (size_t)c.d.n_pnt * ld;
    const size_t need = n * (2 * sizeof(float) + sizeof(double));
    if (c.step_buf.bytes < need) {
        GD_CUDA(cudaStreamSynchronize(st));
        cudaFree(c.step_buf.ptr);
        c.step_buf.ptr = nullptr;
        c.step_buf.bytes = 0;
        GD_CUDA(cudaMalloc(&c.step_buf.ptr, need));
        c.step_buf.bytes = need;
    }
    unsigned char *p = static_cast<unsigned char *>(c.step_buf.ptr);
    if (!*q) *q = reinterpret_cast<double *>(p);
    if (!*nu) *nu = reinterpret_cast<float *>(p + n * sizeof(double));
    if (!*gain) *gain = reinterpret_cast<float *>(p + n * (sizeof(double) + sizeof(float)));
    return GD_OK;
}

int set_error(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

int cuda_error(cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return set_error(e == cudaErrorMemoryAllocation ? GD_ERR_OUT_OF_MEMORY : GD_ERR_CUDA, m);
}

int ensure_scratch(Context &c, size_t bytes)
{
    if (c.scratch.bytes >= bytes) return GD_OK;
    if (c.scratch.ptr) {
        GD_CUDA(cudaDeviceSynchronize());
        GD_CUDA(cudaFree(c.scratch.ptr));
        c.scratch.ptr = nullptr;
        c.scratch.bytes = 0;
    }
    const size_t grow = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&c.scratch.ptr, grow);
    if (e != cudaSuccess) {
        c.scratch.ptr = nullptr;
        return cuda_error(e, "scratch allocation");
    }
    c.scratch.bytes = grow;
    return GD_OK;
}

static void destroy_context(Context &c)
{
    gd_cmatrix_destroy(c.cmatrix);
    c.cmatrix = nullptr;
    pair_tc_free(c);
    cudaFree(c.d_cmap);
    cudaFree(c.d_nodes);
    cudaFree(c.d_b);
    cudaFree(c.d_phi);
    cudaFree(c.d_list_off);
    cudaFree(c.d_list);
    cudaFree(c.d_grp_row_off);
    cudaFree(c.d_grp_rows);
    cudaFree(c.d_grp_mem_off);
    cudaFree(c.d_grp_members);
    cudaFree(c.d_D_item_off);
    cudaFree(c.d_D_items);
    cudaFree(c.d_D_members);
    for (auto &kv : c.s_bounds_dev) cudaFree(kv.second);
    c.s_bounds_dev.clear();
    for (auto &kv : c.pt_units_dev) cudaFree(kv.second.first);
    c.pt_units_dev.clear();
    cudaFree(c.d_reduce);
    cudaFree(c.d_status);
    cudaFree(c.scratch.ptr);
    cudaFree(c.step_buf.ptr);
}

static int create_context(Context &c, const gd_grid_spec &spec, int device)
{
    c.spec = spec;
    c.device = device;
    Dims &d = c.d;
    d.nx = spec.nx;
    d.ny = spec.ny;
    d.nz = spec.nz;
    d.nyz = d.ny * d.nz;
    d.nxyz = d.nx * d.nyz;
    d.hx = d.nx / 2;
    d.hy = d.ny / 2;
    d.hz = d.nz / 2;
    d.nclass = d.hx * d.hy * d.hz;
    d.sx = 2 * d.nx - 1;
    d.sy = 2 * d.ny - 1;
    d.sz = 2 * d.nz - 1;
    d.ns = (int64_t)d.sx * d.sy * d.sz;
    const int np = grid_count(spec);
    if (np < 1) return set_error(GD_ERR_INVALID_ARG, "no lattice node lies inside the sphere");
    if (np > 32767) return set_error(GD_ERR_UNSUPPORTED, "more than 32767 in-sphere nodes");

    c.u.resize(d.nx);
    c.v.resize(d.ny);
    c.w.resize(d.nz);
    c.ui.resize(np);
    c.vi.resize(np);
    c.wi.resize(np);
    float steps[4];
    d.n_pnt = grid_fill(spec, c.u.data(), c.v.data(), c.w.data(), c.ui.data(), c.vi.data(), c.wi.data(), steps);
    d.du = steps[0];
    d.dv = steps[1];
    d.dw = steps[2];
    d.d3v = steps[3];

    c.cmap.assign(d.nxyz, -1);
    std::vector<int16_t> cmap16(d.nxyz, -1);
    std::vector<uint32_t> nodes(d.n_pnt);
    std::vector<double> phi((size_t)5 * d.n_pnt);
    for (int p = 0; p < d.n_pnt; p++) {
        const int bi = (c.ui[p] * d.ny + c.vi[p]) * d.nz + c.wi[p];
        c.cmap[bi] = p;
        cmap16[bi] = (int16_t)p;
        nodes[p] = (uint32_t)c.ui[p] | ((uint32_t)c.vi[p] << 10) | ((uint32_t)c.wi[p] << 20);
        const double xu = c.u[c.ui[p]], xv = c.v[c.vi[p]], xw = c.w[c.wi[p]];
        phi[p] = 1.0;
        phi[(size_t)d.n_pnt + p] = xu;
        phi[(size_t)2 * d.n_pnt + p] = xv;
        phi[(size_t)3 * d.n_pnt + p] = xw;
        phi[(size_t)4 * d.n_pnt + p] = xu * xu + xv * xv + xw * xw;
    }

    int ndev = 0;
    GD_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return set_error(GD_ERR_INVALID_ARG, "no such CUDA device");
    DeviceGuard guard(device);
    if (!guard.ok) return set_error(GD_ERR_CUDA, "cudaSetDevice failed");
    GD_CUDA(cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device));
    cudaStream_t st = nullptr;
    int rc = GD_OK;
    GD_CUDA(cudaMalloc(&c.d_cmap, sizeof(int16_t) * d.nxyz));
    GD_CUDA(cudaMalloc(&c.d_nodes, sizeof(uint32_t) * d.n_pnt));
    GD_CUDA(cudaMalloc(&c.d_phi, sizeof(double) * 5 * d.n_pnt));
    GD_CUDA(cudaMalloc(&c.d_b, sizeof(float) * d.nxyz));
    GD_CUDA(cudaMalloc(&c.d_reduce, sizeof(float) * kReduceFloats));
    GD_CUDA(cudaMalloc(&c.d_status, sizeof(unsigned int) * 2));
    {
        const unsigned int clear[2] = {0u, 0xffffffffu};
        GD_CUDA(cudaMemcpy(c.d_status, clear, sizeof(clear), cudaMemcpyHostToDevice));
    }
    GD_CUDA(cudaMemcpy(c.d_cmap, cmap16.data(), sizeof(int16_t) * d.nxyz, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_nodes, nodes.data(), sizeof(uint32_t) * d.n_pnt, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(c.d_phi, phi.data(), sizeof(double) * 5 * d.n_pnt, cudaMemcpyHostToDevice));

    if ((rc = gain_plan_cells(c))) return rc;
    // analytic weights: dense FP64-built table (transient), compacted to rows
    const size_t na = (size_t)d.hx * d.nx * d.hy * d.hz * d.nyz;
    float *a_dense = nullptr;
    GD_CUDA(cudaMalloc(&a_dense, sizeof(float) * na));
    rc = launch_dense_tables(d, c.d_b, a_dense, st);
    if (!rc) rc = build_weight_rows(c, a_dense, st);
    cudaFree(a_dense);
    if (rc) return rc;
    if ((rc = build_row_groups(c))) return rc;
    // scatter updates: distinct sign patterns of g whose target lies in the sphere
    int64_t sc = 0;
    for (int sx = 0; sx < d.sx; sx++)
        for (int sy = 0; sy < d.sy; sy++)
            for (int sz = 0; sz < d.sz; sz++) {
                const int Dx = std::min(sx, 2 * d.nx - 2 - sx), Dy = std::min(sy, 2 * d.ny - 2 - sy),
                          Dz = std::min(sz, 2 * d.nz - 2 - sz);
                for (int gx = sx & 1; gx <= Dx; gx += 2)
                    for (int gy = sy & 1; gy <= Dy; gy += 2)
                        for (int gz = sz & 1; gz <= Dz; gz += 2)
                            for (int sg = 0; sg < 8; sg++) {
                                if (((sg & 1) && gx == 0) || ((sg & 2) && gy == 0) || ((sg & 4) && gz == 0)) continue;
                                const int ix = (sx + ((sg & 1) ? -gx : gx)) >> 1;
                                const int iy = (sy + ((sg & 2) ? -gy : gy)) >> 1;
                                const int iz = (sz + ((sg & 4) ? -gz : gz)) >> 1;
                                sc += c.cmap[(ix * d.ny + iy) * d.nz + iz] >= 0;
                            }
            }
    c.scatter_terms = sc;
    GD_CUDA(cudaDeviceSynchronize());
    return GD_OK;
}

}  // namespace gd

using gd::set_error;

// error message setter for the C++ host layer (gd_api.cpp)
int gd_set_error_message(int code, const std::string &msg) { return gd::set_error(code, msg); }

extern "C" {

int gd_version(void) { return 100; }

const char *gd_last_error(void) { return gd::g_last_error.c_str(); }

int gd_grid_count(const gd_grid_spec *spec, int *n_pnt)
{
    int rc = gd::check_spec(spec);
    if (rc) return rc;
    if (!n_pnt) return set_error(GD_ERR_INVALID_ARG, "n_pnt is NULL");
    *n_pnt = gd::grid_count(*spec);
    return GD_OK;
}

int gd_grid_fill(const gd_grid_spec *spec, float *u, float *v, float *w, int *ui, int *vi, int *wi,
                 float *steps)
{
    int rc = gd::check_spec(spec);
    if (rc) return rc;
    gd::grid_fill(*spec, u, v, w, ui, vi, wi, steps);
    return GD_OK;
}

int gd_ctx_create(const gd_grid_spec *spec, int device, gd_ctx **out)
{
    if (!out) return set_error(GD_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int rc = gd::check_spec(spec);
    if (rc) return rc;
    gd_ctx *ctx = new (std::nothrow) gd_ctx();
    if (!ctx) return set_error(GD_ERR_OUT_OF_MEMORY, "host allocation failed");
    rc = gd::create_context(ctx->c, *spec, device);
    if (rc) {
        gd::DeviceGuard g(device);
        gd::destroy_context(ctx->c);
        delete ctx;
        return rc;
    }
    *out = ctx;
    return GD_OK;
}

int gd_ctx_destroy(gd_ctx *ctx)
{
    if (!ctx) return GD_OK;
    {
        gd::DeviceGuard g(ctx->c.device);
        gd::destroy_context(ctx->c);
    }
    delete ctx;
    return GD_OK;
}

int gd_ctx_set_gain_path(gd_ctx *ctx, int path)
{
    if (!ctx) return set_error(GD_ERR_INVALID_ARG, "context is NULL");
    if (path != GD_GAIN_PAIR && path != GD_GAIN_CMATRIX_BF16 && path != GD_GAIN_CMATRIX_BF16X3 &&
        path != GD_GAIN_PAIR_TC)
        return set_error(GD_ERR_INVALID_ARG, "unknown gain path");
    gd::Context &c = ctx->c;
    if (path == c.gain_path) return GD_OK;
    gd::DeviceGuard g(c.device);
    gd_cmatrix_destroy(c.cmatrix);
    c.cmatrix = nullptr;
    gd::pair_tc_free(c);
    c.gain_path = GD_GAIN_PAIR;
    if (path == GD_GAIN_PAIR_TC) {
        int rc = gd::pair_tc_build(c);
        // the loss on the tensor cores too (the loss matrix alone)
        if (!rc && (rc = gd::cmatrix_create_loss_only(ctx, &c.cmatrix))) gd::pair_tc_free(c);
        if (rc) return rc;
    } else if (path != GD_GAIN_PAIR) {
        const int mode = path == GD_GAIN_CMATRIX_BF16 ? GD_CMATRIX_BF16 : GD_CMATRIX_BF16X3;
        int rc = gd_cmatrix_create(ctx, mode, &c.cmatrix);
        if (rc) return rc;
    }
    c.gain_path = path;
    return GD_OK;
}

int gd_ctx_info(const gd_ctx *ctx, gd_info *out)
{
    if (!ctx || !out) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    const gd::Dims &d = ctx->c.d;
    out->nx = d.nx;
    out->ny = d.ny;
    out->nz = d.nz;
    out->n_pnt = d.n_pnt;
    out->du = d.du;
    out->dv = d.dv;
    out->dw = d.dw;
    out->d3v = d.d3v;
    out->nonzero_weights = ctx->c.n_entries;
    out->table_a_elems = (int64_t)d.hx * d.nx * d.hy * d.hz * d.nyz;
    out->pair_products = ctx->c.pair_products;
    out->contraction_terms = ctx->c.contraction_terms;
    out->scatter_terms = ctx->c.scatter_terms;
    out->cmatrix_tiles = gd::cmatrix_stored_tiles(ctx->c.cmatrix);
    out->cmatrix_slices = gd::cmatrix_issued_slices(ctx->c.cmatrix);
    out->cmatrix_node_tiles = gd::cmatrix_node_tiles(ctx->c.cmatrix);
    return GD_OK;
}

int gd_pair_tables(gd_ctx *ctx, gd_pair_table_sizes *sizes, int *grp_row_off, int *entry_class, float *entry_w,
                   int *item_off, int *items, uint32_t *members)
{
    if (!ctx || !sizes) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    gd::Context &c = ctx->c;
    gd::DeviceGuard g(c.device);
    const gd::Dims &d = c.d;
    std::vector<int> ioff(d.nxyz + 1);
    GD_CUDA(cudaMemcpy(ioff.data(), c.d_D_item_off, sizeof(int) * (d.nxyz + 1), cudaMemcpyDeviceToHost));
    const int64_t n_items = ioff[d.nxyz];
    std::vector<int4> it(n_items + 1);
    GD_CUDA(cudaMemcpy(it.data(), c.d_D_items, sizeof(int4) * n_items, cudaMemcpyDeviceToHost));
    const int64_t n_members = n_items > 0 ? it[n_items - 1].z : 0;
    sizes->n_groups = c.n_groups;
    sizes->nclass = d.nclass;
    sizes->n_entries = c.n_grp_entries;
    sizes->n_items = n_items;
    sizes->n_members = n_members;
    if (grp_row_off) std::memcpy(grp_row_off, c.h_grp_row_off.data(), sizeof(int) * (c.n_groups + 1));
    const uint32_t unit = (uint32_t)c.gain_cb * 4u;  // WEntry.off = class index x cells per block x 4
    for (int64_t e = 0; e < c.n_grp_entries; e++) {
        if (entry_class) entry_class[e] = (int)(c.h_grp_rows[e].off / unit);
        if (entry_w) entry_w[e] = c.h_grp_rows[e].w;
    }
    if (item_off) std::memcpy(item_off, ioff.data(), sizeof(int) * (d.nxyz + 1));
    if (items)
        for (int64_t t = 0; t < n_items; t++) {
            items[3 * t] = it[t].x;
            items[3 * t + 1] = it[t].y;
            items[3 * t + 2] = it[t].z;
        }
    if (members && n_members > 0)
        GD_CUDA(cudaMemcpy(members, c.d_D_members, sizeof(uint32_t) * n_members, cudaMemcpyDeviceToHost));
    return GD_OK;
}

int gd_export_tables(gd_ctx *ctx, float *b, float *a, gd_stream stream)
{
    if (!ctx) return set_error(GD_ERR_INVALID_ARG, "context is NULL");
    gd::DeviceGuard g(ctx->c.device);
    return gd::launch_dense_tables(ctx->c.d, b, a, (cudaStream_t)stream);
}

int gd_correction_basis(gd_ctx *ctx, float *basis, gd_stream stream)
{
    if (!ctx || !basis) return set_error(GD_ERR_INVALID_ARG, "NULL argument");
    gd::DeviceGuard g(ctx->c.device);
    return gd::run_basis(ctx->c, basis, (cudaStream_t)stream);
}

int gd_collision(gd_ctx *ctx, const float *f, int ncells, int ld, float *nu, float *gain, gd_stream stream)
{
    int rc = gd::check_batch(ctx, f, ncells, ld);
    if (rc) return rc;
    gd::DeviceGuard g(ctx->c.device);
    cudaStream_t st = (cudaStream_t)stream;
    if (nu && (rc = gd::run_loss_path(ctx->c, f, ncells, ld, nu, st))) return rc;
    if (gain && (rc = gd::run_gain_path(ctx->c, f, ncells, ld, gain, st))) return rc;
    return GD_OK;
}

int gd_project(gd_ctx *ctx, const float *f, const float *nu, const float *gain, int ncells, int ld,
               float *nu_corr, double *q, double *x, gd_stream stream)
{
    int rc = gd::check_batch(ctx, f, ncells, ld);
    if (rc) return rc;
    if (!nu || !gain) return set_error(GD_ERR_INVALID_ARG, "nu and gain are required");
    gd::DeviceGuard g(ctx->c.device);
    return gd::run_project(ctx->c, f, nu, gain, ncells, ld, nu_corr, q, x, 0, 0.f, nullptr, nullptr,
                           (cudaStream_t)stream);
}

int gd_relax(gd_ctx *ctx, float *f, const float *nu_corr, const float *gain, int ncells, int ld, int mode,
             float param, float *time_dev, float *dt_dev, gd_stream stream)
{
    int rc = gd::check_batch(ctx, f, ncells, ld);
    if (rc) return rc;
    if (!nu_corr || !gain) return set_error(GD_ERR_INVALID_ARG, "nu and gain are required");
    if (mode != GD_DT_COURANT && mode != GD_DT_FIXED) return set_error(GD_ERR_INVALID_ARG, "unknown dt mode");
    if (!(param > 0.f) || !std::isfinite(param)) return set_error(GD_ERR_INVALID_ARG, "dt parameter must be > 0");
    gd::DeviceGuard g(ctx->c.device);
    return gd::run_relax(ctx->c, f, nu_corr, gain, ncells, ld, mode, param, time_dev, dt_dev,
                         (cudaStream_t)stream);
}

int gd_step(gd_ctx *ctx, float *f, int ncells, int ld, int mode, float param, float *nu, float *gain,
            double *q, double *m5, float *time_dev, float *dt_dev, gd_stream stream)
{
    int rc = gd::check_batch(ctx, f, ncells, ld);
    if (rc) return rc;
    if (mode != GD_DT_COURANT && mode != GD_DT_FIXED) return set_error(GD_ERR_INVALID_ARG, "unknown dt mode");
    if (!(param > 0.f) || !std::isfinite(param)) return set_error(GD_ERR_INVALID_ARG, "dt parameter must be > 0");
    gd::DeviceGuard g(ctx->c.device);
    gd::Context &c = ctx->c;
    cudaStream_t st = (cudaStream_t)stream;
    float *nu_b = nu, *gain_b = gain;
    double *q_b = q;
    if ((rc = gd::step_buffers(c, ld, st, &nu_b, &gain_b, &q_b))) return rc;
    rc = gd::run_loss_path(c, f, ncells, ld, nu_b, st);
    if (!rc) rc = gd::run_gain_path(c, f, ncells, ld, gain_b, st);
    if (!rc) rc = gd::run_project(c, f, nu_b, gain_b, ncells, ld, nu_b, q_b, nullptr, 0, 0.f, nullptr, m5, st);
    if (!rc) rc = gd::run_relax_q(c, f, nu_b, gain_b, q_b, ncells, ld, mode, param, time_dev, dt_dev, st);
    return rc;
}

int gd_set_memory_limit(size_t bytes)
{
    gd::g_memory_limit.store(bytes);
    return GD_OK;
}

int gd_ctx_check(gd_ctx *ctx, gd_stream stream)
{
    if (!ctx) return set_error(GD_ERR_INVALID_ARG, "context is NULL");
    gd::DeviceGuard g(ctx->c.device);
    gd::Context &c = ctx->c;
    cudaStream_t st = (cudaStream_t)stream;
    // read every record first (each read clears its own), then report: a
    // numeric record and a time-out of the same step come out in one message
    unsigned int h[2] = {0u, 0u};
    GD_CUDA(cudaMemcpyAsync(h, c.d_status, sizeof(h), cudaMemcpyDeviceToHost, st));
    GD_CUDA(cudaStreamSynchronize(st));
    if (h[0]) {
        static const unsigned int clear[2] = {0u, 0xffffffffu};
        GD_CUDA(cudaMemcpyAsync(c.d_status, clear, sizeof(clear), cudaMemcpyHostToDevice, st));
        GD_CUDA(cudaStreamSynchronize(st));
    }
    bool cm_timeout = false, pt_timeout = false;
    if (c.cmatrix) {
        const int rc = gd::cmatrix_take_timeout(c.cmatrix, st, &cm_timeout);
        if (rc) return rc;
    }
    if (c.pair_tc) {
        const int rc = gd::pair_tc_take_timeout(c, st, &pt_timeout);
        if (rc) return rc;
    }
    std::string msg;
    if (cm_timeout) msg += "collision-matrix kernel: a pipeline wait timed out";
    if (pt_timeout) msg += std::string(msg.empty() ? "" : "; ") + "pair tensor-core gain kernel: a pipeline wait timed out";
    if (h[0])
        msg += std::string(msg.empty() ? "" : "; ") +
               (h[0] & 1u ? "non-finite distribution, frequency or gain" : "singular conservation system") +
               " in the projection (first affected cell " + std::to_string(h[1]) + ")";
    if (cm_timeout || pt_timeout) return set_error(GD_ERR_CUDA, msg);
    if (h[0]) return set_error(GD_ERR_SINGULAR, msg);
    return GD_OK;
}

int gd_moments(gd_ctx *ctx, const float *f, int ncells, int ld, double *m5, gd_stream stream)
{
    int rc = gd::check_batch(ctx, f, ncells, ld);
    if (rc) return rc;
    if (!m5) return set_error(GD_ERR_INVALID_ARG, "m5 is NULL");
    gd::DeviceGuard g(ctx->c.device);
    return gd::run_moments(ctx->c, f, ncells, ld, m5, (cudaStream_t)stream);
}

}  // extern "C"
