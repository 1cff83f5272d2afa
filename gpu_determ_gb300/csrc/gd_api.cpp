// gd_api.cpp -- the reference's C++ host interface (include/gpu_determ_api.hpp)
// implemented over the C ABI.
//
// Reference: options.hpp/options.cu (Options, load_options, print_options),
// velocity_grid.hpp/.cu (VelocityGrid, DeviceVelocityGrid), compute_matrix.h
// (init_matrices), velocity.h (init_correction_array), collision_integral.h
// (evolve_colisions, relax_f).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu_determ_api.hpp"

int gd_set_error_message(int code, const std::string &msg);

namespace {

std::mutex g_mu;
gd_ctx *g_current = nullptr;  // context of the most recent DeviceVelocityGrid

void report(const char *what, int rc)
{
    std::printf("%s: %s\n", what, rc ? gd_last_error() : "no error");
}

void report_cuda(const char *what, cudaError_t e)
{
    std::printf("%s: %s\n", what, cudaGetErrorString(e));
}

// Key/value line parsing of options.cu:12-32: trim, skip empty lines and '#'
// comments, split at the first '='.
void trim(std::string &s)
{
    const char *ws = " \t\n\r\f\v";
    s.erase(0, s.find_first_not_of(ws));
    const auto last = s.find_last_not_of(ws);
    if (last != std::string::npos) s.erase(last + 1);
}

bool split_line(std::string line, std::string &key, std::string &value)
{
    trim(line);
    const auto eq = line.find('=');
    if (line.empty() || line[0] == '#' || eq == std::string::npos) return false;
    key = line.substr(0, eq);
    value = line.substr(eq + 1);
    trim(key);
    trim(value);
    return true;
}

template <typename F>
void for_each_option(const std::string &fname, F &&fn)
{
    std::ifstream f(fname.c_str());
    if (!f) throw std::runtime_error("Can't open " + fname);
    std::string line, key, value;
    while (std::getline(f, line))
        if (split_line(line, key, value)) fn(key, value);
}

void parse_vec3(const std::string &v, float out[3])
{
    std::istringstream is(v);
    float a = 0, b = 0, c = 0;
    is >> a;
    if (is >> b >> c) {
        out[0] = a;
        out[1] = b;
        out[2] = c;
    } else {
        out[0] = out[1] = out[2] = a;
    }
}

gd_grid_spec spec_of(const VelocityGridBase &g, float R)
{
    gd_grid_spec s{};
    s.nx = g.n_u;
    s.ny = g.n_v;
    s.nz = g.n_w;
    s.vmin[0] = g.min_u;
    s.vmin[1] = g.min_v;
    s.vmin[2] = g.min_w;
    s.vmax[0] = g.max_u;
    s.vmax[1] = g.max_v;
    s.vmax[2] = g.max_w;
    s.R = R;
    return s;
}

// Compact scratch for grids whose sphere cuts the box.
struct CompactScratch {
    float *f = nullptr, *nu = nullptr, *gain = nullptr;
    size_t elems = 0;
    bool ensure(size_t n)
    {
        if (n <= elems) return true;
        cudaFree(f);
        cudaFree(nu);
        cudaFree(gain);
        f = nu = gain = nullptr;
        elems = 0;
        if (cudaMalloc(&f, n * sizeof(float)) != cudaSuccess || cudaMalloc(&nu, n * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&gain, n * sizeof(float)) != cudaSuccess)
            return false;
        elems = n;
        return true;
    }
};
CompactScratch g_scratch;

uint64_t fnv1a(const void *data, size_t n)
{
    const unsigned char *p = static_cast<const unsigned char *>(data);
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

struct CheckpointHeader {
    char magic[8];
    int32_t version;
    gd_grid_spec spec;
    int32_t nxyz, npx;
    int64_t step;
    double time;
    uint64_t payload_hash;
};

}  // namespace

// options.cu:34-53
void load_options(Options &opts, const std::string &fname)
{
    for_each_option(fname, [&](const std::string &key, const std::string &value) {
        if (key == "nx") opts.nx = std::stoi(value);
        else if (key == "ny") opts.ny = std::stoi(value);
        else if (key == "nz") opts.nz = std::stoi(value);
        else if (key == "npx") opts.npx = std::stoi(value);
    });
    opts.nyz = opts.ny * opts.nz;
    opts.nxyz = opts.nx * opts.nyz;
}

// options.cu:55-65
void print_options(const Options &opts)
{
    std::cout << "N_X: \t" << opts.nx << std::endl;
    std::cout << "N_Y: \t" << opts.ny << std::endl;
    std::cout << "N_Z: \t" << opts.nz << std::endl;
    std::cout << "N_YZ: \t" << opts.nyz << std::endl;
    std::cout << "N_XYZ: \t" << opts.nxyz << std::endl;
    std::cout << "N_PX: \t" << opts.npx << std::endl;
}

void load_run_options(RunOptions &ro, const std::string &fname)
{
    load_options(ro.base, fname);
    for_each_option(fname, [&](const std::string &key, const std::string &value) {
        if (key == "vmin") parse_vec3(value, ro.vmin);
        else if (key == "vmax") parse_vec3(value, ro.vmax);
        else if (key == "R") ro.R = std::stof(value);
        else if (key == "steps") ro.steps = std::stoi(value);
        else if (key == "dt_mode") ro.dt_mode = (value == "fixed") ? GD_DT_FIXED : GD_DT_COURANT;
        else if (key == "courant") ro.courant = std::stof(value);
        else if (key == "dt") ro.dt = std::stof(value);
        else if (key == "out_step") ro.out_step = std::stoi(value);
        else if (key == "init") ro.init = value;
        else if (key == "seed") ro.seed = std::stoi(value);
        else if (key == "results") ro.results = value;
        else if (key == "checkpoint") ro.checkpoint = value;
        else if (key == "resume") ro.resume = value;
        else if (key == "rows") ro.literal_rows = (value != "cells");
        else if (key == "correction") ro.correction = (value != "none");
        else if (key == "gain") {
            if (value != "pair" && value != "pair_tc" && value != "bf16" && value != "bf16x3")
                throw std::runtime_error("gain must be pair, pair_tc, bf16 or bf16x3, not '" + value + "'");
            ro.gain = value;
        }
    });
}

// velocity_grid.cu:73-126 via the library's host grid
VelocityGrid::VelocityGrid(Vector3i n_points, Vector3f v_min, Vector3f v_max, float r)
{
    init(n_points, v_min, v_max, r);
}

void VelocityGrid::init(Vector3i n_points, Vector3f v_min, Vector3f v_max, float R)
{
    if (u) {
        delete[] u;
        delete[] v;
        delete[] w;
        delete[] u_index;
        delete[] v_index;
        delete[] w_index;
    }
    gd_grid_spec s{};
    s.nx = n_points.x;
    s.ny = n_points.y;
    s.nz = n_points.z;
    s.vmin[0] = v_min.x;
    s.vmin[1] = v_min.y;
    s.vmin[2] = v_min.z;
    s.vmax[0] = v_max.x;
    s.vmax[1] = v_max.y;
    s.vmax[2] = v_max.z;
    s.R = R;
    R_ = R;
    int np = 0;
    if (gd_grid_count(&s, &np)) throw std::runtime_error(gd_last_error());
    n_pnt = np;
    n_u = s.nx;
    n_v = s.ny;
    n_w = s.nz;
    n_uvw = s.nx * s.ny * s.nz;
    u = new float[n_u];
    v = new float[n_v];
    w = new float[n_w];
    u_index = new int[n_pnt];
    v_index = new int[n_pnt];
    w_index = new int[n_pnt];
    float steps[4];
    gd_grid_fill(&s, u, v, w, u_index, v_index, w_index, steps);
    min_u = v_min.x;
    min_v = v_min.y;
    min_w = v_min.z;
    max_u = v_max.x;
    max_v = v_max.y;
    max_w = v_max.z;
    d_u = steps[0];
    d_v = steps[1];
    d_w = steps[2];
    d3v = steps[3];
}

VelocityGrid::~VelocityGrid()
{
    if (device_) {
        device_->free();
        delete device_;
    }
    if (!u) return;
    delete[] u;
    delete[] v;
    delete[] w;
    delete[] u_index;
    delete[] v_index;
    delete[] w_index;
}

DeviceVelocityGrid &VelocityGrid::device() const
{
    if (!device_) device_ = new DeviceVelocityGrid(*this);
    return *device_;
}

// velocity_grid.cu:27-48: device copies of the grid arrays, plus the context
DeviceVelocityGrid::DeviceVelocityGrid(const VelocityGrid &g) : VelocityGridBase(g)
{
    u = v = w = nullptr;
    u_index = v_index = w_index = nullptr;
    cudaMalloc((void **)&u_index, n_pnt * sizeof(int));
    cudaMemcpy(u_index, g.u_index, n_pnt * sizeof(int), cudaMemcpyHostToDevice);
    cudaMalloc((void **)&v_index, n_pnt * sizeof(int));
    cudaMemcpy(v_index, g.v_index, n_pnt * sizeof(int), cudaMemcpyHostToDevice);
    cudaMalloc((void **)&w_index, n_pnt * sizeof(int));
    cudaMemcpy(w_index, g.w_index, n_pnt * sizeof(int), cudaMemcpyHostToDevice);
    cudaMalloc((void **)&u, n_u * sizeof(float));
    cudaMemcpy(u, g.u, n_u * sizeof(float), cudaMemcpyHostToDevice);
    cudaMalloc((void **)&v, n_v * sizeof(float));
    cudaMemcpy(v, g.v, n_v * sizeof(float), cudaMemcpyHostToDevice);
    cudaMalloc((void **)&w, n_w * sizeof(float));
    cudaMemcpy(w, g.w, n_w * sizeof(float), cudaMemcpyHostToDevice);
    int dev = 0;
    cudaGetDevice(&dev);
    const gd_grid_spec s = spec_of(g, g.radius());
    const int rc = gd_ctx_create(&s, dev, &ctx_);
    if (rc) report("DEVICE VELOCITY GRID", rc);
    std::lock_guard<std::mutex> lk(g_mu);
    g_current = ctx_;
}

void DeviceVelocityGrid::free()
{
    cudaFree(u);
    cudaFree(v);
    cudaFree(w);
    cudaFree(u_index);
    cudaFree(v_index);
    cudaFree(w_index);
    u = v = w = nullptr;
    u_index = v_index = w_index = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_current == ctx_) g_current = nullptr;
    }
    gd_ctx_destroy(ctx_);
    ctx_ = nullptr;
}

// compute_matrix.cu:564-600
void init_matrices(const DeviceVelocityGrid &vgrid, float **b, float **a, const Options &opts)
{
    gd_info inf{};
    if (!vgrid.context() || gd_ctx_info(vgrid.context(), &inf)) {
        report("INIT MATRICES", GD_ERR_INVALID_ARG);
        return;
    }
    cudaError_t e = cudaMalloc((void **)a, sizeof(float) * (size_t)inf.table_a_elems);
    if (e != cudaSuccess) return report_cuda("ALLOCATION FOR INVERSE COLISIONS MATRIX", e);
    e = cudaMalloc((void **)b, sizeof(float) * (size_t)opts.nxyz);
    if (e != cudaSuccess) return report_cuda("ALLOCATION FOR DIRECT COLISIONS", e);
    const int rc = gd_export_tables(vgrid.context(), *b, *a, nullptr);
    if (rc) report("MATRICES STORED IN GLOBAL MEMORY", rc);
    cudaDeviceSynchronize();
}

// velocity.cu:53-65
void init_correction_array(float **correction_array, const DeviceVelocityGrid &vgrid, const Options &opts)
{
    cudaError_t e = cudaMalloc((void **)correction_array, sizeof(float) * 14 * (size_t)opts.nxyz);
    if (e != cudaSuccess) return report_cuda("CORRECTION ARRAY", e);
    const int rc = gd_correction_basis(vgrid.context(), *correction_array, nullptr);
    if (rc) report("CORRECTION ARRAY", rc);
}

namespace {
void evolve_any(float *f, float *direct_integral, float *inverse_integral, bool correct, const Options &opts)
{
    gd_ctx *ctx;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        ctx = g_current;
    }
    gd_info inf{};
    if (!ctx || gd_ctx_info(ctx, &inf)) return report("EVOLVE COLISIONS: no device velocity grid", GD_ERR_INVALID_ARG);
    if (inf.nx * inf.ny * inf.nz != opts.nxyz) {
        std::printf("EVOLVE COLISIONS: options grid %d does not match the device grid %d\n", opts.nxyz,
                    inf.nx * inf.ny * inf.nz);
        return;
    }
    const int npx = opts.npx;
    int rc;
    if (inf.n_pnt == opts.nxyz) {
        rc = gd_collision(ctx, f, npx, npx, direct_integral, inverse_integral, nullptr);
        if (!rc && correct)
            rc = gd_project(ctx, f, direct_integral, inverse_integral, npx, npx, direct_integral, nullptr, nullptr,
                            nullptr);
    } else {
        if (!g_scratch.ensure((size_t)inf.n_pnt * npx)) return report_cuda("EVOLVE COLISIONS", cudaErrorMemoryAllocation);
        rc = gd_box_to_compact(ctx, f, npx, npx, g_scratch.f, npx, nullptr);
        if (!rc) rc = gd_collision(ctx, g_scratch.f, npx, npx, g_scratch.nu, g_scratch.gain, nullptr);
        if (!rc && correct)
            rc = gd_project(ctx, g_scratch.f, g_scratch.nu, g_scratch.gain, npx, npx, g_scratch.nu, nullptr, nullptr,
                            nullptr);
        if (!rc) rc = gd_compact_to_box(ctx, g_scratch.nu, npx, npx, direct_integral, npx, nullptr);
        if (!rc) rc = gd_compact_to_box(ctx, g_scratch.gain, npx, npx, inverse_integral, npx, nullptr);
    }
    if (rc) report("EVOLVE COLISIONS", rc);
}
}  // namespace

// collision_integral.cu:550-773
void evolve_colisions(float *f, float *direct_integral, float *inverse_integral, float *, float *, float *,
                      const Options &opts)
{
    evolve_any(f, direct_integral, inverse_integral, true, opts);
}

void evolve_colisions_raw(float *f, float *direct_integral, float *inverse_integral, const Options &opts)
{
    evolve_any(f, direct_integral, inverse_integral, false, opts);
}

extern "C" int gd_load_options(const char *path, gd_options *out)
{
    if (!path || !out) return gd_set_error_message(GD_ERR_INVALID_ARG, "NULL argument");
    Options o{};
    try {
        load_options(o, path);
    } catch (const std::runtime_error &e) {
        return gd_set_error_message(GD_ERR_IO, e.what());
    } catch (const std::exception &e) {
        return gd_set_error_message(GD_ERR_INVALID_ARG, std::string("bad option value: ") + e.what());
    }
    out->nx = o.nx;
    out->ny = o.ny;
    out->nz = o.nz;
    out->nyz = o.nyz;
    out->nxyz = o.nxyz;
    out->npx = o.npx;
    return GD_OK;
}

namespace {
void relax_any(float *f, float *frequency, float *inverse_integral, int mode, float param, float *time,
               const Options &opts)
{
    gd_ctx *ctx;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        ctx = g_current;
    }
    gd_info inf{};
    if (!ctx || gd_ctx_info(ctx, &inf)) return report("RELAX F: no device velocity grid", GD_ERR_INVALID_ARG);
    const int npx = opts.npx;
    int rc;
    if (inf.n_pnt == opts.nxyz) {
        rc = gd_relax(ctx, f, frequency, inverse_integral, npx, npx, mode, param, time, nullptr, nullptr);
    } else {
        if (!g_scratch.ensure((size_t)inf.n_pnt * npx)) return report_cuda("RELAX F", cudaErrorMemoryAllocation);
        rc = gd_box_to_compact(ctx, f, npx, npx, g_scratch.f, npx, nullptr);
        if (!rc) rc = gd_box_to_compact(ctx, frequency, npx, npx, g_scratch.nu, npx, nullptr);
        if (!rc) rc = gd_box_to_compact(ctx, inverse_integral, npx, npx, g_scratch.gain, npx, nullptr);
        if (!rc) rc = gd_relax(ctx, g_scratch.f, g_scratch.nu, g_scratch.gain, npx, npx, mode, param, time, nullptr,
                               nullptr);
        if (!rc) rc = gd_compact_to_box(ctx, g_scratch.f, npx, npx, f, npx, nullptr);
    }
    if (rc) report("RELAX F", rc);
    cudaDeviceSynchronize();
}
}  // namespace

// collision_integral.cu:835-880
void relax_f(float *f, float *frequency, float *inverse_integral, float courant, float *time, const Options &opts)
{
    relax_any(f, frequency, inverse_integral, GD_DT_COURANT, courant, time, opts);
}

void relax_f_fixed(float *f, float *frequency, float *inverse_integral, float dt, float *time, const Options &opts)
{
    relax_any(f, frequency, inverse_integral, GD_DT_FIXED, dt, time, opts);
}

bool save_checkpoint(const std::string &path, const gd_grid_spec &spec, const float *f_dev, int nxyz, int npx,
                     int64_t step, double time)
{
    std::vector<float> h((size_t)nxyz * npx);
    cudaError_t e = cudaMemcpy(h.data(), f_dev, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "checkpoint %s: %s\n", path.c_str(), cudaGetErrorString(e));
        return false;
    }
    CheckpointHeader hd{};
    std::memcpy(hd.magic, "GDCKPT01", 8);
    hd.version = 1;
    hd.spec = spec;
    hd.nxyz = nxyz;
    hd.npx = npx;
    hd.step = step;
    hd.time = time;
    hd.payload_hash = fnv1a(h.data(), h.size() * sizeof(float));
    std::ofstream out(path, std::ios::binary);
    out.write(reinterpret_cast<const char *>(&hd), sizeof(hd));
    out.write(reinterpret_cast<const char *>(h.data()), (std::streamsize)(h.size() * sizeof(float)));
    if (!out) {
        std::fprintf(stderr, "checkpoint %s: write failed\n", path.c_str());
        return false;
    }
    return true;
}

bool load_checkpoint(const std::string &path, const gd_grid_spec &spec, float *f_dev, int nxyz, int npx,
                     int64_t *step, double *time)
{
    std::ifstream in(path, std::ios::binary);
    CheckpointHeader hd{};
    if (!in.read(reinterpret_cast<char *>(&hd), sizeof(hd)) || std::memcmp(hd.magic, "GDCKPT01", 8) != 0 ||
        hd.version != 1) {
        std::fprintf(stderr, "checkpoint %s: not a checkpoint file\n", path.c_str());
        return false;
    }
    if (std::memcmp(&hd.spec, &spec, sizeof(spec)) != 0 || hd.nxyz != nxyz || hd.npx != npx) {
        std::fprintf(stderr, "checkpoint %s: grid or batch differs from this run\n", path.c_str());
        return false;
    }
    std::vector<float> h((size_t)nxyz * npx);
    if (!in.read(reinterpret_cast<char *>(h.data()), (std::streamsize)(h.size() * sizeof(float))) ||
        fnv1a(h.data(), h.size() * sizeof(float)) != hd.payload_hash) {
        std::fprintf(stderr, "checkpoint %s: payload truncated or corrupt\n", path.c_str());
        return false;
    }
    if (cudaMemcpy(f_dev, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    *step = hd.step;
    *time = hd.time;
    return true;
}
