// gpu_determ_api.hpp -- the reference's C++ host interface over libgpu_determ.so.
//
// Same names, argument meaning and conventions as savthe/gpu_determ's host
// API (device pointers, layout [node][cell] with npx cells fastest), so a
// caller of the reference links this library instead of the reference's
// objects.  Everything forwards to the C ABI in gpu_determ.h.
//
// Differences from the reference, all deliberate:
//  - VelocityGrid::device() returns a device mirror owned by that grid (the
//    reference keeps one function-static mirror per process,
//    velocity_grid.cu:21-25); the most recently created mirror is the one
//    evolve_colisions / relax_f use, since their signatures carry no grid.
//  - evolve_colisions solves the 5x5 conservation system of every cell
//    (the reference solves cell 0 only, collision_integral.cu:471) and writes
//    the gain of node (i, j, k) to node (i, j, k) (the reference writes it at
//    i*nx + (j*nz + k), collision_integral.cu:162).
//  - Failures print the CUDA or library message and return, as the reference
//    does; load_options throws std::runtime_error("Can't open <file>") as the
//    reference does (options.cu:37).
#pragma once

#include <cstdint>
#include <string>

#include "gpu_determ.h"

// options.hpp:6-17 -------------------------------------------------------------
struct Options {
    int nx;
    int ny;
    int nz;
    int nyz;
    int nxyz;
    int npx;
};

// "key = value" lines, '#' comments, unknown keys ignored; derives nyz, nxyz.
void load_options(Options &, const std::string &);
void print_options(const Options &);

// Extension of the same file format with the run parameters the reference
// hard-codes in determ.cu:47-50,69,77 (new keys; a plain reference gpu.conf
// parses to the reference's values).
struct RunOptions {
    Options base{16, 16, 16, 256, 4096, 256};
    float vmin[3] = {-5.f, -5.f, -5.f};
    float vmax[3] = {5.f, 5.f, 5.f};
    float R = 16.5f;          // key "R"
    int steps = 1;            // key "steps"
    int dt_mode = GD_DT_COURANT;  // key "dt_mode": courant | fixed
    float courant = 0.5f;     // key "courant"
    float dt = 0.05f;         // key "dt"
    int out_step = 5;         // key "out_step": steps between moment reports
    std::string init = "reference";  // key "init": reference | two_beam | mixture
    int seed = 0;             // key "seed"
    std::string results = "results.out";  // key "results"
    std::string checkpoint;   // key "checkpoint": file written after the last step
    std::string resume;       // key "resume": checkpoint file to start from
    bool literal_rows = true; // key "rows": literal (reference row order) | cells
    bool correction = true;   // key "correction": per_cell | none
    std::string gain = "pair";  // key "gain": pair (FP32 kernel) | pair_tc (its contraction on tensor cores) |
                                // bf16 | bf16x3 (collision matrices)
};
void load_run_options(RunOptions &, const std::string &);

// common.hpp:26-35 ---------------------------------------------------------------
template <typename T>
struct Vector3D {
    Vector3D() : x(), y(), z() {}
    Vector3D(const T &x_, const T &y_, const T &z_) : x(x_), y(y_), z(z_) {}
    T x, y, z;
};
using Vector3i = Vector3D<int>;
using Vector3f = Vector3D<float>;

// velocity_grid.hpp:6-54 ---------------------------------------------------------
class VelocityGridBase {
public:
    virtual ~VelocityGridBase() {}
    int n_pnt = 0;
    int n_u = 0;
    int n_w = 0;
    int n_v = 0;
    float *u = nullptr;
    float *v = nullptr;
    float *w = nullptr;
    int *u_index = nullptr;
    int *v_index = nullptr;
    int *w_index = nullptr;
    int n_uvw = 0;
    float min_u = 0, min_v = 0, min_w = 0;
    float max_u = 0, max_v = 0, max_w = 0;
    float d_u = 0, d_v = 0, d_w = 0;
    float d3v = 0;
};

class DeviceVelocityGrid;

class VelocityGrid : public VelocityGridBase {
public:
    VelocityGrid() {}
    VelocityGrid(Vector3i n_points, Vector3f v_min, Vector3f v_max, float r);
    virtual ~VelocityGrid();
    void init(Vector3i n_points, Vector3f v_min, Vector3f v_max, float R);
    DeviceVelocityGrid &device() const;
    float radius() const { return R_; }

private:
    float R_ = 0.f;
    mutable DeviceVelocityGrid *device_ = nullptr;
};

// Device copies of the grid arrays (pointers are device pointers) plus the
// library context with the weight tables.
class DeviceVelocityGrid : public VelocityGridBase {
    friend class VelocityGrid;
    explicit DeviceVelocityGrid(const VelocityGrid &);

public:
    void free();
    gd_ctx *context() const { return ctx_; }

private:
    gd_ctx *ctx_ = nullptr;
};

// compute_matrix.h:13 -- allocates b[nxyz] and a[nxyz*nxyz/8] on the device
// (caller frees with cudaFree) and fills them with the analytic weights.
void init_matrices(const DeviceVelocityGrid &, float **b, float **a, const Options &opts);
// velocity.h:41 -- allocates and fills the 14 x nxyz moment basis.
void init_correction_array(float **correction_array, const DeviceVelocityGrid &, const Options &opts);
// collision_integral.h:11-17 -- direct_integral <- corrected collision
// frequency nu', inverse_integral <- gain I, for npx cells of f [nxyz][npx].
// b, a and correction_array are accepted for signature compatibility; the
// library uses its own compact tables.
void evolve_colisions(float *f, float *direct_integral, float *inverse_integral, float *b, float *a,
                      float *correction_array, const Options &opts);
// The same without the conservation correction: direct_integral <- nu.
// This is what the reference delivers for every cell but cell 0 (its 5x5
// solve runs for cell 0 only), so results.out rows can be compared with its
// golden file.
void evolve_colisions_raw(float *f, float *direct_integral, float *inverse_integral, const Options &opts);
// collision_integral.h:19-24 -- dt = courant / max nu, f <- f + dt (I - f nu),
// *time += dt (time is a device float).
void relax_f(float *f, float *frequency, float *inverse_integral, float courant, float *time,
             const Options &opts);

// Same update with a fixed time step dt (the reference has only the Courant
// form); *time += dt.
void relax_f_fixed(float *f, float *frequency, float *inverse_integral, float dt, float *time,
                   const Options &opts);

// Checkpoint of a distribution f [nxyz][npx] (device) with step and time:
// a small header (magic, version, grid spec, npx, step, time, FNV-1a hash of
// the payload) followed by the float payload.  Returns false on I/O or
// format errors (message on stderr).
bool save_checkpoint(const std::string &path, const gd_grid_spec &spec, const float *f_dev, int nxyz,
                     int npx, int64_t step, double time);
bool load_checkpoint(const std::string &path, const gd_grid_spec &spec, float *f_dev, int nxyz, int npx,
                     int64_t *step, double *time);
