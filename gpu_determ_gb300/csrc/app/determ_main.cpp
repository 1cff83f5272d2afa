// determ_main.cpp -- command-line driver over the reference's C++ interface.
//
// Runs what the reference's main does (determ.cu:41-99): read the options
// file, build the velocity grid, set the initial distribution, build the
// correction basis and weight tables, advance `steps` collision steps with
// evolve_colisions + relax_f, and write results.out in the reference's
// nine-column format (index I J K F DC IC CI ACC, determ.cu:146-160).
//
//   gd_determ [options-file]      (default ./gpu.conf)
//
// Option keys beyond the reference's nx, ny, nz, npx: vmin, vmax, R, steps,
// dt_mode (courant|fixed), courant, dt, out_step, init (reference|two_beam|
// mixture), seed, results, checkpoint, resume, rows (literal|cells),
// correction (per_cell|none), gain (pair|pair_tc|bf16|bf16x3).
// rows = literal writes the reference's row set (it reads the [node][cell]
// arrays with a flat node index, so row "index" is node*npx + cell over the
// first nx*ny*nz entries); rows = cells writes one row per (node, cell).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "gpu_determ_api.hpp"

namespace {

// determ.cu:101-121, and the two other seeded initial states
void init_f(const RunOptions &ro, const VelocityGrid &g, std::vector<float> &h)
{
    const Options &o = ro.base;
    uint64_t state = 0x9E3779B97F4A7C15ull ^ (uint64_t)ro.seed;
    auto uniform = [&]() {
        state = state * 6364136223846793005ull + 1442695040888963407ull;
        return ((state >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() { return std::sqrt(-2.0 * std::log(uniform())) * std::cos(6.283185307179586 * uniform()); };
    struct M { double n, ux, uy, uz, T; };
    std::vector<std::vector<M>> mix(o.npx);
    for (int c = 0; c < o.npx; c++) {
        if (ro.init == "two_beam") {
            mix[c] = {{0.5, 1.5, 0, 0, 1.0}, {0.5, -1.5, 0, 0, 1.0}};
        } else if (ro.init == "mixture") {
            const int k = 1 + (int)(uniform() * 3);
            for (int q = 0; q < k; q++)
                mix[c].push_back({std::exp(0.3 * normal()), 0.7 * normal(), 0.7 * normal(), 0.7 * normal(),
                                  0.6 + 1.2 * uniform()});
        }
    }
    for (int i = 0, index = 0; i < o.nx; i++)
        for (int j = 0; j < o.ny; j++)
            for (int k = 0; k < o.nz; k++, index++) {
                const float u = g.u[i], v = g.v[j], w = g.w[k];
                for (int c = 0; c < o.npx; c++) {
                    float val;
                    if (ro.init == "reference") {
                        const float u1 = 1.75f, v1 = 0.25f;
                        val = std::exp(-(u - u1) * (u - u1) - (v - v1) * (v - v1) - w * w);
                    } else {
                        double s = 0;
                        for (const M &m : mix[c]) {
                            const double c2 = (u - m.ux) * (u - m.ux) + (v - m.uy) * (v - m.uy) + (w - m.uz) * (w - m.uz);
                            s += m.n * std::pow(M_PI * m.T, -1.5) * std::exp(-c2 / m.T);
                        }
                        val = (float)s;
                    }
                    h[(size_t)index * o.npx + c] = val;
                }
            }
}

}  // namespace

int main(int argc, char **argv)
{
    RunOptions ro;
    try {
        load_run_options(ro, argc > 1 ? argv[1] : "gpu.conf");
    } catch (const std::exception &e) {
        std::cerr << e.what() << std::endl;
        return 2;
    }
    const Options &opts = ro.base;
    print_options(opts);
    VelocityGrid vgrid(Vector3i(opts.nx, opts.ny, opts.nz), Vector3f(ro.vmin[0], ro.vmin[1], ro.vmin[2]),
                       Vector3f(ro.vmax[0], ro.vmax[1], ro.vmax[2]), ro.R);
    if (vgrid.n_pnt != opts.nxyz && ro.literal_rows) {
        std::cerr << "rows = literal needs every box node inside the sphere; use rows = cells" << std::endl;
        return 2;
    }
    // the sphere mask zeroes f outside: build it on the compact order
    std::vector<float> h_f((size_t)opts.nxyz * opts.npx);
    init_f(ro, vgrid, h_f);
    if (vgrid.n_pnt != opts.nxyz) {
        std::vector<char> inside(opts.nxyz, 0);
        for (int p = 0; p < vgrid.n_pnt; p++)
            inside[(vgrid.u_index[p] * opts.ny + vgrid.v_index[p]) * opts.nz + vgrid.w_index[p]] = 1;
        for (int b = 0; b < opts.nxyz; b++)
            if (!inside[b])
                for (int c = 0; c < opts.npx; c++) h_f[(size_t)b * opts.npx + c] = 0.f;
    }
    const size_t bytes = sizeof(float) * opts.nxyz * (size_t)opts.npx;
    float *d_f = nullptr, *d_direct = nullptr, *d_inverse = nullptr, *d_time = nullptr;
    if (cudaMalloc((void **)&d_f, bytes) != cudaSuccess || cudaMalloc((void **)&d_direct, bytes) != cudaSuccess ||
        cudaMalloc((void **)&d_inverse, bytes) != cudaSuccess || cudaMalloc((void **)&d_time, sizeof(float)) != cudaSuccess) {
        std::cerr << "device allocation failed: " << cudaGetErrorString(cudaGetLastError()) << std::endl;
        return 4;
    }
    cudaMemcpy(d_f, h_f.data(), bytes, cudaMemcpyHostToDevice);
    float *correction_array = nullptr, *a = nullptr, *b = nullptr;
    init_correction_array(&correction_array, vgrid.device(), opts);
    init_matrices(vgrid.device(), &b, &a, opts);
    if (ro.gain != "pair") {
        const int path = ro.gain == "bf16"      ? GD_GAIN_CMATRIX_BF16
                         : ro.gain == "pair_tc" ? GD_GAIN_PAIR_TC
                                                : GD_GAIN_CMATRIX_BF16X3;
        if (gd_ctx_set_gain_path(vgrid.device().context(), path) != GD_OK) {
            std::cerr << "gain path " << ro.gain << ": " << gd_last_error() << std::endl;
            return 5;
        }
    }

    gd_grid_spec spec{opts.nx, opts.ny, opts.nz, {ro.vmin[0], ro.vmin[1], ro.vmin[2]},
                      {ro.vmax[0], ro.vmax[1], ro.vmax[2]}, ro.R};
    int64_t step0 = 0;
    double t0 = 0.0;
    if (!ro.resume.empty() && !load_checkpoint(ro.resume, spec, d_f, opts.nxyz, opts.npx, &step0, &t0)) return 3;
    float h_time = (float)t0;
    cudaMemcpy(d_time, &h_time, sizeof(float), cudaMemcpyHostToDevice);
    for (int64_t step = step0; step < step0 + ro.steps; ++step) {
        cudaMemcpy(&h_time, d_time, sizeof(float), cudaMemcpyDeviceToHost);
        std::cout << "STEP=" << step << ",  TIME=" << h_time << std::endl;
        if (step % ro.out_step == 0) cudaMemcpy(h_f.data(), d_f, bytes, cudaMemcpyDeviceToHost);
        if (ro.correction) evolve_colisions(d_f, d_direct, d_inverse, b, a, correction_array, opts);
        else evolve_colisions_raw(d_f, d_direct, d_inverse, opts);
        if (ro.dt_mode == GD_DT_FIXED) relax_f_fixed(d_f, d_direct, d_inverse, ro.dt, d_time, opts);
        else relax_f(d_f, d_direct, d_inverse, ro.courant, d_time, opts);
    }
    cudaDeviceSynchronize();
    std::cout << "COLLISIONS EVOLVED: " << cudaGetErrorString(cudaGetLastError()) << std::endl;

    std::vector<float> h_direct((size_t)opts.nxyz * opts.npx), h_inverse((size_t)opts.nxyz * opts.npx);
    cudaMemcpy(h_direct.data(), d_direct, bytes, cudaMemcpyDeviceToHost);
    cudaMemcpy(h_inverse.data(), d_inverse, bytes, cudaMemcpyDeviceToHost);
    std::ofstream fresults(ro.results.c_str());
    if (ro.literal_rows) {
        for (int index = 0; index < opts.nxyz; index++)
            if (vgrid.u_index[index] < vgrid.n_u / 2 && vgrid.v_index[index] < vgrid.n_v / 2 &&
                vgrid.w_index[index] < vgrid.n_w / 2)
                fresults << index << ' ' << index / opts.nyz << ' ' << (index % opts.nyz) / opts.nz << ' '
                         << (index % opts.nyz) % opts.nz << ' ' << h_f[index] << ' ' << h_direct[index] << ' '
                         << h_inverse[index] << ' ' << -h_f[index] * h_direct[index] + h_inverse[index] << ' '
                         << -h_f[index] * h_direct[index] / h_inverse[index] + 1.0 << std::endl;
    } else {
        for (int p = 0; p < vgrid.n_pnt; p++) {
            const int i = vgrid.u_index[p], j = vgrid.v_index[p], k = vgrid.w_index[p];
            const size_t node = ((size_t)i * opts.ny + j) * opts.nz + k;
            for (int c = 0; c < opts.npx; c++) {
                const size_t o = node * opts.npx + c;
                fresults << node << ' ' << i << ' ' << j << ' ' << k << ' ' << c << ' ' << h_f[o] << ' '
                         << h_direct[o] << ' ' << h_inverse[o] << ' ' << -h_f[o] * h_direct[o] + h_inverse[o] << ' '
                         << -h_f[o] * h_direct[o] / h_inverse[o] + 1.0 << std::endl;
            }
        }
    }
    if (!ro.checkpoint.empty()) {
        cudaMemcpy(&h_time, d_time, sizeof(float), cudaMemcpyDeviceToHost);
        if (!save_checkpoint(ro.checkpoint, spec, d_f, opts.nxyz, opts.npx, step0 + ro.steps, h_time)) return 3;
    }
    cudaFree(d_f);
    cudaFree(d_direct);
    cudaFree(d_inverse);
    cudaFree(d_time);
    cudaFree(correction_array);
    cudaFree(a);
    cudaFree(b);
    std::cout << "END_PROGRAM: " << cudaGetErrorString(cudaGetLastError()) << std::endl;
    return 0;
}
