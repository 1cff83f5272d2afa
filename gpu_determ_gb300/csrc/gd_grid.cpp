// gd_grid.cpp -- velocity lattice and sphere mask (host).
//
// Compiled with -ffp-contract=off: the membership test must round exactly as
// the reference's host code does, since the in-sphere index lists are part of
// the bit-exact contract.  Reference: velocity_grid.cu:6-14 (membership),
// :73-126 (VelocityGrid::init).
#include <cmath>

#include "gd_internal.h"

namespace gd {

namespace {

// Centre of node (i, j, k) as the membership test forms it: extent times
// (2i + 1 - n) in float, halved and divided by n in double, rounded to float;
// then u^2 + v^2 + w^2 < R^2 in float (R <= 0 keeps every node).
bool in_sphere(const gd_grid_spec &s, int i, int j, int k)
{
    const float tu = (s.vmax[0] - s.vmin[0]) * (float)(2 * i + 1 - s.nx);
    const float tv = (s.vmax[1] - s.vmin[1]) * (float)(2 * j + 1 - s.ny);
    const float tw = (s.vmax[2] - s.vmin[2]) * (float)(2 * k + 1 - s.nz);
    const float u = (float)((double)tu / 2. / (double)s.nx);
    const float v = (float)((double)tv / 2. / (double)s.ny);
    const float w = (float)((double)tw / 2. / (double)s.nz);
    if (s.R <= 0) return true;
    float r2 = u * u;
    r2 = r2 + v * v;
    r2 = r2 + w * w;
    return r2 < s.R * s.R;
}

}  // namespace

int grid_count(const gd_grid_spec &s)
{
    int n = 0;
    for (int i = 0; i < s.nx; i++)
        for (int j = 0; j < s.ny; j++)
            for (int k = 0; k < s.nz; k++) n += in_sphere(s, i, j, k) ? 1 : 0;
    return n;
}

// Steps d = (max - min)/n in float, d3v = du dv dw in float, node centres
// min + d (2i + 1)/2 evaluated in double and stored as float.
int grid_fill(const gd_grid_spec &s, float *u, float *v, float *w, int *ui, int *vi, int *wi,
              float *steps)
{
    const float du = (s.vmax[0] - s.vmin[0]) / (float)s.nx;
    const float dv = (s.vmax[1] - s.vmin[1]) / (float)s.ny;
    const float dw = (s.vmax[2] - s.vmin[2]) / (float)s.nz;
    float d3v = du * dv;
    d3v = d3v * dw;
    if (u)
        for (int i = 0; i < s.nx; i++) u[i] = (float)((double)s.vmin[0] + (double)du * (2. * i + 1.) / 2.);
    if (v)
        for (int i = 0; i < s.ny; i++) v[i] = (float)((double)s.vmin[1] + (double)dv * (2. * i + 1.) / 2.);
    if (w)
        for (int i = 0; i < s.nz; i++) w[i] = (float)((double)s.vmin[2] + (double)dw * (2. * i + 1.) / 2.);
    int n = 0;
    for (int i = 0; i < s.nx; i++)
        for (int j = 0; j < s.ny; j++)
            for (int k = 0; k < s.nz; k++)
                if (in_sphere(s, i, j, k)) {
                    if (ui) ui[n] = i;
                    if (vi) vi[n] = j;
                    if (wi) wi[n] = k;
                    n++;
                }
    if (steps) {
        steps[0] = du;
        steps[1] = dv;
        steps[2] = dw;
        steps[3] = d3v;
    }
    return n;
}

}  // namespace gd
