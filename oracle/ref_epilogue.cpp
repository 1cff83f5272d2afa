/* Epilogue streamed after the reference's weight functions: a C entry point
 * for the tests.  Test infrastructure only. */
extern "C" double ref_calc_matrix_element(double du, double dv, double dw, int in, int jn, int kn,
                                          double g)
{
    return calc_matrix_element(du, dv, dw, in, jn, kn, g);
}

/* Dense weight table a[(nx/2)*nx*(ny/2)*(nz/2)*ny*nz] with the reference's
 * own calc_matrix_element and the store rule of compute_matrix.cu:546-558
 * (|g| from float components and a float square root; area < 1e-10 -> 0;
 * else area * 2 |g| d3v in double, stored as float). */
#include <cmath>
extern "C" void ref_build_dense_a(int nx, int ny, int nz, float du, float dv, float dw, float d3v,
                                  float *a)
{
    const int nyz = ny * nz, hy = ny / 2, hz = nz / 2;
    for (int in1 = 0; in1 < nx / 2; in1++)
        for (int gi = 0; gi < nx; gi++)
            for (int jn1 = 0; jn1 < hy; jn1++)
                for (int kn1 = 0; kn1 < hz; kn1++)
                    for (int gj = 0; gj < ny; gj++)
                        for (int gk = 0; gk < nz; gk++) {
                            float gu = du * (float)gi, gv = dv * (float)gj, gw = dw * (float)gk;
                            float s = gu * gu;
                            s = s + gv * gv;
                            s = s + gw * gw;
                            double g1 = (double)std::sqrt(s);
                            int in = (gi & 1) | (in1 << 1), jn = (gj & 1) | (jn1 << 1),
                                kn = (gk & 1) | (kn1 << 1);
                            double A = calc_matrix_element(du, dv, dw, in, jn, kn, g1);
                            a[((size_t)(in1 * nx + gi) * (hy * hz) + jn1 * hz + kn1) * nyz +
                              gj * nz + gk] = (A < ERR) ? 0.0f : (float)(A * 2.0 * g1 * (double)d3v);
                        }
}
