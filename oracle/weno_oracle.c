/* WENO5 advection oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * C restatement of the reference's periodic WENO advection operator
 * (cuSten/src/kernels/2d_xyADVWENO_p_kernel.cu): for every point
 *   out[y][x] = u[y][x] * Fx + v[y][x] * Fy                                        (:424)
 * with Fx / Fy the fifth-order WENO reconstruction (wenoSten, :52-88) of the one-sided differences
 * D(i) = (f[i] - f[i-1]) * coe, taken at x-2 .. x+2 when u > 0 and at x+3 .. x-1 (reversed) otherwise
 * (:286-348; y direction :352-414). Both directions are periodic; with the handle's standard halo
 * pointers the reference's per-tile halos are the periodic neighbours, so the tile and block
 * structure does not enter the result.
 *
 * Arithmetic: every multiply-add that the CUDA compiler may contract in the reference kernel is an
 * explicit fma() here (this file is compiled with -ffp-contract=off), in the pattern LLVM's contraction
 * produces for these expressions: (A*p - B*q) + C*r -> fma(C, r, fma(A, p, -(B*q))) and so on.
 *
 * Tolerance, not bit-exactness: the reference squares its smoothness terms with CUDA's single-precision
 * powf(t, 2), whose result is not always the correctly rounded square of t; this oracle takes the
 * correctly rounded square (CUDA's powf is not restated). The two agree to the float precision of those
 * terms: against the reference kernel's own outputs (tests/golden/reference_weno.npz) the relative L2
 * difference is at most 1.4e-8 and the largest difference at most 3.4e-8 of the largest value. Bit-exact
 * parity of the library's kernel is established against the reference kernel itself on the GPU, where
 * both call the same powf. */
#include <math.h>
#include <stddef.h>

static double sq_f32(double t) {
    const float f = (float)t;
    return (double)(float)((double)f * (double)f);   /* the product of two floats is exact in double */
}

static double weno5_ref(double v1, double v2, double v3, double v4, double v5) {
    const double phi1 = fma(11.0 / 6.0, v3, fma(1.0 / 3.0, v1, -((7.0 / 6.0) * v2)));
    const double phi2 = fma(1.0 / 3.0, v4, fma(-(1.0 / 6.0), v2, (5.0 / 6.0) * v3));
    const double phi3 = fma(-(1.0 / 6.0), v5, fma(1.0 / 3.0, v3, (5.0 / 6.0) * v4));

    const double s1 = fma(13.0 / 12.0, sq_f32(fma(-2.0, v2, v1) + v3),
                          0.25 * sq_f32(fma(3.0, v3, fma(-4.0, v2, v1))));
    const double s2 = fma(13.0 / 12.0, sq_f32(fma(-2.0, v3, v2) + v4), 0.25 * sq_f32(v2 - v4));
    const double s3 = fma(13.0 / 12.0, sq_f32(fma(-2.0, v4, v3) + v5),
                          0.25 * sq_f32(fma(3.0, v3, -(4.0 * v4)) + v5));

    const double eps = 1e-06;
    const double a1 = 0.1 / sq_f32(s1 + eps);
    const double a2 = 0.6 / sq_f32(s2 + eps);
    const double a3 = 0.3 / sq_f32(s3 + eps);
    const double denom = 1.0 / (a1 + a2 + a3);
    const double w1 = a1 * denom, w2 = a2 * denom, w3 = a3 * denom;
    return fma(phi3, w3, fma(phi1, w1, phi2 * w2));
}

static int wrapi(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

/* Fields nx x ny, row-major; cdx = 1/dx, cdy = 1/dy as the handle stores them. */
void oracle_weno_f64(int nx, int ny, const double* in, const double* u, const double* v, double* out, double cdx,
                     double cdy) {
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            double dxk[6], dyk[6];   /* D at x-2 .. x+3 and at y-2 .. y+3 */
            for (int k = 0; k < 6; ++k) {
                const int xi = wrapi(x - 2 + k, nx), xm = wrapi(x - 3 + k, nx);
                const int yi = wrapi(y - 2 + k, ny), ym = wrapi(y - 3 + k, ny);
                dxk[k] = (in[(size_t)y * nx + xi] - in[(size_t)y * nx + xm]) * cdx;
                dyk[k] = (in[(size_t)yi * nx + x] - in[(size_t)ym * nx + x]) * cdy;
            }
            const double uu = u[(size_t)y * nx + x], vv = v[(size_t)y * nx + x];
            const double fx = uu > 0.0 ? weno5_ref(dxk[0], dxk[1], dxk[2], dxk[3], dxk[4])
                                       : weno5_ref(dxk[5], dxk[4], dxk[3], dxk[2], dxk[1]);
            const double fy = vv > 0.0 ? weno5_ref(dyk[0], dyk[1], dyk[2], dyk[3], dyk[4])
                                       : weno5_ref(dyk[5], dyk[4], dyk[3], dyk[2], dyk[1]);
            out[(size_t)y * nx + x] = fma(uu, fx, vv * fy);
        }
    }
}
