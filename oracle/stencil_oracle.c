/* CPU oracle for the cuSten stencil kernels -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference kernels (cuSten/src/kernels/2d_*_kernel.cu), used by the
 * tests, by smoke() and by the CPU baseline leg of bench.py as the checker. Nothing in the library
 * links or calls this file. Build: gcc -O2 -ffp-contract=off -fPIC -shared (contraction must stay
 * off: every fused multiply-add here is an explicit fma()/fmaf() call, in the reference's order).
 *
 * Pinning: the restatement is checked against the reference examples' analytic answers
 * (the examples under examples/src) on the CPU, and against the reference kernels themselves, rebuilt for sm_103a
 * from the reference sources (oracle/ref_kernels.cu), on the GPU.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define REAL double
#define FMA fma
#define SFX f64
#include "stencil_oracle_impl.h"
#undef REAL
#undef FMA
#undef SFX

#define REAL float
#define FMA fmaf
#define SFX f32
#include "stencil_oracle_impl.h"
#undef REAL
#undef FMA
#undef SFX

/* Plain host loop of a periodic XY stencil (the "plain host loop with the same weights" CPU
 * baseline): out[y][x] = fma chain over the H x V window with modular indexing, rows [y0, y1). */
void oracle_host_loop_xyp_f64(int nx, int ny, const double* in, double* out, const double* w, int H, int L, int V,
                              int T, int y0, int y1) {
    for (int y = y0; y < y1; ++y) {
        for (int x = 0; x < nx; ++x) {
            double s = 0.0;
            int k = 0;
            for (int j = 0; j < V; ++j) {
                int yy = y - T + j;
                yy = yy < 0 ? yy + ny : (yy >= ny ? yy - ny : yy);
                const double* row = in + (size_t)yy * nx;
                for (int i = 0; i < H; ++i) {
                    int xx = x - L + i;
                    xx = xx < 0 ? xx + nx : (xx >= nx ? xx - nx : xx);
                    s = fma(w[k++], row[xx], s);
                }
            }
            out[(size_t)y * nx + x] = s;
        }
    }
}

/* Plain host loop with modular indexing for any variant's window (CPU baseline): periodic in both
 * directions, out[y][x] = fma chain of w[j*H+i] * g(in[y-T+j][x-L+i]), g(c) = c (cube = 0) or
 * c^3 - c computed as fma(c*c, c, -c) (cube = 1), rows [y0, y1). */
void oracle_host_loop_f64(int nx, int ny, const double* in, double* out, const double* w, int H, int L, int V, int T,
                          int cube, int y0, int y1) {
    for (int y = y0; y < y1; ++y) {
        for (int x = 0; x < nx; ++x) {
            double s = 0.0;
            int k = 0;
            for (int j = 0; j < V; ++j) {
                int yy = y - T + j;
                yy = yy < 0 ? yy + ny : (yy >= ny ? yy - ny : yy);
                const double* row = in + (size_t)yy * nx;
                for (int i = 0; i < H; ++i) {
                    int xx = x - L + i;
                    xx = xx < 0 ? xx + nx : (xx >= nx ? xx - nx : xx);
                    double c = row[xx];
                    double g = cube ? fma(c * c, c, -c) : c;
                    s = fma(w[k++], g, s);
                }
            }
            out[(size_t)y * nx + x] = s;
        }
    }
}
