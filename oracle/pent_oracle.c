/* Batched pentadiagonal oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * C restatement of cuPentBatch's pentFactorBatch and pentSolveBatch
 * (cuPentCahnADI/src/cuPentBatch.cu:35-113, :119-198) over the interleaved layout [row * batch + sys].
 * The expressions the CUDA compiler contracts are explicit fma() calls here (this file is compiled with
 * -ffp-contract=off): x - a*b - c*d -> fma(-c, d, fma(-a, b, x)); divisions are IEEE divisions in both.
 * Checked bit for bit against the reference kernels on the GPU (tests/golden/reference_pent.npz). */
#include <math.h>
#include <stddef.h>

void oracle_pent_factor(double* ds, double* dl, double* d, double* du, double* dw, int m, int batch) {
    for (int s = 0; s < batch; ++s) {
#define AT(a, i) a[(size_t)(i) * batch + s]
        AT(du, 0) = AT(du, 0) / AT(d, 0);
        AT(dw, 0) = AT(dw, 0) / AT(d, 0);
        AT(d, 1) = fma(-AT(dl, 1), AT(du, 0), AT(d, 1));
        AT(du, 1) = fma(-AT(dl, 1), AT(dw, 0), AT(du, 1)) / AT(d, 1);
        AT(dw, 1) = AT(dw, 1) / AT(d, 1);
        for (int i = 2; i < m; ++i) {
            AT(dl, i) = fma(-AT(ds, i), AT(du, i - 2), AT(dl, i));
            AT(d, i) = fma(-AT(dl, i), AT(du, i - 1), fma(-AT(ds, i), AT(dw, i - 2), AT(d, i)));
            if (i < m - 2) AT(dw, i) = AT(dw, i) / AT(d, i);
            if (i < m - 1) AT(du, i) = fma(-AT(dl, i), AT(dw, i - 1), AT(du, i)) / AT(d, i);
        }
#undef AT
    }
}

void oracle_pent_solve(const double* ds, const double* dl, const double* d, const double* du, const double* dw,
                       double* b, int m, int batch) {
    for (int s = 0; s < batch; ++s) {
#define AT(a, i) a[(size_t)(i) * batch + s]
        AT(b, 0) = AT(b, 0) / AT(d, 0);
        AT(b, 1) = fma(-AT(dl, 1), AT(b, 0), AT(b, 1)) / AT(d, 1);
        for (int i = 2; i < m; ++i)
            AT(b, i) = fma(-AT(dl, i), AT(b, i - 1), fma(-AT(ds, i), AT(b, i - 2), AT(b, i))) / AT(d, i);
        AT(b, m - 2) = fma(-AT(du, m - 2), AT(b, m - 1), AT(b, m - 2));
        for (int i = m - 3; i >= 0; --i)
            AT(b, i) = fma(-AT(dw, i), AT(b, i + 2), fma(-AT(du, i), AT(b, i + 1), AT(b, i)));
#undef AT
    }
}
