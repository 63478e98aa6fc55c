/* CPU oracle for the Cahn-Hilliard ADI solver -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of cuPentSpeedUp/serialCahnADITiming/serialCahnADI.c (the reference's CPU
 * solver), used by the tests and the CPU baseline leg of bench.py as the checker; nothing in the
 * library links it. Every expression keeps the reference's operation order and the file is compiled
 * without floating-point contraction, so it reproduces the reference program bit for bit (checked
 * against the reference itself, built from its source by oracle/ref_build.py, where it is present).
 *
 * Scheme (serialCahnADI.c:1010-1047, one step):
 *   cBar  = 2 cCurr - cOld
 *   rhs   = L5x5(cBar) + N3x3(cCurr^3 - cCurr) - (2/3)(cCurr - cOld);  cOld = cCurr
 *   solve (1 + s Dxxxx) along x, then along y (cyclic pentadiagonal, Schur complement on the last
 *   two unknowns);  cCurr = cBar + solution.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* serialCahnADI.c:45-85 */
static void ch_set_lhs(double* ds, double* dl, double* dg, double* du, double* dw, double a, double b, double c,
                       double d, double e, int m) {
    for (int i = 0; i < m; ++i) {
        if (i > 1) ds[i] = a;
        if (i > 0) dl[i] = b;
        dg[i] = c;
        if (i < m - 1) du[i] = d;
        if (i < m - 2) dw[i] = e;
    }
}

/* serialCahnADI.c:91-162: in-place factorisation of the (non-cyclic) pentadiagonal matrix */
static void ch_pent_factor(double* ds, double* dl, double* dg, double* du, double* dw, int m) {
    du[0] = du[0] / dg[0];
    dw[0] = dw[0] / dg[0];
    dg[1] = dg[1] - dl[1] * du[0];
    du[1] = (du[1] - dl[1] * dw[0]) / dg[1];
    dw[1] = dw[1] / dg[1];
    for (int i = 2; i < m - 2; ++i) {
        dl[i] = dl[i] - ds[i] * du[i - 2];
        dg[i] = dg[i] - ds[i] * dw[i - 2] - dl[i] * du[i - 1];
        dw[i] = dw[i] / dg[i];
        du[i] = (du[i] - dl[i] * dw[i - 1]) / dg[i];
    }
    int i = m - 2;
    dl[i] = dl[i] - ds[i] * du[i - 2];
    dg[i] = dg[i] - ds[i] * dw[i - 2] - dl[i] * du[i - 1];
    du[i] = (du[i] - dl[i] * dw[i - 1]) / dg[i];
    i = m - 1;
    dl[i] = dl[i] - ds[i] * du[i - 2];
    dg[i] = dg[i] - ds[i] * dw[i - 2] - dl[i] * du[i - 1];
}

/* serialCahnADI.c:168-241: forward then backward substitution, in place (stride `st`) */
static void ch_pent_solve(const double* ds, const double* dl, const double* dg, const double* du, const double* dw,
                          double* x, int m, int st) {
    x[0] = x[0] / dg[0];
    x[st] = (x[st] - dl[1] * x[0]) / dg[1];
    for (int i = 2; i < m; ++i) x[i * st] = (x[i * st] - ds[i] * x[(i - 2) * st] - dl[i] * x[(i - 1) * st]) / dg[i];
    x[(m - 2) * st] = x[(m - 2) * st] - du[m - 2] * x[(m - 1) * st];
    for (int i = m - 3; i >= 0; --i) x[i * st] = x[i * st] - du[i] * x[(i + 1) * st] - dw[i] * x[(i + 2) * st];
}

/* serialCahnADI.c:247-414: the two border columns and the inverse of the 2x2 Schur complement */
static void ch_find_omega(double* omega, double* inv1, double* inv2, double a, double b, double c, double d, double e,
                          int m) {
    double* ds = malloc(sizeof(double) * m);
    double* dl = malloc(sizeof(double) * m);
    double* dg = malloc(sizeof(double) * m);
    double* du = malloc(sizeof(double) * m);
    double* dw = malloc(sizeof(double) * m);
    ch_set_lhs(ds, dl, dg, du, dw, a, b, c, d, e, m);
    ch_pent_factor(ds, dl, dg, du, dw, m);
    for (int i = 0; i < m; ++i) { inv1[i] = 0.0; inv2[i] = 0.0; }
    inv1[0] = a; inv1[m - 2] = e; inv1[m - 1] = d;      /* setInv1 */
    inv2[0] = b; inv2[1] = a; inv2[m - 1] = e;          /* setInv2 */
    ch_pent_solve(ds, dl, dg, du, dw, inv1, m, 1);
    ch_pent_solve(ds, dl, dg, du, dw, inv2, m, 1);
    double z11 = e * inv1[0] + a * inv1[m - 2] + b * inv1[m - 1];
    double z12 = e * inv2[0] + a * inv2[m - 2] + b * inv2[m - 1];
    double z21 = d * inv1[0] + e * inv1[1] + a * inv1[m - 1];
    double z22 = d * inv2[0] + e * inv2[1] + a * inv2[m - 1];
    double y11 = c - z11, y12 = d - z12, y21 = b - z21, y22 = c - z22;
    double det = 1.0 / (y11 * y22 - y21 * y12);
    omega[0] = y22 * det;
    omega[1] = -y12 * det;
    omega[2] = -y21 * det;
    omega[3] = y11 * det;
    free(ds); free(dl); free(dg); free(du); free(dw);
}

/* serialCahnADI.c:628-722: cyclic solve of one line of n values (stride st) */
static void ch_cyclic(const double* ds, const double* dl, const double* dg, const double* du, const double* dw,
                      const double* inv1, const double* inv2, const double* om, double* x, double a, double b,
                      double d, double e, int n, int st) {
    ch_pent_solve(ds, dl, dg, du, dw, x, n - 2, st);
    double n2 = x[(n - 2) * st] - (e * x[0] + a * x[(n - 4) * st] + b * x[(n - 3) * st]);
    double n1 = x[(n - 1) * st] - (d * x[0] + e * x[st] + a * x[(n - 3) * st]);
    x[(n - 2) * st] = om[0] * n2 + om[1] * n1;
    x[(n - 1) * st] = om[2] * n2 + om[3] * n1;
    double o2 = x[(n - 2) * st], o1 = x[(n - 1) * st];
    for (int i = 0; i < n - 2; ++i) x[i * st] = x[i * st] - (inv1[i] * o2 + inv2[i] * o1);
}

/* Periodic weighted window sum with the reference's modular indexing (serialCahnADI.c:478-622);
 * cube != 0 applies c^3 - c to every sample first. */
static double ch_window(const double* f, int n, int j, int i, const double* w, int V, int H, int off, int cube) {
    double sum = 0.0;
    for (int oj = 0; oj < V; ++oj) {
        int cj = j - off + oj;
        int row = (cj < 0) ? (cj + n) * n : (cj % n) * n;
        for (int oi = 0; oi < H; ++oi) {
            int ci = i - off + oi;
            int idx = (ci < 0) ? row + (ci + n) : row + (ci % n);
            double v = f[idx];
            sum += w[oj * H + oi] * (cube ? ((v * v * v) - v) : v);
        }
    }
    return sum;
}

struct ch_oracle_state {
    int n;
    double a, b, c, d, e;
    double *ds, *dl, *dg, *du, *dw, *inv1, *inv2, omega[4];
    double wl[25], wn[9];
    double *cOld, *cCurr, *cBar, *cHalf, *cNL, *tmp;
};

/* Set-up of serialCahnADI.c:761-1005 for an n x n periodic grid of side lx (D = 1, gamma = 0.01,
 * dt = 0.1 dx); c0 is both cOld and cCurr. */
struct ch_oracle_state* ch_oracle_create(int n, double lx, const double* c0) {
    struct ch_oracle_state* s = calloc(1, sizeof(*s));
    const double D = 1.0, gam = 0.01, dx = lx / n, dt = 0.1 * dx;
    const int m = n - 2;
    s->n = n;
    double sl = 2.0 * dt * D * gam / (3.0 * (dx * dx * dx * dx));
    s->a = sl; s->b = -4 * sl; s->c = 1 + 6 * sl; s->d = -4 * sl; s->e = sl;
    s->ds = malloc(sizeof(double) * m); s->dl = malloc(sizeof(double) * m); s->dg = malloc(sizeof(double) * m);
    s->du = malloc(sizeof(double) * m); s->dw = malloc(sizeof(double) * m);
    s->inv1 = malloc(sizeof(double) * m); s->inv2 = malloc(sizeof(double) * m);
    ch_set_lhs(s->ds, s->dl, s->dg, s->du, s->dw, s->a, s->b, s->c, s->d, s->e, m);
    ch_pent_factor(s->ds, s->dl, s->dg, s->du, s->dw, m);
    ch_find_omega(s->omega, s->inv1, s->inv2, s->a, s->b, s->c, s->d, s->e, m);
    static const double wl[25] = {0, 0, -1, 0, 0, 0, -2, 8, -2, 0, -1, 8, -20, 8, -1, 0, -2, 8, -2, 0, 0, 0, -1, 0, 0};
    static const double wn[9] = {0, 1, 0, 1, -4, 1, 0, 1, 0};
    const double snl = (dt / 3.0) * D * (2.0 / (dx * dx));
    for (int k = 0; k < 25; ++k) s->wl[k] = wl[k] * sl;
    for (int k = 0; k < 9; ++k) s->wn[k] = wn[k] * snl;
    size_t nn = (size_t)n * n;
    s->cOld = malloc(sizeof(double) * nn); s->cCurr = malloc(sizeof(double) * nn);
    s->cBar = malloc(sizeof(double) * nn); s->cHalf = malloc(sizeof(double) * nn);
    s->cNL = malloc(sizeof(double) * nn);
    memcpy(s->cOld, c0, sizeof(double) * nn);
    memcpy(s->cCurr, c0, sizeof(double) * nn);
    return s;
}

/* One step of serialCahnADI.c:1010-1047. The reference transposes the field between the two sweeps;
 * solving the y lines in place with stride n is the same arithmetic on the same values. */
void ch_oracle_step(struct ch_oracle_state* s, int steps) {
    const int n = s->n;
    const size_t nn = (size_t)n * n;
    for (int it = 0; it < steps; ++it) {
        for (size_t k = 0; k < nn; ++k) s->cBar[k] = 2.0 * s->cCurr[k] - s->cOld[k];
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                s->cHalf[(size_t)j * n + i] = ch_window(s->cBar, n, j, i, s->wl, 5, 5, 2, 0);
                s->cNL[(size_t)j * n + i] = ch_window(s->cCurr, n, j, i, s->wn, 3, 3, 1, 1);
            }
        for (size_t k = 0; k < nn; ++k) {
            s->cHalf[k] += -(2.0 / 3.0) * (s->cCurr[k] - s->cOld[k]) + s->cNL[k];
            s->cOld[k] = s->cCurr[k];
        }
        for (int j = 0; j < n; ++j)   /* x lines */
            ch_cyclic(s->ds, s->dl, s->dg, s->du, s->dw, s->inv1, s->inv2, s->omega, s->cHalf + (size_t)j * n, s->a,
                      s->b, s->d, s->e, n, 1);
        for (int i = 0; i < n; ++i)   /* y lines */
            ch_cyclic(s->ds, s->dl, s->dg, s->du, s->dw, s->inv1, s->inv2, s->omega, s->cHalf + i, s->a, s->b,
                      s->d, s->e, n, n);
        for (size_t k = 0; k < nn; ++k) s->cCurr[k] = s->cBar[k] + s->cHalf[k];
    }
}

void ch_oracle_get(const struct ch_oracle_state* s, double* c_curr, double* c_old) {
    size_t nn = (size_t)s->n * s->n;
    if (c_curr) memcpy(c_curr, s->cCurr, sizeof(double) * nn);
    if (c_old) memcpy(c_old, s->cOld, sizeof(double) * nn);
}

/* Solver tables (factored diagonals, border columns, omega) for n: 5*(n-2) + 2*(n-2) + 4 values. */
void ch_oracle_tables(const struct ch_oracle_state* s, double* out) {
    const int m = s->n - 2;
    memcpy(out, s->ds, sizeof(double) * m); memcpy(out + m, s->dl, sizeof(double) * m);
    memcpy(out + 2 * m, s->dg, sizeof(double) * m); memcpy(out + 3 * m, s->du, sizeof(double) * m);
    memcpy(out + 4 * m, s->dw, sizeof(double) * m); memcpy(out + 5 * m, s->inv1, sizeof(double) * m);
    memcpy(out + 6 * m, s->inv2, sizeof(double) * m); memcpy(out + 7 * m, s->omega, sizeof(double) * 4);
}

void ch_oracle_destroy(struct ch_oracle_state* s) {
    free(s->ds); free(s->dl); free(s->dg); free(s->du); free(s->dw); free(s->inv1); free(s->inv2);
    free(s->cOld); free(s->cCurr); free(s->cBar); free(s->cHalf); free(s->cNL);
    free(s);
}

/* Mass with a compensated (Kahan-Babuska-Neumaier) sum. */
double ch_oracle_mean(const double* c, long long count) {
    double s = 0.0, comp = 0.0;
    for (long long k = 0; k < count; ++k) {
        double t = s + c[k];
        if (fabs(s) >= fabs(c[k])) comp += (s - t) + c[k];
        else comp += (c[k] - t) + s;
        s = t;
    }
    return (s + comp) / (double)count;
}
