/* Harness around the reference serial Cahn-Hilliard ADI program -- TEST INFRASTRUCTURE ONLY.
 * Compiled by oracle/ref_build.py with the reference source #included from where it lies
 * (cuPentSpeedUp/serialCahnADITiming/serialCahnADI.c, its main renamed), so the reference's own
 * static functions run unchanged. ref_ch_run performs the set-up and time loop of the reference main
 * (serialCahnADI.c:761-1047) with n, the domain length, the step count and c0 as parameters instead of
 * argv / lx = 16 pi / T = 10 / rand(). */
#include SERIAL_CH_SOURCE

int ref_ch_run(int n, double lx, int steps, const double* c0, double* c_out, double* c_old_out) {
    double dCahn = 1.0, gammaCahn = 0.01;
    int nSolve = n - 2;
    double dx = lx / n;
    double dt = 0.1 * dx;
    double *cOld = malloc(sizeof(double) * n * n), *cCurr = malloc(sizeof(double) * n * n);
    double *cNonLinRHS = malloc(sizeof(double) * n * n), *cBar = malloc(sizeof(double) * n * n);
    double *cHalf = malloc(sizeof(double) * n * n);
    double *ds = malloc(sizeof(double) * nSolve), *dl = malloc(sizeof(double) * nSolve);
    double *diag = malloc(sizeof(double) * nSolve), *du = malloc(sizeof(double) * nSolve);
    double *dw = malloc(sizeof(double) * nSolve);
    double *omega = malloc(4 * sizeof(double)), *inv1 = malloc(sizeof(double) * nSolve);
    double *inv2 = malloc(sizeof(double) * nSolve);
    double *weightsLinRHS = malloc(25 * sizeof(double)), *weightsNonLinRHS = malloc(9 * sizeof(double));
    for (int i = 0; i < n * n; i++) { cOld[i] = c0[i]; cCurr[i] = c0[i]; }
    double simgaLin = 2.0 * dt * dCahn * gammaCahn / (3.0 * (dx * dx * dx * dx));
    double a = simgaLin, b = -4 * simgaLin, c = 1 + 6 * simgaLin, d = -4 * simgaLin, e = simgaLin;
    setLHS(ds, dl, diag, du, dw, a, b, c, d, e, nSolve);
    pentFactor(ds, dl, diag, du, dw, nSolve);
    findOmega(omega, inv1, inv2, a, b, c, d, e, nSolve);
    const double wl[25] = {0, 0, -1, 0, 0, 0, -2, 8, -2, 0, -1, 8, -20, 8, -1, 0, -2, 8, -2, 0, 0, 0, -1, 0, 0};
    for (int k = 0; k < 25; k++) weightsLinRHS[k] = wl[k] * simgaLin;
    double sigmaNonLin = (dt / 3.0) * dCahn * (2.0 / (dx * dx));
    const double wn[9] = {0, 1, 0, 1, -4, 1, 0, 1, 0};
    for (int k = 0; k < 9; k++) weightsNonLinRHS[k] = wn[k] * sigmaNonLin;
    for (int s = 0; s < steps; s++) {
        findCBar(cOld, cCurr, cBar, n);
        linearRHS(cBar, cHalf, weightsLinRHS, 5, 5, 2, 2, n);
        nonlinearRHS(cCurr, cNonLinRHS, weightsNonLinRHS, 3, 3, 1, 1, n);
        findRHS(cOld, cCurr, cHalf, cNonLinRHS, n);
        for (int i = 0; i < n; i++) cyclicInv(ds, dl, diag, du, dw, inv1, inv2, omega, &cHalf[i * n], a, b, d, e, nSolve, n);
        transpose(cHalf, cCurr, n);
        for (int i = 0; i < n; i++) cyclicInv(ds, dl, diag, du, dw, inv1, inv2, omega, &cCurr[i * n], a, b, d, e, nSolve, n);
        transpose(cCurr, cHalf, n);
        findNew(cCurr, cBar, cHalf, n);
    }
    for (int i = 0; i < n * n; i++) { c_out[i] = cCurr[i]; if (c_old_out) c_old_out[i] = cOld[i]; }
    free(cOld); free(cCurr); free(cNonLinRHS); free(cBar); free(cHalf); free(ds); free(dl); free(diag); free(du);
    free(dw); free(omega); free(inv1); free(inv2); free(weightsLinRHS); free(weightsNonLinRHS);
    return 0;
}
