// A user program written against the reference's C++ API (cuSten.h), built with nvcc -rdc=true and
// linked against this library's static archive (libcuSten.a) -- the drop-in path of a reference user.
// It follows the pattern of the reference examples: managed memory, Create / Compute / Swap / Destroy,
// and a Fun variant whose device function is defined here, in the user's own translation unit.
//
// Usage: dropin_program <output prefix>. Writes <prefix>_<name>.bin (raw doubles, row-major) for the
// inputs and outputs that the test compares with the oracle.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "cuSten.h"

// A user device function with the reference's XY signature (2d_xy_p_fun_kernel.cu:51): the weighted
// sum over the H x V window, as an explicit FMA chain.
typedef double (*devArgXY)(double*, double*, int, int, int, int);
__device__ double user_window_sum(double* data, double* coe, int topLeft, int jump, int nxs, int nys) {
    double s = 0.0;
    int k = 0;
    for (int j = 0; j < nys; ++j)
        for (int i = 0; i < nxs; ++i) s = __fma_rn(coe[k++], data[topLeft + j * jump + i], s);
    return s;
}
__device__ devArgXY user_fun = user_window_sum;

static void save(const std::string& prefix, const char* name, const double* p, size_t n) {
    std::string path = prefix + "_" + name + ".bin";
    FILE* f = fopen(path.c_str(), "wb");
    if (!f || fwrite(p, sizeof(double), n, f) != n) {
        printf("cannot write %s\n", path.c_str());
        exit(1);
    }
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 2) {
        printf("usage: %s <output prefix>\n", argv[0]);
        return 2;
    }
    const std::string prefix = argv[1];
    const int nx = 256, ny = 128, numTiles = 2, BX = 32, BY = 8;
    const size_t n = (size_t)nx * ny;
    double *a, *b, *c, *w, *coe, *u, *v;
    cudaMallocManaged(&a, n * sizeof(double));
    cudaMallocManaged(&b, n * sizeof(double));
    cudaMallocManaged(&c, n * sizeof(double));
    cudaMallocManaged(&u, n * sizeof(double));
    cudaMallocManaged(&v, n * sizeof(double));
    cudaMallocManaged(&w, 9 * sizeof(double));
    cudaMallocManaged(&coe, 9 * sizeof(double));
    checkError("allocating managed memory");
    const double dx = 2 * M_PI / nx, dy = 2 * M_PI / ny;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            a[(size_t)j * nx + i] = sin(3 * i * dx) * cos(5 * j * dy);
            b[(size_t)j * nx + i] = 0.0;
            c[(size_t)j * nx + i] = 0.0;
            u[(size_t)j * nx + i] = cos(i * dx + 2 * j * dy);
            v[(size_t)j * nx + i] = sin(2 * i * dx - j * dy);
        }
    const double cross[9] = {1, 0, -1, 0, 0, 0, -1, 0, 1};   // the reference example's cross derivative
    for (int k = 0; k < 9; ++k) {
        w[k] = cross[k] / (4 * dx * dy);
        coe[k] = (k % 2 == 0 ? 0.5 : -0.25) + 0.125 * k;
    }
    save(prefix, "input", a, n);
    save(prefix, "u", u, n);
    save(prefix, "v", v, n);

    // 1. XY periodic, two Computes with a Swap between: b = D(a); a = D(b)
    cuSten_t xy;
    cuStenCreate2DXYp(&xy, 0, numTiles, nx, ny, BX, BY, b, a, w, 3, 1, 1, 3, 1, 1);
    cuStenCompute2DXYp(&xy, 0);
    cudaDeviceSynchronize();
    save(prefix, "xyp_1", b, n);
    cuStenSwap2DXYp(&xy, b);
    cuStenCompute2DXYp(&xy, 1);   // HOST offload
    cudaDeviceSynchronize();
    save(prefix, "xyp_2", a, n);
    cuStenDestroy2DXYp(&xy);

    // 2. XY non-periodic with the user's device function (indirect call across translation units)
    for (size_t i = 0; i < n; ++i) a[i] = sin(3 * (i % nx) * dx) * cos(5 * (i / nx) * dy);
    for (size_t i = 0; i < n; ++i) c[i] = -7.0;   // untouched points keep this
    double* func;
    cudaMemcpyFromSymbol(&func, user_fun, sizeof(devArgXY));
    cuSten_t fn;
    cuStenCreate2DXYnpFun(&fn, 0, numTiles, nx, ny, BX, BY, c, a, coe, 3, 1, 1, 3, 1, 1, func);
    cuStenCompute2DXYnpFun(&fn, 0);
    cudaDeviceSynchronize();
    save(prefix, "xynpfun", c, n);
    cuStenDestroy2DXYnpFun(&fn);

    // 3. X periodic through the reference's misspelt XpFun compute is not used here; X non-periodic
    //    weights, 5-point
    const double d2[5] = {-1.0 / 12, 16.0 / 12, -30.0 / 12, 16.0 / 12, -1.0 / 12};
    for (int k = 0; k < 5; ++k) w[k] = d2[k] / (dx * dx);
    for (size_t i = 0; i < n; ++i) b[i] = 3.0;
    cuSten_t x;
    cuStenCreate2DXnp(&x, 0, 1, nx, ny, BX, BY, b, a, w, 5, 2, 2);
    cuStenCompute2DXnp(&x, 0);
    cudaDeviceSynchronize();
    save(prefix, "xnp", b, n);
    cuStenDestroy2DXnp(&x);

    // 4. WENO advection, periodic
    cuSten_t we;
    cuStenCreate2DXYWENOADVp(&we, 0, numTiles, nx, ny, BX, BY, dx, dy, u, v, b, a);
    cuStenCompute2DXYWENOADVp(&we, 0);
    cudaDeviceSynchronize();
    save(prefix, "weno", b, n);
    cuStenDestroy2DXYWENOADVp(&we);

    checkError("running the drop-in program");
    printf("ok\n");
    return 0;
}
