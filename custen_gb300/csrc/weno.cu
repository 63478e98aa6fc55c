// WENO5 advection stencil, periodic in x and y (the thirteenth cuSten operator,
// cuSten/src/kernels/2d_xyADVWENO_p_kernel.cu), for sm_103a.
//
// out[y][x] = u[y][x] * Fx + v[y][x] * Fy, where Fx (Fy) is the fifth-order WENO reconstruction of the
// upwind one-sided differences D[i] = (in[i] - in[i-1]) * coeDx along x (along y with coeDy): for u > 0
// the differences at x-2 .. x+2, otherwise those at x+3 .. x-1 in reverse order (the reference's
// upwind selection, 2d_xyADVWENO_p_kernel.cu:286-348 and :352-414).
//
// GB300 shape: about 200 FP64 operations per point (eight correctly rounded divisions among them)
// against 32 bytes of compulsory traffic, so the FP64 pipe bounds this operator by a wide margin.
// The kernel therefore spends no FP64 work twice: a 64 x 32 tile with its 3-point periodic halo is
// staged once, and the x and y differences are formed once per tile into shared memory (the
// reference forms five differences per point and direction). The reconstruction keeps the reference's
// operation order, including its single-precision powf on the smoothness terms, so that results are
// bit-identical to the reference's kernel on the same GPU.
#include <cuda_runtime.h>

#include <atomic>

#include "checked.cuh"
#include "custen_internal.h"

namespace custen {
namespace {

constexpr int kWenoTW = 64;                 // tile columns (one per thread column)
constexpr int kWenoTH = 32;                 // tile rows
constexpr int kWenoHalo = 3;                // i-3 .. i+3
constexpr int kWenoThreads = 256;           // 64 columns x 4 thread rows
constexpr int kWenoSW = kWenoTW + 2 * kWenoHalo;   // 70 staged columns
constexpr int kWenoSH = kWenoTH + 2 * kWenoHalo;   // 38 staged rows
constexpr int kWenoDXW = kWenoTW + 5;       // x differences at columns x0-2 .. x0+TW+2
constexpr int kWenoDYH = kWenoTH + 5;       // y differences at rows y0-2 .. y0+TH+2
constexpr size_t kWenoSmem = sizeof(double) * ((size_t)kWenoSH * kWenoSW + (size_t)kWenoTH * kWenoDXW +
                                               (size_t)kWenoDYH * kWenoTW);

// Coefficients of the reconstruction. They are read from device memory into registers once per
// thread (WenoCoeffs::load): an FP64 FMA or add with a literal or kernel-parameter operand issues about
// 19% slower on GB300 than one whose operands are all registers (507 against 602-628 G FMA/s
// measured). The values are the literals of the reference's expressions, so every result is the same.
__device__ double g_weno_coeffs[15] = {1.0 / 3.0, 7.0 / 6.0, 11.0 / 6.0, 1.0 / 6.0, 5.0 / 6.0,
                                       2.0,       4.0,       3.0,        13.0 / 12.0, 0.25,
                                       1e-06,     0.1,       0.6,        0.3,         0.0};

struct WenoCoeffs {
    double third, seven_sixths, eleven_sixths, sixth, five_sixths, two, four, three, thirteen_twelfths,
        quarter, eps, g1, g2, g3;
    __device__ __forceinline__ void load() {
        const volatile double* k = g_weno_coeffs;
        third = k[0]; seven_sixths = k[1]; eleven_sixths = k[2]; sixth = k[3]; five_sixths = k[4];
        two = k[5]; four = k[6]; three = k[7]; thirteen_twelfths = k[8]; quarter = k[9];
        eps = k[10]; g1 = k[11]; g2 = k[12]; g3 = k[13];
    }
};

// Fifth-order WENO reconstruction (Jiang & Shu 1996, in the notation of Osher & Fedkiw, "Level Set
// Methods and Dynamic Implicit Surfaces", 3.4) from five consecutive differences a..e. The three
// candidate stencils, the smoothness indicators and the nonlinear weights are evaluated in the order
// of the reference's wenoSten (2d_xyADVWENO_p_kernel.cu:52-88): same expressions, same contraction,
// and the smoothness squares and the squared (indicator + 1e-6) taken by powf in single precision.
__device__ __forceinline__ double weno5(const WenoCoeffs& k, double a, double b, double c, double d, double e) {
    const double q1 = k.third * a - k.seven_sixths * b + k.eleven_sixths * c;
    const double q2 = -k.sixth * b + k.five_sixths * c + k.third * d;
    const double q3 = k.third * c + k.five_sixths * d - k.sixth * e;

    const double is1 = k.thirteen_twelfths * powf((float)(a - k.two * b + c), 2.0f) +
                       k.quarter * powf((float)(a - k.four * b + k.three * c), 2.0f);
    const double is2 = k.thirteen_twelfths * powf((float)(b - k.two * c + d), 2.0f) +
                       k.quarter * powf((float)(b - d), 2.0f);
    const double is3 = k.thirteen_twelfths * powf((float)(c - k.two * d + e), 2.0f) +
                       k.quarter * powf((float)(k.three * c - k.four * d + e), 2.0f);

    const double g1 = k.g1 / powf((float)(is1 + k.eps), 2.0f);
    const double g2 = k.g2 / powf((float)(is2 + k.eps), 2.0f);
    const double g3 = k.g3 / powf((float)(is3 + k.eps), 2.0f);
    const double norm = 1.0 / (g1 + g2 + g3);
    const double w1 = g1 * norm, w2 = g2 * norm, w3 = g3 * norm;
    return q1 * w1 + q2 * w2 + q3 * w3;
}

__device__ __forceinline__ int wrap_col(int c, int nx) {
    c %= nx;
    return c < 0 ? c + nx : c;
}

// One CTA per 64 x 32 tile of the launch's rows. Rows above / below the launch come from the T = 3
// halo rows at `top` / `bot` (the handle's boundaryTop/boundaryBottom of the tile, periodic); columns
// wrap around the field.
__global__ void __launch_bounds__(kWenoThreads, 2) weno_adv_kernel(double* __restrict__ out,
                                                                   const double* __restrict__ in,
                                                                   const double* __restrict__ uvel,
                                                                   const double* __restrict__ vvel,
                                                                   const double* __restrict__ top,
                                                                   const double* __restrict__ bot, double cdx,
                                                                   double cdy, int nx, int rows) {
    extern __shared__ __align__(16) double wsm[];
    double* tile = wsm;                                   // [SH][SW]
    double* dxs = tile + kWenoSH * kWenoSW;               // [TH][DXW]
    double* dys = dxs + kWenoTH * kWenoDXW;               // [DYH][TW]
    const int x0 = blockIdx.x * kWenoTW, y0 = blockIdx.y * kWenoTH;
    const int tid = threadIdx.x;

    // stage the tile and its halo: staged (r, c) is field row y0-3+r, column x0-3+c (wrapped)
    for (int e = tid; e < kWenoSH * kWenoSW; e += kWenoThreads) {
        const int r = e / kWenoSW, c = e - r * kWenoSW;
        const int gy = y0 - kWenoHalo + r;
        const int gx = wrap_col(x0 - kWenoHalo + c, nx);
        double val = 0.0;
        if (gy < 0) val = top[(size_t)(gy + kWenoHalo) * nx + gx];
        else if (gy < rows) val = in[(size_t)gy * nx + gx];
        else if (gy < rows + kWenoHalo) val = bot[(size_t)(gy - rows) * nx + gx];
        tile[e] = val;
    }
    __syncthreads();
    // differences, each formed once: D(i) = (f[i] - f[i-1]) * coe (2d_xyADVWENO_p_kernel.cu:290-309)
    for (int e = tid; e < kWenoTH * kWenoDXW; e += kWenoThreads) {
        const int r = e / kWenoDXW, c = e - r * kWenoDXW;
        const double* row = tile + (r + kWenoHalo) * kWenoSW;
        dxs[e] = (row[c + 1] - row[c]) * cdx;
    }
    for (int e = tid; e < kWenoDYH * kWenoTW; e += kWenoThreads) {
        const int r = e / kWenoTW, c = e - r * kWenoTW;
        dys[e] = (tile[(r + 1) * kWenoSW + c + kWenoHalo] - tile[r * kWenoSW + c + kWenoHalo]) * cdy;
    }
    __syncthreads();

    const int tx = tid % kWenoTW;
    const int x = x0 + tx;
    if (x >= nx) return;
    WenoCoeffs k;
    k.load();
    for (int ty = tid / kWenoTW; ty < kWenoTH; ty += kWenoThreads / kWenoTW) {
        const int y = y0 + ty;
        if (y >= rows) break;
        const size_t q = (size_t)y * nx + x;
        const double uu = uvel[q], vv = vvel[q];
        // Upwind side: the five differences are selected first and reconstructed once (two calls in a
        // conditional expression would let the compiler evaluate both and double the FP64 work).
        if (!span_ok((long long)ty * kWenoDXW + tx, 6, (long long)kWenoTH * kWenoDXW) ||
            !span_ok((long long)ty * kWenoTW + tx, 5 * kWenoTW + 1, (long long)kWenoDYH * kWenoTW) ||
            !in_bounds((long long)q, 0, (long long)rows * nx))
            continue;
        const double* dr = dxs + ty * kWenoDXW + tx;      // dr[k] = D at column x - 2 + k
        const bool ux = uu > 0.0;
        const double fx = weno5(k, ux ? dr[0] : dr[5], ux ? dr[1] : dr[4], dr[2 + !ux], ux ? dr[3] : dr[2],
                                ux ? dr[4] : dr[1]);
        const double* dc = dys + ty * kWenoTW + tx;       // dc[k * TW] = D at row y - 2 + k
        const bool vy = vv > 0.0;
        const double fy = weno5(k, vy ? dc[0] : dc[5 * kWenoTW], vy ? dc[kWenoTW] : dc[4 * kWenoTW],
                                dc[(2 + !vy) * kWenoTW], vy ? dc[3 * kWenoTW] : dc[2 * kWenoTW],
                                vy ? dc[4 * kWenoTW] : dc[kWenoTW]);
        // (2d_xyADVWENO_p_kernel.cu:424)
        out[q] = uu * fx + vv * fy;
    }
}

}  // namespace

cudaError_t launch_weno_adv(const StencilArgs& a, cudaStream_t s) {
    // setting the attribute is idempotent: threads that race here both set it
    static std::atomic<bool> attr_set[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64 && !attr_set[dev].load(std::memory_order_acquire)) {
        e = cudaFuncSetAttribute(weno_adv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWenoSmem);
        if (e != cudaSuccess) return e;
        attr_set[dev].store(true, std::memory_order_release);
    }
    if (a.rows <= 0 || a.nx <= 0) return cudaSuccess;
    dim3 grid((a.nx + kWenoTW - 1) / kWenoTW, (a.rows + kWenoTH - 1) / kWenoTH);
    weno_adv_kernel<<<grid, kWenoThreads, kWenoSmem, s>>>(
        static_cast<double*>(a.out), static_cast<const double*>(a.in), static_cast<const double*>(a.u),
        static_cast<const double*>(a.v), static_cast<const double*>(a.top), static_cast<const double*>(a.bot),
        a.cdx, a.cdy, a.nx, a.rows);
    return cudaGetLastError();
}

}  // namespace custen
