// Device functions shipped for the Fun (device-function-pointer) variants.
//
// They have the reference's function-pointer signatures (cuSten/src/kernels/2d_x_p_fun_kernel.cu:47,
// 2d_y_p_fun_kernel.cu:49, 2d_xy_p_fun_kernel.cu:51) and compute the user functions of the reference
// examples and of the Cahn-Hilliard solver. Every operation is an explicit round-to-nearest intrinsic
// in a fixed order, so a host restatement with std::fma reproduces them bit for bit.
#include <cuda_runtime.h>

#include "../../include/custen_gb300.h"

namespace custen {
namespace {

template <typename T> __device__ __forceinline__ T fma_rn(T a, T b, T c);
template <> __device__ __forceinline__ double fma_rn<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <> __device__ __forceinline__ float fma_rn<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <typename T> __device__ __forceinline__ T mul_rn(T a, T b);
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <typename T> __device__ __forceinline__ T add_rn(T a, T b);
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

// c^3 - c as fma(c*c, c, -c)
template <typename T> __device__ __forceinline__ T cube_minus(T c) { return fma_rn<T>(mul_rn<T>(c, c), c, -c); }

// id 0: examples/src/2d_x_np_fun.cu:49-51, (d[l-1] - 2 d[l] + d[l+1]) * coe[0]
template <typename T> __device__ T x_second_diff(T* d, T* coe, int l) {
    T t = fma_rn<T>(T(-2), d[l], d[l - 1]);
    t = add_rn<T>(t, d[l + 1]);
    return mul_rn<T>(t, coe[0]);
}
// id 1: sum_k coe[k] (d^3 - d) over l-2..l+2
template <typename T> __device__ T x_cube_lap5(T* d, T* coe, int l) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 5; ++k) s = fma_rn<T>(coe[k], cube_minus<T>(d[l - 2 + k]), s);
    return s;
}
// id 2: examples/src/2d_y_p_fun.cu:49-60, 9-point along y
template <typename T> __device__ T y_central9(T* d, T* coe, int l, int jump) {
    T s = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) s = fma_rn<T>(coe[i], d[(l - 4 * jump) + i * jump], s);
    return s;
}
// id 3: sum_k coe[k] (d^3 - d) over rows l-2..l+2
template <typename T> __device__ T y_cube_lap5(T* d, T* coe, int l, int jump) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 5; ++k) s = fma_rn<T>(coe[k], cube_minus<T>(d[l + (k - 2) * jump]), s);
    return s;
}
// id 4: examples/src/2d_xy_p_fun.cu:58-80, weighted sum over the H x V window
template <typename T> __device__ T xy_weighted(T* d, T* coe, int tl, int jump, int nxs, int nys) {
    T s = T(0);
    int count = 0;
    for (int j = 0; j < nys; ++j)
        for (int i = 0; i < nxs; ++i) s = fma_rn<T>(coe[count++], d[tl + j * jump + i], s);
    return s;
}
// id 5: cuPentCahnADI/src/cuPentCahnADI.cu:164-190 (nonLinRHS), sum coe * (c^3 - c) over the window
template <typename T> __device__ T xy_cube(T* d, T* coe, int tl, int jump, int nxs, int nys) {
    T s = T(0);
    int count = 0;
    for (int j = 0; j < nys; ++j)
        for (int i = 0; i < nxs; ++i) s = fma_rn<T>(coe[count++], cube_minus<T>(d[tl + j * jump + i]), s);
    return s;
}

typedef double (*FxD)(double*, double*, int);
typedef double (*FyD)(double*, double*, int, int);
typedef double (*FxyD)(double*, double*, int, int, int, int);
typedef float (*FxF)(float*, float*, int);
typedef float (*FyF)(float*, float*, int, int);
typedef float (*FxyF)(float*, float*, int, int, int, int);

__device__ FxD g_fun_d0 = x_second_diff<double>;
__device__ FxD g_fun_d1 = x_cube_lap5<double>;
__device__ FyD g_fun_d2 = y_central9<double>;
__device__ FyD g_fun_d3 = y_cube_lap5<double>;
__device__ FxyD g_fun_d4 = xy_weighted<double>;
__device__ FxyD g_fun_d5 = xy_cube<double>;
__device__ FxF g_fun_f0 = x_second_diff<float>;
__device__ FxF g_fun_f1 = x_cube_lap5<float>;
__device__ FyF g_fun_f2 = y_central9<float>;
__device__ FyF g_fun_f3 = y_cube_lap5<float>;
__device__ FxyF g_fun_f4 = xy_weighted<float>;
__device__ FxyF g_fun_f5 = xy_cube<float>;

}  // namespace
}  // namespace custen

extern "C" int custen_builtin_function(int id, int dtype, void** func) {
    using namespace custen;
    if (func == nullptr) return 2;
    cudaError_t e = cudaErrorInvalidValue;
    void* p = nullptr;
    if (dtype == CUSTEN_F64) {
        switch (id) {
        case 0: e = cudaMemcpyFromSymbol(&p, g_fun_d0, sizeof(void*)); break;
        case 1: e = cudaMemcpyFromSymbol(&p, g_fun_d1, sizeof(void*)); break;
        case 2: e = cudaMemcpyFromSymbol(&p, g_fun_d2, sizeof(void*)); break;
        case 3: e = cudaMemcpyFromSymbol(&p, g_fun_d3, sizeof(void*)); break;
        case 4: e = cudaMemcpyFromSymbol(&p, g_fun_d4, sizeof(void*)); break;
        case 5: e = cudaMemcpyFromSymbol(&p, g_fun_d5, sizeof(void*)); break;
        default: return 2;
        }
    } else if (dtype == CUSTEN_F32) {
        switch (id) {
        case 0: e = cudaMemcpyFromSymbol(&p, g_fun_f0, sizeof(void*)); break;
        case 1: e = cudaMemcpyFromSymbol(&p, g_fun_f1, sizeof(void*)); break;
        case 2: e = cudaMemcpyFromSymbol(&p, g_fun_f2, sizeof(void*)); break;
        case 3: e = cudaMemcpyFromSymbol(&p, g_fun_f3, sizeof(void*)); break;
        case 4: e = cudaMemcpyFromSymbol(&p, g_fun_f4, sizeof(void*)); break;
        case 5: e = cudaMemcpyFromSymbol(&p, g_fun_f5, sizeof(void*)); break;
        default: return 2;
        }
    } else {
        return 2;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    *func = p;
    return 0;
}
