// Device functions shipped for the Fun (device-function-pointer) variants, as templates over the
// element type. Shared by the library (builtin_funs.cu) and by the test-only wrapper that compiles
// the reference kernels (oracle/ref_kernels.cu), so both call identical user functions.
//
// They have the reference's function-pointer signatures (cuSten/src/kernels/2d_x_p_fun_kernel.cu:47,
// 2d_y_p_fun_kernel.cu:49, 2d_xy_p_fun_kernel.cu:51) and compute the user functions of the reference
// examples and of the Cahn-Hilliard solver. Every operation is an explicit round-to-nearest intrinsic
// in a fixed order, so a host restatement with std::fma reproduces them bit for bit.
#pragma once

namespace custen_funs {

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

}  // namespace custen_funs
