// FP64 <-> FP32 conversions on the integer pipes (sm_103a).
//
// On GB300 the F2F conversions between double and float issue to the FP64 pipe, about one conversion
// per FP64 operation slot. The FP32-stencil Cahn-Hilliard right-hand side converts every staged cCurr and
// cOld value to float and every h value back, 3.8 conversions per point: its FP64 pipe was busy with
// those alone. These functions give the same results with integer operations, from the IEEE 754
// binary64 / binary32 encodings:
//   f64_to_f32_rn: round to nearest, ties to even; the 52-bit significand keeps its top 23 bits and the
//   29 bits below decide the rounding (a carry out of the significand moves into the exponent, which is
//   the encoding's own carry). Zeros keep their sign. Values whose result is not a normal float (below
//   2^-126, overflowing, infinite or NaN) take the hardware conversion.
//   f32_to_f64: exact; the exponent is rebiased (+896) and the significand moved up 29 bits. Zeros keep
//   their sign; subnormal, infinite and NaN floats take the hardware conversion.
#pragma once

#include <cstdint>

namespace custen {

static __device__ __noinline__ float f64_to_f32_hw(double x) { return __double2float_rn(x); }
static __device__ __noinline__ double f32_to_f64_hw(float x) { return (double)x; }

__device__ __forceinline__ float f64_to_f32_rn(double x) {
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;    // float exponent field before rounding
    // 23-bit significand: bits 51..29 of the double's; rounding bits 28..0
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1fffffffu;
    const uint32_t half = 0x10000000u;
    const uint32_t up = (rest > half || (rest == half && (m & 1u))) ? 1u : 0u;
    const uint32_t bits = sign | (((uint32_t)e << 23) + m + up);   // a significand carry bumps the exponent
    const bool zero = ((hi & 0x7fffffffu) | lo) == 0;
    if (zero) return __uint_as_float(sign);
    const bool normal = e >= 1 && e <= 254 && ((bits & 0x7f800000u) != 0x7f800000u);
    return normal ? __uint_as_float(bits) : f64_to_f32_hw(x);
}

__device__ __forceinline__ double f32_to_f64(float x) {
    const uint32_t u = __float_as_uint(x);
    const uint32_t sign = u & 0x80000000u, ef = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    if ((u & 0x7fffffffu) == 0) return __longlong_as_double((long long)((uint64_t)sign << 32));
    if (ef == 0 || ef == 0xffu) return f32_to_f64_hw(x);
    const uint32_t hi = sign | ((ef + 896u) << 20) | (m >> 3), lo = m << 29;
    return __longlong_as_double((long long)(((uint64_t)hi << 32) | lo));
}

}  // namespace custen
