// Self-test of the bounded mbarrier wait of the TMA-staged stencil kernels (stencil_tma.cuh).
//
// One CTA initialises an mbarrier that nothing will ever arrive on and waits on it with the same
// mbar_wait as the stencil kernels, with a short round limit. The wait must give up, the kernel must
// record kErrMbarrierTimeout in the device error flags and return, and the context must stay usable.
// No copy is in flight and no thread traps: this exercises the failure path the stencil kernels take
// when a tensor copy never completes, without making one fail.
#include <cuda_runtime.h>

#include "../../include/custen_gb300.h"
#include "cvt_int.cuh"
#include "stencil_tma.cuh"

namespace custen {
namespace {

__global__ void wait_expiry_kernel(long long limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const bool ok = threadIdx.x == 0 ? mbar_wait(&bar, 0, limit) : true;
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(&g_custen_device_error, kErrMbarrierTimeout);
}

}  // namespace
}  // namespace custen

// Runs the wait with `rounds` try_wait rounds (1 .. 2^22) and returns the device error flags seen
// afterwards in *flags (bit 0 expected); the flags are left set for the caller to read and clear with
// custen_device_error. Returns 0 when the kernel ran and returned.
extern "C" int custen_selftest_wait_expiry(long long rounds, unsigned int* flags) {
    if (rounds < 1 || rounds > custen::kWaitLimit || !flags) return 2;
    custen::wait_expiry_kernel<<<1, 32>>>(rounds);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(flags, custen::g_custen_device_error, sizeof(unsigned int));
    return e == cudaSuccess ? 0 : 1;
}

// Conversions on the integer pipes (cvt_int.cuh) against the hardware conversions: n doubles (random
// encodings, values near the float range's ends, exact halfway cases, zeros) through f64_to_f32_rn, and n
// floats (random encodings) through f32_to_f64. Counts the results whose encodings differ (NaNs compare
// equal to NaNs).
namespace custen {
namespace {

__device__ __forceinline__ uint64_t st_mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void conversion_check_kernel(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long local = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint64_t h = st_mix(seed ^ (i * 2 + 0)), g = st_mix(seed ^ (i * 2 + 1));
        uint64_t bits;
        switch (g & 7) {
        case 0: bits = h; break;                                              // any encoding
        case 1: bits = (h & 0x800fffffffffffffull) | ((uint64_t)(896 + (g >> 8) % 256) << 52); break;  // float range
        case 2: bits = (h & 0x800fffffe0000000ull) | 0x10000000ull | ((uint64_t)(1023 + (g >> 8) % 64 - 32) << 52); break;  // halfway
        case 3: bits = (h & 0x800fffffffffffffull) | ((uint64_t)(896 + (g >> 8) % 4) << 52); break;   // near 2^-126
        case 4: bits = (h & 0x800fffffffffffffull) | ((uint64_t)(1150 + (g >> 8) % 4) << 52); break;  // near 2^128
        case 5: bits = (h & 0x8000000000000000ull) | 0x37ffffffe0000000ull | ((g >> 8) & 0x1fffffffull); break;
        case 6: bits = h & 0x8000000000000000ull; break;                     // zeros
        default: bits = (h & 0x800fffffffffffffull) | ((uint64_t)(1023 + (g >> 8) % 16 - 8) << 52); break;
        }
        const double x = __longlong_as_double((long long)bits);
        const float want = __double2float_rn(x), got = f64_to_f32_rn(x);
        if (__float_as_uint(want) != __float_as_uint(got) && !(want != want && got != got)) ++local;
        const float y = __uint_as_float((uint32_t)(h >> 32));
        const double wy = (double)y, gy = f32_to_f64(y);
        if (__double_as_longlong(wy) != __double_as_longlong(gy) && !(wy != wy && gy != gy)) ++local;
    }
    if (local) atomicAdd(bad, local);
}

}  // namespace
}  // namespace custen

// Runs the conversion check on n values of each kind (seeded) and returns the mismatch count in *mismatches.
// Returns 0 when the kernel ran.
extern "C" int custen_selftest_conversions(unsigned long long n, unsigned long long seed,
                                           unsigned long long* mismatches) {
    if (!mismatches) return 2;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return 1;
    cudaError_t e = cudaMemset(d, 0, sizeof(*d));
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) {
        custen::conversion_check_kernel<<<sms * 8, 256>>>(n, seed, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof(*d), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : 1;
}
