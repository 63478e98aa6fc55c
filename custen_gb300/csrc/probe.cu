// Peak FMA-rate probe (FP64 / FP32) used as the compute-roofline denominator by the benchmark: the
// FP64 stencils on GB300 are bound by the FP64 FMA pipe, whose rate is not in the measured HBM/GEMM
// peak table. Each thread runs independent FMA chains, 8 CTAs of 256 threads per SM, for about 60 ms.
// The multiplier and addend are loaded from device memory so that every FMA reads register operands:
// with them passed as kernel parameters (constant-bank operands) the FP64 rate measured 506 G FMA/s
// against 600-628 G FMA/s with register operands, where 628 is 2.0 FMA per clock per SM at 2.07 GHz.
// Two chain counts are timed and the faster is reported. The results are stored so nothing is elided.
#include <cuda_runtime.h>

#include "../../include/custen_gb300.h"

namespace custen {

template <typename T, int CH>
__global__ void __launch_bounds__(256) fma_rate_kernel(T* out, const T* ab, int iters) {
    const T a = ab[0], b = ab[1];
    T acc[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) acc[c] = T(threadIdx.x + c);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CH; ++c) acc[c] = fma(acc[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CH; ++c) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T, int CH>
static float time_kernel(T* out, const T* ab, int blocks, int iters) {
    fma_rate_kernel<T, CH><<<blocks, 256>>>(out, ab, iters / 10 + 1);   // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    fma_rate_kernel<T, CH><<<blocks, 256>>>(out, ab, iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err == cudaSuccess ? ms : -1.f;
}

template <typename T>
static int run_probe(double* fma_per_s, int iters16) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * (blocks * threads + 2)) != cudaSuccess) return 1;
    T* ab = out + blocks * threads;
    const T hab[2] = {T(0.999999), T(1e-7)};
    if (cudaMemcpy(ab, hab, sizeof(hab), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(out);
        return 1;
    }
    const float ms16 = time_kernel<T, 16>(out, ab, blocks, iters16);
    const float ms8 = time_kernel<T, 8>(out, ab, blocks, 2 * iters16);   // same FMA count
    cudaFree(out);
    if (ms16 <= 0.f || ms8 <= 0.f) return 1;
    const float ms = ms16 < ms8 ? ms16 : ms8;
    *fma_per_s = (double)blocks * threads * iters16 * 16.0 / (ms * 1e-3);
    return 0;
}

}  // namespace custen

extern "C" int custen_probe_fma_rate(int dtype, double* fma_per_s) {
    if (fma_per_s == nullptr) return 2;
    return dtype == CUSTEN_F64 ? custen::run_probe<double>(fma_per_s, 8000)
                               : custen::run_probe<float>(fma_per_s, 400000);
}
