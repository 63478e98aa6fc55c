// Peak FMA-rate probe (FP64 / FP32) used as the compute-roofline denominator by the benchmark: the
// FP64 stencils on GB300 are bound by the FP64 FMA pipe, whose rate is not in the measured HBM/GEMM
// peak table. Each thread runs 16 independent FMA chains, 16 CTAs of 256 threads per SM; the result is
// stored so nothing is elided.
#include <cuda_runtime.h>

#include "../../include/custen_gb300.h"

namespace custen {

template <typename T>
__global__ void __launch_bounds__(256) fma_rate_kernel(T* out, T a, T b, int iters) {
    T acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = T(threadIdx.x + c);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[c] = fma(acc[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 16; ++c) s += acc[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
static int run_probe(double* fma_per_s, int iters) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 16, threads = 256;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_rate_kernel<T><<<blocks, threads>>>(out, T(0.999999), T(1e-7), iters / 10 + 1);   // warm-up
    cudaEventRecord(e0);
    fma_rate_kernel<T><<<blocks, threads>>>(out, T(0.999999), T(1e-7), iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return 1;
    *fma_per_s = (double)blocks * threads * iters * 16.0 / (ms * 1e-3);
    return 0;
}

}  // namespace custen

extern "C" int custen_probe_fma_rate(int dtype, double* fma_per_s) {
    if (fma_per_s == nullptr) return 2;
    return dtype == CUSTEN_F64 ? custen::run_probe<double>(fma_per_s, 1000)
                               : custen::run_probe<float>(fma_per_s, 10000);
}
