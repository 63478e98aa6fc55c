/* Force-included when compiling reference sources with CUDA 13 -- TEST INFRASTRUCTURE ONLY.
 * CUDA 13 removed the cudaMemPrefetchAsync(ptr, bytes, int device, stream) overload the reference
 * calls; this restores it on top of the cudaMemLocation form. */
#pragma once
#include <cuda_runtime.h>
static inline cudaError_t cudaMemPrefetchAsync(const void* p, size_t n, int dev, cudaStream_t s) {
    cudaMemLocation loc;
    loc.type = (dev == cudaCpuDeviceId) ? cudaMemLocationTypeHost : cudaMemLocationTypeDevice;
    loc.id = (dev == cudaCpuDeviceId) ? 0 : dev;
    return cudaMemPrefetchAsync(p, n, loc, 0, s);
}
