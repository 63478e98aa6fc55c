// Self-test of the bounded mbarrier wait of the TMA-staged stencil kernels (stencil_tma.cuh).
//
// One CTA initialises an mbarrier that nothing will ever arrive on and waits on it with the same
// mbar_wait as the stencil kernels, with a short round limit. The wait must give up, the kernel must
// record kErrMbarrierTimeout in the device error flags and return, and the context must stay usable.
// No copy is in flight and no thread traps: this exercises the failure path the stencil kernels take
// when a tensor copy never completes, without making one fail.
#include <cuda_runtime.h>

#include "../../include/custen_gb300.h"
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
