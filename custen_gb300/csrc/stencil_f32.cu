// FP32 instantiation of the stencil kernels.
#include "stencil_launch.cuh"

namespace custen {

cudaError_t launch_stencil_f32(const StencilArgs& a, cudaStream_t s, int* path) {
    // 128 x 32 output tile, 4 columns x 4 rows per thread: 256 threads.
    cudaError_t e = launch_tma<float, 128, 32, 4, 3>(a, s);
    *path = 1;
    if (e != cudaErrorNotSupported) return e;
    *path = 0;
    return launch_ldg<float, 128, 32, 4>(a, s);
}

}  // namespace custen
