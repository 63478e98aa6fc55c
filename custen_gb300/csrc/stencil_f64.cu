// FP64 instantiation of the stencil kernels.
#include "stencil_launch.cuh"

namespace custen {

cudaError_t launch_stencil_f64(const StencilArgs& a, cudaStream_t s, int* path) {
    // 64 x 32 output tile, 2 columns x 4 rows per thread: 256 threads, 8 independent FMA chains each.
    cudaError_t e = launch_tma<double, 64, 32, 4, 3>(a, s);
    *path = 1;
    if (e != cudaErrorNotSupported) return e;
    *path = 0;
    return launch_ldg<double, 64, 32, 4>(a, s);
}

}  // namespace custen
