// Device-function pointers of the shipped Fun functions (builtin_funs.cuh) and their C-ABI lookup.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "builtin_funs.cuh"

#include "../../include/custen_gb300.h"

namespace custen {
namespace {

using namespace custen_funs;

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

// Which shipped function `f` is on the current device (0..5), or -1. The twelve addresses are read once
// per device.
extern "C" int custen_builtin_fun_id(const void* f, int dtype) {
    // filled once per device under the mutex; the flag publishes the filled table to other threads
    static void* cache[64][2][6];
    static std::atomic<bool> ready[64] = {};
    static std::mutex mu;
    int dev = 0;
    if (f == nullptr || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    if (!ready[dev].load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> lock(mu);
        if (!ready[dev].load(std::memory_order_relaxed)) {
            for (int t = 0; t < 2; ++t)
                for (int id = 0; id < 6; ++id)
                    if (custen_builtin_function(id, t == 0 ? CUSTEN_F64 : CUSTEN_F32, &cache[dev][t][id]) != 0)
                        return -1;
            ready[dev].store(true, std::memory_order_release);
        }
    }
    const int t = dtype == CUSTEN_F64 ? 0 : 1;
    for (int id = 0; id < 6; ++id)
        if (cache[dev][t][id] == f) return id;
    return -1;
}
