// One entry of the stencil configuration table (stencil_configs.h), selected at compile time by
// CUSTEN_CFG_DTYPE (0 FP64, 1 FP32) and CUSTEN_CFG_INDEX: the TMA-staged kernels of every mode and
// the plain-load fallback for that tile shape. The build compiles this file once per entry.
#include "stencil_configs.h"
#include "stencil_launch.cuh"

#ifndef CUSTEN_CFG_DTYPE
#error "CUSTEN_CFG_DTYPE must be defined (0 FP64, 1 FP32)"
#endif
#ifndef CUSTEN_CFG_INDEX
#error "CUSTEN_CFG_INDEX must be defined"
#endif

#define CUSTEN_CFG_FN_(d, k) launch_cfg_##d##_##k
#define CUSTEN_CFG_FN(d, k) CUSTEN_CFG_FN_(d, k)

namespace custen {

#if CUSTEN_CFG_DTYPE == 0
using CfgT = double;
constexpr StencilConfig kCfg = kConfigsF64[CUSTEN_CFG_INDEX];
#else
using CfgT = float;
constexpr StencilConfig kCfg = kConfigsF32[CUSTEN_CFG_INDEX];
#endif

cudaError_t CUSTEN_CFG_FN(CUSTEN_CFG_DTYPE, CUSTEN_CFG_INDEX)(const StencilArgs& a, cudaStream_t s, int* path) {
    cudaError_t e = launch_tma<CfgT, kCfg.tw, kCfg.th, kCfg.rpt, kCfg.vec, 3>(a, s);
    *path = 1;
    if (e != cudaErrorNotSupported) return e;
    *path = 0;
    return launch_ldg<CfgT, kCfg.tw, kCfg.th, kCfg.rpt, kCfg.vec>(a, s);
}

}  // namespace custen
