// Routes a stencil launch to the kernel configuration a handle uses (stencil_configs.h).
#include <atomic>
#include <cstdio>

#include "stencil_configs.h"

namespace custen {

using LaunchFn = cudaError_t (*)(const StencilArgs&, cudaStream_t, int*);

#define CUSTEN_DECLARE_CFG(d, k) cudaError_t launch_cfg_##d##_##k(const StencilArgs&, cudaStream_t, int*);
CUSTEN_DECLARE_CFG(0, 0) CUSTEN_DECLARE_CFG(0, 1) CUSTEN_DECLARE_CFG(0, 2) CUSTEN_DECLARE_CFG(0, 3) CUSTEN_DECLARE_CFG(0, 4)
CUSTEN_DECLARE_CFG(0, 5)
CUSTEN_DECLARE_CFG(1, 0) CUSTEN_DECLARE_CFG(1, 1) CUSTEN_DECLARE_CFG(1, 2) CUSTEN_DECLARE_CFG(1, 3) CUSTEN_DECLARE_CFG(1, 4)
CUSTEN_DECLARE_CFG(1, 5)
#undef CUSTEN_DECLARE_CFG

// One entry per configuration of stencil_configs.h (the sizes are checked: a shorter list would leave
// null launchers).
static const LaunchFn kLaunchF64[] = {launch_cfg_0_0, launch_cfg_0_1, launch_cfg_0_2,
                                      launch_cfg_0_3, launch_cfg_0_4, launch_cfg_0_5};
static const LaunchFn kLaunchF32[] = {launch_cfg_1_0, launch_cfg_1_1, launch_cfg_1_2,
                                      launch_cfg_1_3, launch_cfg_1_4, launch_cfg_1_5};
static_assert(sizeof(kLaunchF64) / sizeof(LaunchFn) == kNumConfigs, "one FP64 launcher per configuration");
static_assert(sizeof(kLaunchF32) / sizeof(LaunchFn) == kNumConfigs, "one FP32 launcher per configuration");

static std::atomic<int> g_grid_cap{0};

int persistent_grid_cap() { return g_grid_cap.load(std::memory_order_relaxed); }

cudaError_t launch_stencil_cfg(const StencilArgs& a, int dtype, int cfg, cudaStream_t s, int* path) {
    if (cfg < 0 || cfg >= kNumConfigs) cfg = 0;
    return (dtype == DT_F64 ? kLaunchF64 : kLaunchF32)[cfg](a, s, path);
}

cudaError_t launch_stencil_f64(const StencilArgs& a, cudaStream_t s, int* path) {
    return launch_stencil_cfg(a, DT_F64, 0, s, path);
}

cudaError_t launch_stencil_f32(const StencilArgs& a, cudaStream_t s, int* path) {
    return launch_stencil_cfg(a, DT_F32, 0, s, path);
}

namespace {
struct ConfigNames {
    char n[2][kNumConfigs][48];
    ConfigNames() {
        for (int k = 0; k < kNumConfigs; ++k) {
            const StencilConfig& c64 = kConfigsF64[k];
            const StencilConfig& c32 = kConfigsF32[k];
            snprintf(n[0][k], sizeof(n[0][k]), "f64_tw%d_th%d_rpt%d_vec%d", c64.tw, c64.th, c64.rpt, c64.vec);
            snprintf(n[1][k], sizeof(n[1][k]), "f32_tw%d_th%d_rpt%d_vec%d", c32.tw, c32.th, c32.rpt, c32.vec);
        }
    }
};
}  // namespace

const char* config_name(int dtype, int cfg) {
    static const ConfigNames names;   // built once, thread-safely
    if (cfg < 0 || cfg >= kNumConfigs) return "?";
    return names.n[dtype == DT_F64 ? 0 : 1][cfg];
}

}  // namespace custen

extern "C" void custen_set_max_ctas(int max_ctas) { custen::g_grid_cap.store(max_ctas > 0 ? max_ctas : 0); }
