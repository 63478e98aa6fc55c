// Tile configurations of the stencil kernels, the autotuner's search space (per element type).
//
// A configuration fixes the output tile (tw x th points per CTA), the rows each thread produces (rpt,
// the depth of its register window) and the vector width (vec adjacent outputs per thread, one
// vec-wide load / store): the CTA has (tw / vec) x (th / rpt) threads, which is the role of the
// reference's BLOCK_X x BLOCK_Y. Every configuration computes each point with the same FMA chain, so
// the choice changes time, never results. Entry 0 is the default.
//
// stencil_cfg.cu is compiled once per entry (CUSTEN_CFG_DTYPE, CUSTEN_CFG_INDEX); stencil_dispatch.cu
// routes a launch to the entry a handle uses.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "custen_internal.h"

namespace custen {

struct StencilConfig {
    int tw, th, rpt, vec;
};

constexpr int kNumConfigs = 6;
constexpr StencilConfig kConfigsF64[kNumConfigs] = {
    {64, 32, 4, 2},    // 32 x 8 threads, 2 x 4 outputs each (16-byte vectors)
    {32, 32, 4, 2},    // 16 x 8: twice the tiles, for small fields
    {64, 16, 2, 2},    // 32 x 8, shallow register window
    {64, 32, 4, 1},    // 64 x 8, 8-byte accesses
    {64, 64, 8, 2},    // 32 x 8, deep register window
    {32, 16, 2, 2},    // 16 x 8: four times the tiles, for the smallest fields
};
constexpr StencilConfig kConfigsF32[kNumConfigs] = {
    {128, 32, 4, 4},   // 32 x 8 threads, 4 x 4 outputs each (16-byte vectors)
    {64, 32, 4, 4},    // 16 x 8
    {128, 16, 2, 4},   // 32 x 8, shallow register window
    {128, 32, 4, 2},   // 64 x 8, 8-byte accesses
    {128, 64, 8, 4},   // 32 x 8, deep register window
    {64, 16, 2, 4},    // 16 x 8: four times the tiles, for the smallest fields
};

// One launch with configuration `cfg` (0 .. kNumConfigs-1) of element type `dtype`; *path = 1 when
// the TMA-staged kernel ran, 0 for the plain-load kernel.
cudaError_t launch_stencil_cfg(const StencilArgs& a, int dtype, int cfg, cudaStream_t s, int* path);

// Upper bound on the CTAs of a persistent stencil launch (0: none, the default). Lowering it makes each
// CTA walk more tiles through its shared-memory ring, so that small fields exercise stage reuse.
int persistent_grid_cap();

// "f64_tw64_th32_rpt4_vec2" and the like.
const char* config_name(int dtype, int cfg);

// Autotuner (autotune.cu): the configuration for a device-resident launch -- cached, tuned, or the
// default -- and its settings.
int choose_config(const StencilArgs& a, int dtype, cudaStream_t s, bool force, int reps);
void set_autotune_mode(int mode);
void set_tune_cache(const char* path);
std::string tune_cache_path();

}  // namespace custen
