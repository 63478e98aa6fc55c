// Kernel entry and launcher template for the shared-memory tiled stencil (see stencil_kernel.cuh).
#pragma once

#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "stencil_configs.h"
#include "stencil_kernel.cuh"
#include "stencil_tma.cuh"

namespace custen {

// Plain-load staged kernel: handles every geometry (odd widths, unaligned rows, any halo).
template <typename T, int TW, int TH, int RPT, int VEC>
__global__ void __launch_bounds__((TW / VEC) * (TH / RPT), min_blocks_for((TW / VEC) * (TH / RPT), true))
stencil_ldg_kernel(const __grid_constant__ StencilArgs a) {
    constexpr int NTX = TW / VEC;
    constexpr int NT = NTX * (TH / RPT);
    extern __shared__ __align__(16) unsigned char smem[];
    TileGeom<T, TW, TH> g(a);
    T* tile = reinterpret_cast<T*>(smem);
    T* coef_s = reinterpret_cast<T*>(smem + g.coef_off(a));
    int* list_off = reinterpret_cast<int*>(smem + g.list_off(a));
    T* list_w = reinterpret_cast<T*>(smem + g.listw_off(a));
    const int tid = threadIdx.x + threadIdx.y * NTX;
    const bool is_fun = variant_is_fun(a.variant) && !a.pre;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    stage_tile_ldg<T, TW, TH, NT, VEC>(a, tile, g, x0, y0, tid);
    const int nlist = stage_coefficients<T, NT>(a, coef_s, list_off, list_w, g.SW, tid, is_fun);  // syncs
    if (a.pre) {
        apply_cube<T, NT>(tile, g.SR * g.SW, tid);
        __syncthreads();
    }
    const bool all_write = tile_all_write(a, x0, x0 + TW, a.row0 + y0, a.row0 + y0 + TH);
    compute_and_store<T, TW, TH, RPT, VEC>(a, tile, coef_s, list_off, list_w, nlist, g, x0, y0, threadIdx.x,
                                           threadIdx.y, is_fun, all_write);
}

// Largest dynamic shared memory a block may opt in to on the current device.
inline int smem_optin_limit() {
    static std::atomic<int> cached[64] = {};   // threads that race store the same value
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64) {
        const int c = cached[dev].load(std::memory_order_relaxed);
        if (c) return c;
    }
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) v = 48 * 1024;
    if (dev >= 0 && dev < 64) cached[dev].store(v, std::memory_order_relaxed);
    return v;
}

template <typename Kernel>
inline cudaError_t ensure_smem(Kernel k, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    if (smem > (size_t)smem_optin_limit()) return cudaErrorInvalidConfiguration;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename T, int TW, int TH, int RPT, int VEC>
cudaError_t launch_ldg(const StencilArgs& a, cudaStream_t s) {
    TileGeom<T, TW, TH> g(a);
    const size_t smem = g.total_bytes(a);
    cudaError_t e = ensure_smem(stencil_ldg_kernel<T, TW, TH, RPT, VEC>, smem);
    if (e != cudaSuccess) return e;
    dim3 block(TW / VEC, TH / RPT);
    dim3 grid((a.nx + TW - 1) / TW, (a.rows + TH - 1) / TH);
    stencil_ldg_kernel<T, TW, TH, RPT, VEC><<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link-time libcuda dependency).
// Looked up once (a function-local static: initialised once even when host threads race).
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
        return nullptr;
    }();
    return fn;
}

template <typename T>
inline bool encode_rows_map(CUtensorMap* m, const void* base, int nx, int rows, int box_w, int box_h) {
    auto enc = tensor_map_encoder();
    if (!enc || base == nullptr || rows < 1 || box_h < 1) return false;
    cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)nx * sizeof(T)};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                     const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

inline int sm_count() {
    static std::atomic<int> cached[64] = {};   // threads that race store the same value
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64) {
        const int c = cached[dev].load(std::memory_order_relaxed);
        if (c) return c;
    }
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (dev >= 0 && dev < 64) cached[dev].store(v, std::memory_order_relaxed);
    return v;
}

// Resident threads per SM of the persistent FP32 grid (see launch_tma_mode).
constexpr int kF32ThreadsPerSM = 768;

// TMA path: returns cudaErrorNotSupported (without launching) when the geometry does not allow it.
template <typename T, int TW, int TH, int RPT, int VEC, int S, int MODE, bool WRAP>
cudaError_t launch_tma_mode(const StencilArgs& a, cudaStream_t s) {
    TileGeom<T, TW, TH> g(a);
    // One box per window: at most 256 columns and 256 rows; rows and columns tile exactly; rows
    // 16-byte aligned (global address and stride rules of cuTensorMapEncodeTiled).
    if (!a.vec_ok || a.nx % TW != 0 || a.rows % TH != 0 || g.SW > 256 || g.SR > 256) return cudaErrorNotSupported;
    TmaMaps maps;
    memset(&maps, 0, sizeof(maps));
    if (!encode_rows_map<T>(&maps.win, a.in, a.nx, a.rows, g.SW, g.SR)) return cudaErrorNotSupported;
    // periodic in x: wrap-around boxes of the LP / RP edge columns (x = nx - LP and x = 0 are 16-byte
    // aligned: rows are, and LP, RP are whole 16-byte units)
    const int wl_bytes = WRAP ? g.wrap_l_bytes(a) : 0, wr_bytes = WRAP ? g.wrap_r_bytes(a) : 0;
    if (wl_bytes && !encode_rows_map<T>(&maps.wrap_l, a.in, a.nx, a.rows, g.LP, g.SR)) return cudaErrorNotSupported;
    if (wr_bytes && !encode_rows_map<T>(&maps.wrap_r, a.in, a.nx, a.rows, g.RP, g.SR)) return cudaErrorNotSupported;
    const size_t stage_bytes = round_up_int((int)((size_t)g.SR * g.SW * sizeof(T)), 128);
    const size_t smem = S * (stage_bytes + wl_bytes + wr_bytes) + round_up_int(a.ncoef * (int)sizeof(T), 16) +
                        round_up_int(a.ncoef * (int)sizeof(int), 16) + round_up_int(a.ncoef * (int)sizeof(T), 16) +
                        256;   // 128 bytes of alignment slack for the ring base + tail padding
    auto kern = stencil_tma_kernel<T, TW, TH, RPT, VEC, S, MODE, WRAP>;
    cudaError_t e = ensure_smem(kern, smem);
    if (e != cudaSuccess) return e == cudaErrorInvalidConfiguration ? cudaErrorNotSupported : e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (TW / VEC) * (TH / RPT), smem);
    if (e != cudaSuccess || per_sm < 1) return cudaErrorNotSupported;
    // FP32 launches are bound by HBM, and more resident CTAs (each keeping S windows in flight) made
    // them slower: over the twelve operators at 16384^2, 650 Gpts/s with every CTA that fits, 730
    // capped at 768 threads per SM, 624 at 512. The FP64 launches, bound by the FP64 pipe, keep every
    // CTA that fits (the 768 cap cost them 0.3%).
    if (sizeof(T) == 4) per_sm = std::min(per_sm, std::max(1, kF32ThreadsPerSM / ((TW / VEC) * (TH / RPT))));
    const int tiles_x = a.nx / TW;
    const int tiles_total = tiles_x * (a.rows / TH);
    int grid = std::min(tiles_total, per_sm * sm_count());
    const int cap = persistent_grid_cap();
    if (cap > 0) grid = std::min(grid, cap);
    dim3 block(TW / VEC, TH / RPT);
    kern<<<grid, block, smem, s>>>(maps, a, tiles_x, tiles_total);
    return cudaGetLastError();
}

// The instantiation with or without the wrap-around boxes; the Y shapes have no columns to wrap.
template <typename T, int TW, int TH, int RPT, int VEC, int S, int MODE>
cudaError_t launch_tma_wrap(const StencilArgs& a, cudaStream_t s, bool wrap) {
    if constexpr (MODE >= 5 && MODE <= 7) {
        return launch_tma_mode<T, TW, TH, RPT, VEC, S, MODE, false>(a, s);
    } else {
        return wrap ? launch_tma_mode<T, TW, TH, RPT, VEC, S, MODE, true>(a, s)
                    : launch_tma_mode<T, TW, TH, RPT, VEC, S, MODE, false>(a, s);
    }
}

template <typename T, int TW, int TH, int RPT, int VEC, int S>
cudaError_t launch_tma(const StencilArgs& a, cudaStream_t s) {
    const int mode = (variant_is_fun(a.variant) && !a.pre) ? (int)MODE_FUN : shape_mode(a.H, a.L, a.V, a.T);
    const bool wrap = a.wrap_x && (a.L > 0 || a.R > 0);
    switch (mode) {
    case MODE_FUN: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, MODE_FUN>(a, s, wrap);
    case 2: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 2>(a, s, wrap);
    case 3: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 3>(a, s, wrap);
    case 4: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 4>(a, s, wrap);
    case 5: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 5>(a, s, wrap);
    case 6: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 6>(a, s, wrap);
    case 7: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 7>(a, s, wrap);
    case 8: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 8>(a, s, wrap);
    case 9: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, 9>(a, s, wrap);
    default: return launch_tma_wrap<T, TW, TH, RPT, VEC, S, MODE_LIST>(a, s, wrap);
    }
}

}  // namespace custen
