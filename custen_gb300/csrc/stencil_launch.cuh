// Kernel entry and launcher template for the shared-memory tiled stencil (see stencil_kernel.cuh).
#pragma once

#include "stencil_kernel.cuh"
#include "stencil_tma.cuh"

namespace custen {

// Plain-load staged kernel: handles every geometry (odd widths, unaligned rows, any halo).
template <typename T, int TW, int TH, int RPT>
__global__ void __launch_bounds__((TW / VecT<T>::n) * (TH / RPT))
stencil_ldg_kernel(const __grid_constant__ StencilArgs a) {
    constexpr int VEC = VecT<T>::n;
    constexpr int NTX = TW / VEC;
    constexpr int NT = NTX * (TH / RPT);
    extern __shared__ __align__(128) unsigned char smem[];
    TileGeom<T, TW, TH> g(a);
    T* tile = reinterpret_cast<T*>(smem);
    T* coef_s = reinterpret_cast<T*>(smem + g.coef_off(a));
    int* list_off = reinterpret_cast<int*>(smem + g.list_off(a));
    T* list_w = reinterpret_cast<T*>(smem + g.listw_off(a));
    const int tid = threadIdx.x + threadIdx.y * NTX;
    const bool is_fun = variant_is_fun(a.variant);
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    stage_tile_ldg<T, TW, TH, NT>(a, tile, g, x0, y0, tid);
    const int nlist = stage_coefficients<T, NT>(a, coef_s, list_off, list_w, g.SW, tid, is_fun);  // syncs
    compute_and_store<T, TW, TH, RPT>(a, tile, coef_s, list_off, list_w, nlist, g, x0, y0, threadIdx.x,
                                      threadIdx.y, is_fun);
}

// Largest dynamic shared memory a block may opt in to on the current device.
inline int smem_optin_limit() {
    static int cached[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && cached[dev]) return cached[dev];
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) v = 48 * 1024;
    if (dev >= 0 && dev < 64) cached[dev] = v;
    return v;
}

template <typename Kernel>
inline cudaError_t ensure_smem(Kernel k, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    if (smem > (size_t)smem_optin_limit()) return cudaErrorInvalidConfiguration;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename T, int TW, int TH, int RPT>
cudaError_t launch_ldg(const StencilArgs& a, cudaStream_t s) {
    constexpr int VEC = VecT<T>::n;
    TileGeom<T, TW, TH> g(a);
    const size_t smem = g.total_bytes(a);
    cudaError_t e = ensure_smem(stencil_ldg_kernel<T, TW, TH, RPT>, smem);
    if (e != cudaSuccess) return e;
    dim3 block(TW / VEC, TH / RPT);
    dim3 grid((a.nx + TW - 1) / TW, (a.rows + TH - 1) / TH);
    stencil_ldg_kernel<T, TW, TH, RPT><<<grid, block, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace custen
