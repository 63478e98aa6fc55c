// TMA-staged, persistent, multi-stage stencil kernel (sm_103a).
//
// Each CTA walks the output tiles tile = blockIdx.x + k * gridDim.x and keeps S tile windows in
// flight in a shared-memory ring. One thread issues one tensor-memory-accelerator copy per window: a
// box of SW = LP + TW + RP columns by SR = T + TH + B rows starting at (x0 - LP, y0 - T), landing at a
// 128-byte aligned stage. Completion is signalled on the stage's mbarrier (complete_tx); the next
// tiles' copies run while the current tile computes. Rows and columns outside the launch arrive
// zero-filled. Periodic variants add wrap-around boxes on the first and last tile column: the LP
// columns left of x = 0 come from x = nx - LP, the RP columns right of nx from x = 0, each into a
// side area of the stage on the same mbarrier, from where the edge tile copies them into place.
// Edge tiles of the first and last tile row fetch their halo rows through the halo pointers with
// plain (coalesced) loads.
//
// Every mbarrier wait is bounded: on expiry the CTA records an error in g_custen_device_error, waits
// (bounded) for its own copies still in flight, and returns.
#pragma once

#include <cuda.h>

#include "stencil_kernel.cuh"

namespace custen {

constexpr unsigned int kErrMbarrierTimeout = 1u;   // g_custen_device_error: checked.cuh
constexpr long long kWaitLimit = 1ll << 22;   // try_wait rounds (each may suspend ~µs) before giving up

struct TmaMaps {
    CUtensorMap win;      // launch rows, box {SW, SR}
    CUtensorMap wrap_l;   // periodic x: box {LP, SR}, read at x = nx - LP for the tiles at x0 = 0
    CUtensorMap wrap_r;   // periodic x: box {RP, SR}, read at x = 0 for the tiles ending at nx
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase with the given parity to complete; false after `limit` rounds.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kWaitLimit) {
    const uint32_t addr = smem_u32(bar);
    for (long long i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Issue the copies of one tile window into the (128-byte aligned) stage `dst`: the window box, and on
// the first / last tile column of a periodic launch the wrap-around boxes into the stage's side areas
// `side` (LP x SR elements, then RP x SR from `side + wl_elems`).
template <typename T, int TW, int TH>
__device__ __forceinline__ void issue_window(const StencilArgs& a, const TmaMaps& m, T* dst, T* side, int wl_elems,
                                             int wr_elems, uint64_t* bar, int x0, int y0,
                                             const TileGeom<T, TW, TH>& g) {
    const bool left = wl_elems > 0 && x0 == 0;
    const bool right = wr_elems > 0 && x0 + TW == a.nx;
    uint32_t bytes = (uint32_t)(g.SR * g.SW * sizeof(T));
    if (left) bytes += (uint32_t)(g.SR * g.LP * sizeof(T));
    if (right) bytes += (uint32_t)(g.SR * g.RP * sizeof(T));
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_2d(dst, &m.win, x0 - g.LP, y0 - a.T, bar);
    if (left) tma_load_2d(side, &m.wrap_l, a.nx - g.LP, y0 - a.T, bar);
    if (right) tma_load_2d(side + wl_elems, &m.wrap_r, 0, y0 - a.T, bar);
}

// Edge tiles: replace the zero-filled cells outside the launch. Rows above / below the launch come
// through the halo pointers (when the variant reads them); columns outside [0, nx) wrap around
// (periodic variants): those of the rows inside the launch from the stage's side areas, filled by the
// wrap-around boxes. Cells with no source are left as zeros: no written point reads them.
template <typename T, int TW, int TH, int NT>
__device__ __forceinline__ void edge_fixup(const StencilArgs& a, T* tile, const T* side, int wl_elems,
                                           const TileGeom<T, TW, TH>& g, int x0, int y0, int tid, bool rows_fix,
                                           bool cols_fix) {
    if (rows_fix) {
        // whole halo rows (all SW columns) of the rows outside [0, rows)
        const int total = g.SR * g.SW;
        for (int e = tid; e < total; e += NT) {
            const int r = e / g.SW;
            const int gyl = y0 - a.T + r;
            if (gyl >= 0 && gyl < a.rows) continue;
            const T* rowp = launch_row<T>(a, gyl);
            if (rowp == nullptr) continue;
            const int c = e - r * g.SW;
            int x = x0 - g.LP + c;
            if (x < 0 || x >= a.nx) {
                if (!a.wrap_x) continue;
                x = x < 0 ? x + a.nx : x - a.nx;
                if (x < 0 || x >= a.nx) continue;
            }
            tile[e] = __ldg(rowp + x);
        }
    }
    if (cols_fix) {
        // wrapped halo columns of the rows inside the launch, from the side areas: column k < LP of
        // row r is side[r * LP + k] (x = nx - LP + k), column LP + TW + k is side_r[r * RP + k] (x = k);
        // the boxes zero-fill x outside [0, nx) as a too-narrow field needs
        const bool left = x0 == 0, right = x0 + TW == a.nx;
        const T* side_r = side + wl_elems;
        const int ncols = g.LP + g.RP;
        const int total = g.SR * ncols;
        for (int e = tid; e < total; e += NT) {
            const int r = e / ncols;
            const int gyl = y0 - a.T + r;
            if (gyl < 0 || gyl >= a.rows) continue;
            const int k = e - r * ncols;
            if (k < g.LP) {
                if (!left) continue;
                if (!in_bounds((long long)r * g.SW + k, 0, (long long)g.SR * g.SW)) continue;
                tile[r * g.SW + k] = side[r * g.LP + k];
            } else {
                if (!right) continue;
                const int kk = k - g.LP;
                if (!in_bounds((long long)r * g.SW + g.LP + TW + kk, 0, (long long)g.SR * g.SW)) continue;
                tile[r * g.SW + g.LP + TW + kk] = side_r[r * g.RP + kk];
            }
        }
    }
}

// MODE: MODE_LIST (weights, generic window), MODE_FUN (device function), or a compile-time shape.
// FP64 shape kernels fall back to the list when a weight is zero (FP64 FMAs are the bottleneck on
// GB300; dropping exact zeros is bit-neutral for finite inputs).
// Resident CTAs the register allocation must allow: 768 threads per SM (512 for the device-function
// mode, whose indirect calls need more registers).
constexpr int min_blocks_for(int threads, bool fun) { return (fun ? 512 : 768) / threads > 0 ? (fun ? 512 : 768) / threads : 1; }

// WRAP: the launch is periodic in x with a left or right halo (wrap-around boxes and side areas); the
// other launches run an instantiation without them, which keeps their register allocation.
template <typename T, int TW, int TH, int RPT, int VEC, int S, int MODE, bool WRAP>
__global__ void __launch_bounds__((TW / VEC) * (TH / RPT), min_blocks_for((TW / VEC) * (TH / RPT), MODE == MODE_FUN))
stencil_tma_kernel(const __grid_constant__ TmaMaps maps, const __grid_constant__ StencilArgs a, int tiles_x,
                   int tiles_total) {
    constexpr int NTX = TW / VEC;
    constexpr int NT = NTX * (TH / RPT);
    // The dynamic segment is only guaranteed 16-byte alignment (with relocatable device code its
    // placement after the static shared objects is fixed at link time); the ring is aligned to 128
    // bytes at run time inside 128 bytes of slack. The address goes through an empty asm so that no
    // alignment assumption can fold the computation away.
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[S];
    TileGeom<T, TW, TH> g(a);
    const size_t stage_elems = (size_t)g.SR * g.SW;
    const size_t stage_bytes = round_up_int((int)(stage_elems * sizeof(T)), 128);
    uint32_t raw_addr = smem_u32(smem_raw);
    asm volatile("" : "+r"(raw_addr));
    unsigned char* smem = smem_raw + ((128u - (raw_addr & 127u)) & 127u);
    T* ring = reinterpret_cast<T*>(smem);
    // side areas of the wrap-around boxes, per stage (zero-sized unless the launch wraps in x)
    const int wl_bytes = WRAP ? g.wrap_l_bytes(a) : 0, wr_bytes = WRAP ? g.wrap_r_bytes(a) : 0;
    const int wl_elems = wl_bytes / (int)sizeof(T), wr_elems = wr_bytes / (int)sizeof(T);
    T* sides = reinterpret_cast<T*>(smem + S * stage_bytes);
    unsigned char* after = smem + S * (stage_bytes + wl_bytes + wr_bytes);
    T* coef_s = reinterpret_cast<T*>(after);
    int* list_off = reinterpret_cast<int*>(after + round_up_int(a.ncoef * (int)sizeof(T), 16));
    T* list_w = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(list_off) +
                                     round_up_int(a.ncoef * (int)sizeof(int), 16));
    const int tid = threadIdx.x + threadIdx.y * NTX;
    constexpr bool is_fun = (MODE == MODE_FUN);

    if (tid == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int k = 0; k < S; ++k) {
            const int t = blockIdx.x + k * gridDim.x;
            if (t >= tiles_total) break;
            const int tyi = t / tiles_x, txi = t - tyi * tiles_x;
            issue_window<T, TW, TH>(a, maps, ring + (size_t)k * stage_bytes / sizeof(T),
                                    sides + (size_t)k * (wl_elems + wr_elems), wl_elems, wr_elems, &full[k],
                                    txi * TW, tyi * TH, g);
        }
    }
    const int nlist = stage_coefficients<T, NT>(a, coef_s, list_off, list_w, g.SW, tid, is_fun);  // syncs

    for (int it = 0;; ++it) {
        const int t = blockIdx.x + it * gridDim.x;
        if (t >= tiles_total) break;
        const int s = it % S;
        const uint32_t parity = (uint32_t)((it / S) & 1);
        T* tile = ring + (size_t)s * stage_bytes / sizeof(T);
        T* side = sides + (size_t)s * (wl_elems + wr_elems);
        // Each thread waits on the stage itself (the wait acquires the copy's data for that thread), so
        // no barrier is needed before reading it. A thread whose wait expired skips the tile's compute;
        // the end-of-tile barrier then makes the exit decision uniform.
        const bool ok = mbar_wait(&full[s], parity);
        const int tyi = t / tiles_x, txi = t - tyi * tiles_x;
        const int x0 = txi * TW, y0 = tyi * TH;
        const bool rows_fix = (y0 == 0 && a.T > 0 && a.has_top) || (y0 + TH == a.rows && a.B > 0 && a.has_bot);
        const bool cols_fix = WRAP && (x0 == 0 || x0 + TW == a.nx);
        if (rows_fix || cols_fix) {
            edge_fixup<T, TW, TH, NT>(a, tile, side, wl_elems, g, x0, y0, tid, rows_fix, cols_fix);
            __syncthreads();
        }
        if (a.pre) {
            apply_cube<T, NT>(tile, (int)stage_elems, tid);
            __syncthreads();
        }
        const bool all_write = tile_all_write(a, x0, x0 + TW, a.row0 + y0, a.row0 + y0 + TH);
        if (ok) {
            if constexpr (MODE >= MODE_FIRST_SHAPE) {
                using SH = typename ShapeOf<MODE>::type;
                if (sizeof(T) == 4 || nlist == SH::H * SH::V)
                    compute_window_store<T, TW, TH, RPT, VEC, SH>(a, tile, coef_s, g, x0, y0, threadIdx.x,
                                                                  threadIdx.y, all_write);
                else
                    compute_and_store<T, TW, TH, RPT, VEC>(a, tile, coef_s, list_off, list_w, nlist, g, x0, y0,
                                                           threadIdx.x, threadIdx.y, false, all_write);
            } else {
                compute_and_store<T, TW, TH, RPT, VEC>(a, tile, coef_s, list_off, list_w, nlist, g, x0, y0,
                                                       threadIdx.x, threadIdx.y, is_fun, all_write);
            }
        }
        fence_proxy_async_smem();
        // every thread is done with stage s; a copy that never completed ends the CTA here: record it,
        // wait (bounded) for the copies this CTA still has in flight, and leave
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(&g_custen_device_error, kErrMbarrierTimeout);
                for (int k = 0; k < S; ++k) {
                    const int tk = blockIdx.x + (it + k) * gridDim.x;
                    if (tk >= tiles_total) break;
                    mbar_wait(&full[(it + k) % S], (uint32_t)(((it + k) / S) & 1));
                }
            }
            __syncthreads();
            return;
        }
        if (tid == 0) {
            const int tn = t + S * gridDim.x;
            if (tn < tiles_total) {
                const int tyn = tn / tiles_x, txn = tn - tyn * tiles_x;
                issue_window<T, TW, TH>(a, maps, tile, side, wl_elems, wr_elems, &full[s], txn * TW, tyn * TH, g);
            }
        }
    }
}

}  // namespace custen
