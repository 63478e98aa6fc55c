// Shared-memory tiled 2D stencil kernel for sm_103a (FP64 and FP32), covering all twelve cuSten
// variants (X / Y / XY, periodic / non-periodic, weights / device-function-pointer).
//
// Per point the value is the reference's FMA chain: sum = 0; for j in 0..V-1, for i in 0..H-1:
// sum = fma(w[j*H+i], in[y-T+j][x-L+i], sum) (cuSten/src/kernels/2d_xy_p_kernel.cu:507-520; the X
// and Y kernels are the V=1 and H=1 cases, 2d_x_p_kernel.cu:166-172, 2d_y_p_kernel.cu:120-124).
// Exact-zero weights are dropped from the chain: fma(0, a, s) == s for every finite a and the chain
// starts from +0.0, so the result is bit-identical for finite inputs.
//
// Each CTA owns an output tile of TW x TH points. It stages the (TH+T+B) x (LP+TW+RP) input window
// in shared memory -- the rows from the launch's own rows or from the top/bottom halo pointers, the
// columns wrapped (periodic) or zero-filled (non-periodic) -- then every thread produces VEC adjacent
// columns x RPT rows with 16-byte vector stores. Halo tiles are staged by TMA (stencil_tma.cuh) when
// the geometry allows; this file holds the compute/store stage and the plain-load staging path.
#pragma once

#include "builtin_funs.cuh"
#include "checked.cuh"
#include "custen_internal.h"

namespace custen {

// VEC adjacent outputs per thread, moved with one VEC-wide load / store. The halo columns of a staged
// row are padded to 16 bytes whatever VEC is: a TMA box starts and spans whole 16-byte units.
template <typename T, int N> struct VecN;
template <> struct VecN<double, 1> { using type = double; };
template <> struct VecN<double, 2> { using type = double2; };
template <> struct VecN<float, 1> { using type = float; };
template <> struct VecN<float, 2> { using type = float2; };
template <> struct VecN<float, 4> { using type = float4; };
template <typename T> struct Pad16 { static constexpr int n = 16 / (int)sizeof(T); };

__host__ __device__ constexpr int round_up_int(int v, int m) { return (v + m - 1) / m * m; }

// Geometry of the staged window, identical on host (shared-memory sizing) and device.
template <typename T, int TW, int TH>
struct TileGeom {
    static constexpr int PAD = Pad16<T>::n;
    int LP, RP, SW, SR;
    __host__ __device__ TileGeom(const StencilArgs& a) {
        LP = round_up_int(a.L, PAD);
        RP = round_up_int(a.R, PAD);
        SW = LP + TW + RP;
        SR = TH + a.T + a.B;
    }
    __host__ __device__ size_t tile_bytes() const { return (size_t)SR * SW * sizeof(T); }
    // TMA path, periodic in x: per stage, the side areas that the wrap-around boxes fill (LP x SR and
    // RP x SR elements, each rounded up to 128 bytes); zero when the launch does not wrap.
    __host__ __device__ int wrap_l_bytes(const StencilArgs& a) const {
        return a.wrap_x && LP > 0 ? round_up_int(LP * SR * (int)sizeof(T), 128) : 0;
    }
    __host__ __device__ int wrap_r_bytes(const StencilArgs& a) const {
        return a.wrap_x && RP > 0 ? round_up_int(RP * SR * (int)sizeof(T), 128) : 0;
    }
    // tile | coefficients (ncoef T) | compact list offsets (ncoef int) | compact list weights (ncoef T)
    __host__ __device__ size_t coef_off(const StencilArgs&) const { return round_up_int((int)tile_bytes(), 16); }
    __host__ __device__ size_t list_off(const StencilArgs& a) const {
        return coef_off(a) + round_up_int(a.ncoef * (int)sizeof(T), 16);
    }
    __host__ __device__ size_t listw_off(const StencilArgs& a) const {
        return list_off(a) + round_up_int(a.ncoef * (int)sizeof(int), 16);
    }
    __host__ __device__ size_t total_bytes(const StencilArgs& a) const {
        return listw_off(a) + round_up_int(a.ncoef * (int)sizeof(T), 16) + 16;
    }
};

template <typename T>
__device__ __forceinline__ const T* launch_row(const StencilArgs& a, int gyl) {
    // Launch-relative row gyl in [-T, rows + B): own rows, or the halo rows behind the top/bottom
    // pointers (the per-tile boundaryTop/boundaryBottom pointers of the handle).
    if (gyl >= 0 && gyl < a.rows) return reinterpret_cast<const T*>(a.in) + (size_t)gyl * a.nx;
    if (gyl < 0) {
        if (a.has_top && gyl + a.T >= 0) return reinterpret_cast<const T*>(a.top) + (size_t)(gyl + a.T) * a.nx;
        return nullptr;
    }
    int k = gyl - a.rows;
    if (a.has_bot && k < a.B) return reinterpret_cast<const T*>(a.bot) + (size_t)k * a.nx;
    return nullptr;
}

// Stage coefficients and, for weight variants, the compact list of non-zero weights in weight order.
template <typename T, int NT>
__device__ __forceinline__ int stage_coefficients(const StencilArgs& a, T* coef_s, int* list_off, T* list_w,
                                                  int SW, int tid, bool is_fun) {
    const T* c = reinterpret_cast<const T*>(a.coef);
    for (int k = tid; k < a.ncoef; k += NT) coef_s[k] = c[k];
    __syncthreads();
    __shared__ int s_count;
    if (!is_fun && tid == 0) {
        int n = 0;
        for (int k = 0; k < a.ncoef; ++k) {
            T w = coef_s[k];
            if (w != T(0)) {
                int j = k / a.H, i = k - j * a.H;
                list_off[n] = j * SW + i;
                list_w[n] = w;
                ++n;
            }
        }
        s_count = n;
    }
    __syncthreads();
    return is_fun ? 0 : s_count;
}

// c -> c^3 - c over a staged window, once per staged value (StencilArgs::pre): the operation of the
// library's c^3 - c Fun functions (builtin_funs.cuh, cube_minus), so that the weights applied afterwards
// give their results bit for bit with one cube per input value instead of one per window point.
template <typename T, int NT>
__device__ __forceinline__ void apply_cube(T* tile, int count, int tid) {
    for (int e = tid; e < count; e += NT) tile[e] = custen_funs::cube_minus<T>(tile[e]);
}

// Plain-load staging of the window (16-byte vector loads where the whole vector is in range).
template <typename T, int TW, int TH, int NT, int VEC>
__device__ __forceinline__ void stage_tile_ldg(const StencilArgs& a, T* tile, const TileGeom<T, TW, TH>& g,
                                               int x0, int y0, int tid) {
    using V = typename VecN<T, VEC>::type;
    const int cvecs = g.SW / VEC;
    const int total = g.SR * cvecs;
    for (int e = tid; e < total; e += NT) {
        int r = e / cvecs;
        int c = (e - r * cvecs) * VEC;
        int gx = x0 - g.LP + c;
        const T* rowp = launch_row<T>(a, y0 - a.T + r);
        if (!span_ok((long long)r * g.SW + c, VEC, (long long)g.SR * g.SW)) continue;
        T* dst = tile + r * g.SW + c;
        if (rowp == nullptr) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) dst[v] = T(0);
            continue;
        }
        if (a.vec_ok && gx >= 0 && gx + VEC <= a.nx) {
            *reinterpret_cast<V*>(dst) = __ldg(reinterpret_cast<const V*>(rowp + gx));
        } else {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                int x = gx + v;
                T val = T(0);
                if (x >= 0 && x < a.nx) val = __ldg(rowp + x);
                else if (a.wrap_x) {
                    int xw = x < 0 ? x + a.nx : x - a.nx;
                    if (xw >= 0 && xw < a.nx) val = __ldg(rowp + xw);
                }
                dst[v] = val;
            }
        }
    }
}

// True when every point of the tile is written with its stencil value (no write rule applies).
__device__ __forceinline__ bool tile_all_write(const StencilArgs& a, int x0, int x1, int gy0, int gy1) {
    switch (a.variant) {
    case V_XNP:
    case V_XNPFUN:
        return x0 >= a.L && x1 <= a.nx - a.R;
    case V_YNP:
    case V_YNPFUN:
        return gy0 >= a.T && gy1 <= a.nyTile * a.numTiles - a.B;
    case V_XYNP:
    case V_XYNPFUN: {
        if (x0 < a.bx || x1 > a.nx - a.bx) return false;
        const int ny = a.nyTile * a.numTiles;
        return gy0 >= a.by && gy1 <= ny - a.by;
    }
    default:
        return true;
    }
}

template <typename T> using FunX = T (*)(T*, T*, int);
template <typename T> using FunY = T (*)(T*, T*, int, int);
template <typename T> using FunXY = T (*)(T*, T*, int, int, int, int);

// Store VEC x RPT outputs of one thread: 16-byte vector stores where every point is written with its
// stencil value, the reference's write rules (untouched / zero) elsewhere.
template <typename T, int RPT, int VEC>
__device__ __forceinline__ void store_outputs(const StencilArgs& a, const T (&acc)[RPT][VEC], int gx, int gy0,
                                              bool all_write_tile) {
    using V = typename VecN<T, VEC>::type;
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr) {
        const int gyl = gy0 + rr;
        if (gyl >= a.rows) break;
        const int gy = a.row0 + gyl;
        const bool row_ok = in_bounds(gyl, 0, a.rows);
        T* orow = reinterpret_cast<T*>(a.out) + (size_t)gyl * a.nx;
        int act[VEC];
        bool all_write = true;
        if (all_write_tile && gx + VEC <= a.nx) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) act[v] = ACT_WRITE;
        } else {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                act[v] = (gx + v < a.nx) ? point_action(a.variant, gx + v, gy, a.nx, a.L, a.R, a.T, a.B, a.bx,
                                                        a.by, a.nyTile, a.numTiles)
                                         : ACT_SKIP;
                all_write = all_write && (act[v] == ACT_WRITE);
            }
        }
        if (all_write && a.vec_ok) {
            V outv;
            T* o = reinterpret_cast<T*>(&outv);
#pragma unroll
            for (int v = 0; v < VEC; ++v) o[v] = acc[rr][v];
            if (row_ok && span_ok(gx, VEC, a.nx)) *reinterpret_cast<V*>(orow + gx) = outv;
        } else {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                if (act[v] == ACT_SKIP || !row_ok || !in_bounds(gx + v, 0, a.nx)) continue;
                orow[gx + v] = act[v] == ACT_WRITE ? acc[rr][v] : T(0);
            }
        }
    }
}

// Compute VEC x RPT outputs per thread from the staged window and store them.
template <typename T, int TW, int TH, int RPT, int VEC>
__device__ __forceinline__ void compute_and_store(const StencilArgs& a, T* tile, T* coef_s, const int* list_off,
                                                  const T* list_w, int nlist, const TileGeom<T, TW, TH>& g,
                                                  int x0, int y0, int tx, int ty, bool is_fun, bool all_write_tile) {
    const int c0 = tx * VEC;    // tile-local column of the first output
    const int r0 = ty * RPT;    // tile-local row of the first output
    T acc[RPT][VEC];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr)
#pragma unroll
        for (int v = 0; v < VEC; ++v) acc[rr][v] = T(0);

    // Smem index of the top-left corner of the window of output (r0, c0).
    const int base = r0 * g.SW + g.LP + c0 - a.L;
    if (!is_fun) {
        for (int e = 0; e < nlist; ++e) {
            const T w = list_w[e];
            if (!span_ok((long long)base + list_off[e], (long long)(RPT - 1) * g.SW + VEC, (long long)g.SR * g.SW))
                continue;
            const T* p = tile + base + list_off[e];
#pragma unroll
            for (int rr = 0; rr < RPT; ++rr)
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[rr][v] = fma(w, p[rr * g.SW + v], acc[rr][v]);
        }
    } else {
        const int dir = variant_dir(a.variant);
#pragma unroll
        for (int rr = 0; rr < RPT; ++rr) {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                const int tl = base + rr * g.SW + v;    // window top-left
                if (!span_ok(tl, (long long)(a.T + a.B) * g.SW + a.L + a.R + 1, (long long)g.SR * g.SW)) continue;
                if (dir == 0) {
                    acc[rr][v] = reinterpret_cast<FunX<T>>(a.func)(tile, coef_s, tl + a.L);
                } else if (dir == 1) {
                    acc[rr][v] = reinterpret_cast<FunY<T>>(a.func)(tile, coef_s, tl + a.T * g.SW + a.L, g.SW);
                } else {
                    acc[rr][v] = reinterpret_cast<FunXY<T>>(a.func)(tile, coef_s, tl, g.SW, a.H, a.V);
                }
            }
        }
    }

    store_outputs<T, RPT, VEC>(a, acc, x0 + c0, y0 + r0, all_write_tile);
}

// ---------------------------------------------------------------------------------------------
// Compile-time stencil shapes: register sliding window along y, 16-byte conflict-free shared loads.
// ---------------------------------------------------------------------------------------------
template <int H_, int L_, int V_, int T_>
struct Shape {
    static constexpr int H = H_, L = L_, V = V_, T = T_;
};

// Kernel modes: 0 generic (list of non-zero weights), 1 device function, >= 2 the shapes below.
enum : int { MODE_LIST = 0, MODE_FUN = 1, MODE_FIRST_SHAPE = 2, MODE_COUNT = 10 };
template <int MODE> struct ShapeOf { using type = Shape<1, 0, 1, 0>; };
template <> struct ShapeOf<2> { using type = Shape<3, 1, 1, 0>; };   // X 3-point
template <> struct ShapeOf<3> { using type = Shape<5, 2, 1, 0>; };   // X 5-point
template <> struct ShapeOf<4> { using type = Shape<9, 4, 1, 0>; };   // X 9-point
template <> struct ShapeOf<5> { using type = Shape<1, 0, 3, 1>; };   // Y 3-point
template <> struct ShapeOf<6> { using type = Shape<1, 0, 5, 2>; };   // Y 5-point
template <> struct ShapeOf<7> { using type = Shape<1, 0, 9, 4>; };   // Y 9-point
template <> struct ShapeOf<8> { using type = Shape<3, 1, 3, 1>; };   // XY 3 x 3
template <> struct ShapeOf<9> { using type = Shape<5, 2, 5, 2>; };   // XY 5 x 5

// Host: the shape mode matching a launch's window, or MODE_LIST.
inline int shape_mode(int H, int L, int V, int T) {
    const int tab[8][4] = {{3, 1, 1, 0}, {5, 2, 1, 0}, {9, 4, 1, 0}, {1, 0, 3, 1},
                           {1, 0, 5, 2}, {1, 0, 9, 4}, {3, 1, 3, 1}, {5, 2, 5, 2}};
    for (int k = 0; k < 8; ++k)
        if (tab[k][0] == H && tab[k][1] == L && tab[k][2] == V && tab[k][3] == T) return MODE_FIRST_SHAPE + k;
    return MODE_LIST;
}

// Each thread slides down its RPT output rows: input row r0 + k is read once (NV 16-byte loads covering
// the columns its VEC outputs need) and applied to every output row whose window contains it. Per
// output the FMAs run j = 0..V-1 (rows, top first), i = 0..H-1 -- the reference order
// (2d_xy_p_kernel.cu:507-520) -- all weights included, zeros too.
template <typename T, int TW, int TH, int RPT, int VEC, class SH>
__device__ __forceinline__ void compute_window_store(const StencilArgs& a, const T* tile, const T* coef_s,
                                                     const TileGeom<T, TW, TH>& g, int x0, int y0, int tx, int ty,
                                                     bool all_write_tile) {
    using VV = typename VecN<T, VEC>::type;
    constexpr int LP = round_up_int(SH::L, Pad16<T>::n);
    constexpr int D = LP - SH::L;                       // first needed column inside the aligned segment
    constexpr int NV = (D + VEC + SH::H - 1 + VEC - 1) / VEC;
    const int c0 = tx * VEC, r0 = ty * RPT;
    T acc[RPT][VEC];
#pragma unroll
    for (int rr = 0; rr < RPT; ++rr)
#pragma unroll
        for (int v = 0; v < VEC; ++v) acc[rr][v] = T(0);
#pragma unroll
    for (int k = 0; k < RPT + SH::V - 1; ++k) {
        T seg[NV * VEC];
        if (!span_ok((long long)(r0 + k) * g.SW + c0, NV * VEC, (long long)g.SR * g.SW)) continue;
        const VV* src = reinterpret_cast<const VV*>(tile + (r0 + k) * g.SW + c0);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const VV t = src[q];
            const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
            for (int v = 0; v < VEC; ++v) seg[q * VEC + v] = tp[v];
        }
#pragma unroll
        for (int rr = 0; rr < RPT; ++rr) {
            const int j = k - rr;
            if (j < 0 || j >= SH::V) continue;
#pragma unroll
            for (int i = 0; i < SH::H; ++i) {
                const T w = coef_s[j * SH::H + i];
#pragma unroll
                for (int v = 0; v < VEC; ++v) acc[rr][v] = fma(w, seg[D + v + i], acc[rr][v]);
            }
        }
    }
    store_outputs<T, RPT, VEC>(a, acc, x0 + c0, y0 + r0, all_write_tile);
}

}  // namespace custen
