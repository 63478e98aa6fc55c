// Internal definitions shared by the host plan layer and the stencil kernels.
//
// Variant numbering, window geometry and the per-point write rules below restate the behaviour of
// the reference kernels (cuSten/src/kernels/2d_{x,y,xy}_{p,np}[_fun]_kernel.cu); each rule cites
// the reference lines it follows.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace custen {

enum Variant : int {
    V_XP = 0, V_XNP = 1, V_XPFUN = 2, V_XNPFUN = 3,
    V_YP = 4, V_YNP = 5, V_YPFUN = 6, V_YNPFUN = 7,
    V_XYP = 8, V_XYNP = 9, V_XYPFUN = 10, V_XYNPFUN = 11,
    V_COUNT = 12,          // the weighted / Fun variants above
    V_XYWENOADVP = 12      // WENO5 advection, periodic (its own Create argument list)
};

enum DType : int { DT_F64 = 0, DT_F32 = 1 };

__host__ __device__ inline bool variant_is_fun(int v) { return v == V_XPFUN || v == V_XNPFUN || v == V_YPFUN || v == V_YNPFUN ||
                                           v == V_XYPFUN || v == V_XYNPFUN; }
__host__ __device__ inline bool variant_is_periodic(int v) { return v == V_XP || v == V_XPFUN || v == V_YP || v == V_YPFUN ||
                                                v == V_XYP || v == V_XYPFUN || v == V_XYWENOADVP; }
__host__ __device__ inline int variant_dir(int v) { return v < 4 ? 0 : (v < 8 ? 1 : 2); }   // 0 = X, 1 = Y, 2 = XY

// Per-point outcome of one Compute.
enum Action : int { ACT_SKIP = 0, ACT_WRITE = 1, ACT_ZERO = 2 };

// Arguments of one stencil launch. A launch covers `rows` consecutive rows of the field starting at
// field row `row0` (a whole tile, or the whole field when the tiles are contiguous).
struct StencilArgs {
    void* out;            // output row row0
    const void* in;       // input row row0
    const void* top;      // T halo rows above the launch (row-major, stride nx); may be null if unused
    const void* bot;      // B halo rows below the launch; may be null if unused
    const void* coef;     // weights (plain variants) or coefficients (Fun variants), device-readable
    void* func;           // device function pointer (Fun variants)
    int nx;               // columns
    int rows;             // rows in this launch
    int row0;             // field row of launch row 0
    int L, R, T, B;       // halo extents
    int H, V;             // window width and height (weights are w[j*H+i])
    int ncoef;            // number of weights/coefficients staged per CTA
    int variant;          // Variant
    int bx, by;           // the caller's BLOCK_X / BLOCK_Y (only the non-periodic write rules use them)
    int nyTile;           // rows per tile
    int numTiles;
    int wrap_x;           // 1: columns outside [0,nx) wrap around (periodic variants)
    int has_top, has_bot; // 1: halo rows above / below may be read
    int vec_ok;           // 1: rows are 16-byte aligned, vector loads/stores allowed
    // 1: every staged input value c is replaced by c^3 - c (as fma(c*c, c, -c)) and the coefficients then
    // apply as plain weights. Set for the Fun variants when the device function is one of the library's
    // own c^3 - c functions, which compute exactly that (builtin_funs.cuh, ids 1, 3, 5).
    int pre;
    // WENO advection only: velocity rows row0.. and the inverse grid spacings (coeDx, coeDy)
    const void* u;
    const void* v;
    double cdx, cdy;
};

// Write rule of the reference for point (x, gy) of the field, gy a field row.
// Division-free: only a tile's first and last block rows and the field's first and last block columns
// have rules, so "first block" is x < bx, "last block" is x >= nx - bx (nx is a multiple of bx), and the
// position inside such a block follows by subtraction; the tile of row gy is found by stepping over
// the (few) tiles. The edge tiles of a launch evaluate this per point.
__host__ __device__ inline int point_action(int variant, int x, int gy, int nx, int L, int R, int T, int B,
                                            int bx, int by, int nyTile, int numTiles) {
    switch (variant) {
    case V_XNP:
        // kernel2DXnp: block 0 skips threads tx < L (2d_x_np_kernel.cu:137); the last block stores
        // the zero-initialised sum for tx >= BLOCK_X - R (:164-176, store outside the if).
        if (x < L) return ACT_SKIP;
        if (x >= nx - R) return ACT_ZERO;
        return ACT_WRITE;
    case V_XNPFUN:
        // kernel2DXnpFun: tx < L skipped in block 0 (2d_x_np_fun_kernel.cu:144-149), tx >= BX - R
        // skipped in the last block (:165-170).
        if (x < L || x >= nx - R) return ACT_SKIP;
        return ACT_WRITE;
    default:
        break;
    }
    int t = 0, yt = gy;   // tile of row gy and the row inside it
    while (yt >= nyTile && t < numTiles - 1) {
        yt -= nyTile;
        ++t;
    }
    switch (variant) {
    case V_YNP:
    case V_YNPFUN:
        // kernel2DYnp / kernel2DYnpFun: in the first tile block row 0 stores rows T..BY-1 only
        // (2d_y_np_kernel.cu:167-192, 2d_y_np_fun_kernel.cu:173-193); in the last tile the last block
        // row stores ty < BY - B (2d_y_np_kernel.cu:246-249, 2d_y_np_fun_kernel.cu:242).
        if (t == 0 && yt < T) return ACT_SKIP;
        if (t == numTiles - 1 && yt >= nyTile - B) return ACT_SKIP;
        return ACT_WRITE;
    case V_XYNP:
    case V_XYNPFUN: {
        // kernel2DXYnp: nine block cases tested in this order (2d_xy_np_kernel.cu:136-958).
        const bool left = x < bx, right = x >= nx - bx;             // first / last block column
        const bool topb = yt < by, botb = yt >= nyTile - by;        // first / last block row of the tile
        const int txl = x, txr = x - (nx - bx);                     // tx inside the first / last block
        const int tyt = yt, tyb = yt - (nyTile - by);               // ty inside the first / last block row
        const bool tileTop = (t == 0), tileBottom = (t == numTiles - 1);
        bool ok;
        if (left && topb) ok = tileTop ? (txl >= L && tyt >= T) : (txl >= L);                     // :208-219
        else if (right && topb) ok = tileTop ? (txr < bx - R && tyt >= T) : (txr < bx - R);       // :301-312
        else if (left && botb) ok = tileBottom ? (txl >= L && tyb < by - B) : (txl >= L);         // :393-404
        else if (right && botb) ok = tileBottom ? (txr < bx - R && tyb < by - B) : (txr < bx - R); // :484-495
        else if (topb) ok = tileTop ? (tyt >= T) : true;                                        // :593-602
        else if (botb) ok = tileBottom ? (tyb < by - B) : true;                                 // :699-708
        else if (left) ok = (txl >= L);                                                         // :784
        // Right edge, middle block rows: the reference guard is tx < BX - L (:862; :787 for Fun).
        // When L < R the reference stores values read from shared memory it never loaded for
        // tx in [BX-R, BX-L); those points are left untouched here.
        else if (right) ok = (txr < bx - L) && (txr < bx - R);
        else ok = true;
        return ok ? ACT_WRITE : ACT_SKIP;
    }
    default:
        return ACT_WRITE;   // periodic variants write every point
    }
}

// Private per-handle state. It lives in the same allocation as the handle's stream array (the
// reference allocates `streams` with malloc and only Destroy frees it), so cuSten_t keeps its layout.
struct PlanPrivate {
    uint32_t magic;
    int variant;
    int dtype;
    int H, V, L, R, T, B;
    int ncoef;            // weights or coefficients read per Compute
    int mem_kind;         // -1 unknown, 0 device, 1 managed, 2 host-accessible system memory
    cudaStream_t user_stream;
    int use_user_stream;
    unsigned long long launches;   // kernels launched by this handle (for instrumentation)
    // Fun variants: the device function last checked against the library's own functions, and whether
    // it can run as c^3 - c followed by plain weights (StencilArgs::pre).
    void* fused_func;
    int fused_pre;
    int cfg;   // kernel configuration (stencil_configs.h) of the device-resident launches; -1 not chosen yet
    // Slab handles (custen_create_slab): the handle's one tile is tile `slab` of a field of `slabs` tiles
    // held by several owners; its halo rows are the caller's buffers. slabs = 0: an ordinary handle.
    int slab, slabs;
    // Host-resident fields (pinned or system memory) are streamed through device staging slots:
    // kStageSlots slots of (T + chunk + B) input rows and chunk output rows, plus the weights.
    // Allocated at the first such Compute, freed by Destroy.
    void* stage;
    size_t stage_slot_bytes;
    int stage_rows;               // rows per chunk
    int stage_events_ready;
    cudaEvent_t stage_ev[3 * 3];  // per slot: inputs copied in, kernel done, outputs copied out
};

constexpr int kStageSlots = 3;

struct StreamBlock {
    cudaStream_t streams[3];
    PlanPrivate priv;
};

constexpr uint32_t kPlanMagic = 0xC5E7B300u;

// Launch entry points implemented in the kernel translation units.
// *path is set to 1 when the TMA-staged kernel ran, 0 for the plain-load kernel.
cudaError_t launch_stencil_f64(const StencilArgs& a, cudaStream_t s, int* path);
cudaError_t launch_stencil_f32(const StencilArgs& a, cudaStream_t s, int* path);
cudaError_t launch_weno_adv(const StencilArgs& a, cudaStream_t s);

}  // namespace custen
