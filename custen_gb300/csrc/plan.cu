// Host plan layer: Create / Swap / Destroy / Compute for the twelve cuSten variants, the reference's
// C++ API (exit-on-error, cuSten/src/util/error.cu:43-53) and the status-returning C-ABI.
//
// The handle is filled as the reference's Create functions fill it (sizes, per-tile input/output
// pointers, per-tile halo pointers, grid, three streams and two events): see
// cuSten/src/struct/custenCreateDestroy2D*.cu. Compute differs in how it runs, not in what it
// computes: when the tiles are contiguous in memory and the data is device-resident, the whole field
// is one launch (the per-tile halo pointers then name rows of the same array); otherwise one launch
// per tile reads its halo rows through the handle's boundaryTop/boundaryBottom pointers.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/cuSten.h"
#include "../../include/custen_gb300.h"
#include "custen_internal.h"
#include "stencil_configs.h"

static_assert(sizeof(cuSten_t) == 200, "cuSten_t must keep the reference layout (200 bytes)");
static_assert(offsetof(cuSten_t, weights) == 104, "cuSten_t::weights offset");
static_assert(offsetof(cuSten_t, streams) == 176, "cuSten_t::streams offset");
static_assert(offsetof(cuSten_t, devFunc) == 192, "cuSten_t::devFunc offset");

// The shipped Fun functions live in the shared library (builtin_funs.cu); a program linking only the
// static archive has none, and every device function takes the indirect-call path.
extern "C" int custen_builtin_fun_id(const void* f, int dtype) __attribute__((weak));

namespace custen {

// Device-side error word: bit 0 = an mbarrier wait of a TMA-staged kernel expired.
__device__ unsigned int g_custen_device_error = 0;

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};
static std::atomic<unsigned long long> g_launches_tma{0};
static std::atomic<unsigned long long> g_h2d_bytes{0};   // host -> device bytes moved by Compute
static std::atomic<unsigned long long> g_d2h_bytes{0};   // device -> host bytes moved by Compute
static std::atomic<size_t> g_stage_chunk_bytes{(size_t)32 << 20};   // staging chunk size, host-resident fields
static std::atomic<int> g_fun_fusion{1};   // run the library's own c^3 - c Fun functions as cube + weights

enum { ST_OK = 0, ST_CUDA = 1, ST_ARG = 2, ST_UNSUPPORTED = 3 };

static int fail_cuda(cudaError_t e, const char* action) {
    char buf[1024];
    snprintf(buf, sizeof(buf), "Error while '%s': %s", action, cudaGetErrorString(e));
    g_last_error = buf;
    cudaGetLastError();   // clear the sticky-free error so the next call starts clean
    return ST_CUDA;
}

static int fail_arg(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return ST_ARG;
}

#define CU_TRY(expr, action)                          \
    do {                                              \
        cudaError_t _e = (expr);                      \
        if (_e != cudaSuccess) return fail_cuda(_e, action); \
    } while (0)

static PlanPrivate* priv_of(const cuSten_t* h) {
    if (h == nullptr || h->streams == nullptr) return nullptr;
    StreamBlock* blk = reinterpret_cast<StreamBlock*>(h->streams);
    if (blk->priv.magic != kPlanMagic) return nullptr;
    return &blk->priv;
}

static inline char* byte_ptr(void* p) { return reinterpret_cast<char*>(p); }

// Periodic halo pointers from `in` (the formulas of every Y/XY Create and Swap, e.g.
// custenCreateDestroy2DYp.cu:182-216 and :248-282).
static void set_halos_periodic(cuSten_t* h, void* in, int esz) {
    const size_t nx = h->nx;
    const int nt = h->numTiles, ny = h->ny, nyT = h->nyTile, T = h->numStenTop;
    char* base = byte_ptr(in);
    for (int t = 0; t < nt; ++t) {
        long top_row = (t == 0) ? (long)(ny - T) : (long)t * nyT - T;
        long bot_row = (t == nt - 1) ? 0 : (long)(t + 1) * nyT;
        h->boundaryTop[t] = reinterpret_cast<double*>(base + top_row * (long)nx * esz);
        h->boundaryBottom[t] = reinterpret_cast<double*>(base + bot_row * (long)nx * esz);
    }
}

// Edge-clamped halo pointers of cuStenCreate2DYnp (custenCreateDestroy2DYnp.cu:182-216): the first
// tile's top and the last tile's bottom name rows of the field itself (they are never read).
static void set_halos_ynp_create(cuSten_t* h, void* in, int esz) {
    const size_t nx = h->nx;
    const int nt = h->numTiles, ny = h->ny, nyT = h->nyTile, T = h->numStenTop, B = h->numStenBottom;
    char* base = byte_ptr(in);
    for (int t = 0; t < nt; ++t) {
        long top_row = (t == 0) ? 0 : (long)t * nyT - T;
        long bot_row = (t == nt - 1) ? (long)(ny - B) : (long)(t + 1) * nyT;
        h->boundaryTop[t] = reinterpret_cast<double*>(base + top_row * (long)nx * esz);
        h->boundaryBottom[t] = reinterpret_cast<double*>(base + bot_row * (long)nx * esz);
    }
}

static int destroy_plan(cuSten_t* h);

int create_plan(cuSten_t* h, int variant, int dtype, int dev, int numTiles, int nx, int ny, int BX, int BY,
                void* out, void* in, void* coef, int H, int L, int R, int V, int T, int B, int ncoef, void* func,
                int numStenField) {
    if (h == nullptr) return fail_arg("cuSten handle is NULL");
    if (variant < 0 || variant > V_XYWENOADVP) return fail_arg("unknown stencil variant %d", variant);
    if (dtype != DT_F64 && dtype != DT_F32) return fail_arg("unknown data type %d", dtype);
    if (numTiles < 1) return fail_arg("numTiles must be >= 1 (got %d)", numTiles);
    if (nx < 1 || ny < 1) return fail_arg("nx and ny must be >= 1 (got %d x %d)", nx, ny);
    if (ny % numTiles != 0) return fail_arg("ny (%d) must be divisible by numTiles (%d)", ny, numTiles);
    if (BX < 1 || BY < 1) return fail_arg("BLOCK_X and BLOCK_Y must be >= 1");
    if (L < 0 || R < 0 || T < 0 || B < 0) return fail_arg("stencil extents must be >= 0");
    if (H < 1 || V < 1) return fail_arg("stencil size must be >= 1");
    if (H > L + R + 1 || V > T + B + 1)
        return fail_arg("stencil (%d x %d) reaches beyond its halo (L=%d R=%d T=%d B=%d)", H, V, L, R, T, B);
    const int nyTile = ny / numTiles;
    if (L >= nx || R >= nx || T > nyTile || B > nyTile)
        return fail_arg("halo larger than the field or tile (nx=%d nyTile=%d L=%d R=%d T=%d B=%d)", nx, nyTile, L,
                        R, T, B);
    const bool np = !variant_is_periodic(variant);
    if (np && (nx % BX != 0 || nyTile % BY != 0))
        return fail_arg("non-periodic stencils need nx %% BLOCK_X == 0 and nyTile %% BLOCK_Y == 0 "
                        "(nx=%d nyTile=%d BLOCK_X=%d BLOCK_Y=%d)", nx, nyTile, BX, BY);
    if (ncoef < 0 || ncoef > 4096) return fail_arg("number of weights/coefficients out of range (%d)", ncoef);
    if (ncoef > 0 && coef == nullptr) return fail_arg("weights/coefficients pointer is NULL");
    if (variant_is_fun(variant) && func == nullptr) return fail_arg("device function pointer is NULL");
    if (in == nullptr || out == nullptr) return fail_arg("data pointers must not be NULL");

    CU_TRY(cudaSetDevice(dev), "Setting current device");

    StreamBlock* blk = static_cast<StreamBlock*>(calloc(1, sizeof(StreamBlock)));
    if (!blk) return fail_arg("out of host memory");
    for (int s = 0; s < 3; ++s) {
        cudaError_t e = cudaStreamCreate(&blk->streams[s]);
        if (e != cudaSuccess) {
            for (int k = 0; k < s; ++k) cudaStreamDestroy(blk->streams[k]);
            free(blk);
            return fail_cuda(e, "Creating stream");
        }
    }
    cudaEvent_t* events = static_cast<cudaEvent_t*>(malloc(2 * sizeof(cudaEvent_t)));
    for (int ev = 0; ev < 2; ++ev) {
        cudaError_t e = cudaEventCreateWithFlags(&events[ev], cudaEventDisableTiming);
        if (e != cudaSuccess) {
            for (int k = 0; k < ev; ++k) cudaEventDestroy(events[k]);
            for (int k = 0; k < 3; ++k) cudaStreamDestroy(blk->streams[k]);
            free(events);
            free(blk);
            return fail_cuda(e, "Creating event");
        }
    }
    PlanPrivate& p = blk->priv;
    p.magic = kPlanMagic;
    p.variant = variant;
    p.dtype = dtype;
    p.H = H; p.V = V; p.L = L; p.R = R; p.T = T; p.B = B;
    p.ncoef = ncoef;
    p.mem_kind = -1;
    p.user_stream = nullptr;
    p.use_user_stream = 0;
    p.launches = 0;
    p.fused_func = nullptr;
    p.fused_pre = 0;
    p.cfg = -1;
    p.stage = nullptr;
    p.stage_slot_bytes = 0;
    p.stage_rows = 0;
    p.stage_events_ready = 0;
    p.slab = 0;
    p.slabs = 0;

    const int esz = dtype == DT_F64 ? 8 : 4;
    const int dir = variant_dir(variant);
    memset(h, 0, sizeof(*h));
    h->deviceNum = dev;
    h->numStreams = 3;
    h->numTiles = numTiles;
    h->nx = nx;
    h->ny = ny;
    h->nyTile = nyTile;
    h->numSten = numStenField;
    h->numStenLeft = L;
    h->numStenRight = R;
    h->numStenTop = T;
    h->numStenBottom = B;
    h->numStenHoriz = (dir == 2) ? H : 0;
    h->numStenVert = (dir == 2) ? V : 0;
    h->BLOCK_X = BX;
    h->BLOCK_Y = BY;
    h->xGrid = (nx % BX == 0) ? nx / BX : nx / BX + 1;
    h->yGrid = (nyTile % BY == 0) ? nyTile / BY : nyTile / BY + 1;
    h->nxLocal = BX + L + R;
    h->nyLocal = BY + T + B;
    h->mem_shared = (int)(((size_t)h->nxLocal * h->nyLocal + (size_t)ncoef) * sizeof(double));
    if (variant_is_fun(variant)) {
        h->coe = static_cast<double*>(coef);
        h->numCoe = ncoef;
        h->devFunc = static_cast<double*>(func);
    } else {
        h->weights = static_cast<double*>(coef);
    }
    h->streams = blk->streams;
    h->events = events;
    h->dataInput = static_cast<double**>(malloc(numTiles * sizeof(double*)));
    h->dataOutput = static_cast<double**>(malloc(numTiles * sizeof(double*)));
    const size_t tile_bytes = (size_t)nx * nyTile * esz;
    for (int t = 0; t < numTiles; ++t) {
        h->dataInput[t] = reinterpret_cast<double*>(byte_ptr(in) + t * tile_bytes);
        h->dataOutput[t] = reinterpret_cast<double*>(byte_ptr(out) + t * tile_bytes);
    }
    if (dir != 0) {
        h->boundaryTop = static_cast<double**>(malloc(numTiles * sizeof(double*)));
        h->boundaryBottom = static_cast<double**>(malloc(numTiles * sizeof(double*)));
        if (variant == V_YNP || variant == V_YNPFUN) set_halos_ynp_create(h, in, esz);
        else set_halos_periodic(h, in, esz);
        h->numBoundaryTop = T * nx;
        h->numBoundaryBottom = B * nx;
    }
    return ST_OK;
}

// cuStenCreate2DXYWENOADVp (custenCreateDestroy2DXYADVWENOp.cu:57-257): a 7 x 7 window (L = R = T =
// B = 3), coeDx = 1/dx, coeDy = 1/dy, per-tile input / output / velocity pointers and periodic halo
// pointers. The reference's kernel also assumes nx % BLOCK_X == 0, nyTile % BLOCK_Y == 0 and at least two
// blocks per direction; this library computes the periodic operator for any nx and any nyTile >= 3.
int create_weno_plan(cuSten_t* h, int dev, int numTiles, int nx, int ny, int BX, int BY, double dx, double dy,
                     double* u, double* v, double* out, double* in) {
    if (h == nullptr) return fail_arg("cuSten handle is NULL");
    if (u == nullptr || v == nullptr) return fail_arg("velocity pointers must not be NULL");
    if (!(dx != 0.0) || !(dy != 0.0)) return fail_arg("grid spacings must be non-zero");
    if (numTiles >= 1 && ny % numTiles == 0 && ny / numTiles < 3)
        return fail_arg("WENO needs at least 3 rows per tile (ny=%d numTiles=%d)", ny, numTiles);
    int st = create_plan(h, V_XYWENOADVP, DT_F64, dev, numTiles, nx, ny, BX, BY, out, in, nullptr, 7, 3, 3, 7, 3, 3,
                         0, nullptr, 49);
    if (st != ST_OK) return st;
    h->coeDx = 1.0 / dx;
    h->coeDy = 1.0 / dy;
    h->numStenHoriz = 7;
    h->numStenVert = 7;
    h->mem_shared = (int)(((size_t)h->nxLocal * h->nyLocal + 49) * sizeof(double));
    const size_t tile_elems = (size_t)nx * h->nyTile;
    h->uVel = static_cast<double**>(malloc(numTiles * sizeof(double*)));
    h->vVel = static_cast<double**>(malloc(numTiles * sizeof(double*)));
    for (int t = 0; t < numTiles; ++t) {
        h->uVel[t] = u + t * tile_elems;
        h->vVel[t] = v + t * tile_elems;
    }
    return ST_OK;
}

static int destroy_plan(cuSten_t* h) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    cudaSetDevice(h->deviceNum);
    StreamBlock* blk = reinterpret_cast<StreamBlock*>(h->streams);
    int st = ST_OK;
    for (int s = 0; s < 3; ++s) {
        cudaError_t e = cudaStreamDestroy(blk->streams[s]);
        if (e != cudaSuccess && st == ST_OK) st = fail_cuda(e, "Destroying stream");
    }
    for (int ev = 0; ev < 2; ++ev) {
        cudaError_t e = cudaEventDestroy(h->events[ev]);
        if (e != cudaSuccess && st == ST_OK) st = fail_cuda(e, "Destroying event");
    }
    if (blk->priv.stage_events_ready)
        for (int ev = 0; ev < 3 * kStageSlots; ++ev) cudaEventDestroy(blk->priv.stage_ev[ev]);
    if (blk->priv.stage) {
        cudaError_t e = cudaFree(blk->priv.stage);
        if (e != cudaSuccess && st == ST_OK) st = fail_cuda(e, "Freeing staging buffers");
    }
    blk->priv.magic = 0;
    free(blk);
    free(h->events);
    free(h->dataInput);
    free(h->dataOutput);
    free(h->boundaryTop);
    free(h->boundaryBottom);
    free(h->uVel);
    free(h->vVel);
    h->uVel = h->vVel = nullptr;
    h->streams = nullptr;
    h->events = nullptr;
    h->dataInput = h->dataOutput = h->boundaryTop = h->boundaryBottom = nullptr;
    return st;
}

static int swap_plan(cuSten_t* h, void* newInput) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    for (int t = 0; t < h->numTiles; ++t) {
        double* tmp = h->dataInput[t];
        h->dataInput[t] = h->dataOutput[t];
        h->dataOutput[t] = tmp;
    }
    // X variants ignore the argument (custenCreateDestroy2DXp.cu:179-190); Y and XY variants
    // recompute every halo pointer from it with the periodic formulas, Ynp included
    // (custenCreateDestroy2DYnp.cu:248-282). Slab handles keep their halo buffers (the exchange fills
    // them before each Compute) and ignore the argument.
    if (variant_dir(p->variant) != 0 && !p->slabs) {
        if (newInput == nullptr) return fail_arg("Swap needs the new input pointer for Y/XY stencils");
        set_halos_periodic(h, newInput, p->dtype == DT_F64 ? 8 : 4);
    }
    return ST_OK;
}

static int memory_kind(const void* ptr) {
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 2;
    }
    switch (at.type) {
    case cudaMemoryTypeManaged: return 1;
    case cudaMemoryTypeDevice: return 0;
    default: return 2;   // pinned or system memory: read in place (NVLink-C2C on Grace systems)
    }
}

static cudaError_t prefetch(const void* p, size_t bytes, int dev, cudaStream_t s) {
    if (p == nullptr || bytes == 0) return cudaSuccess;
    cudaMemLocation loc;
    if (dev >= 0) {
        loc.type = cudaMemLocationTypeDevice;
        loc.id = dev;
    } else {
        loc.type = cudaMemLocationTypeHost;
        loc.id = 0;
    }
    return cudaMemPrefetchAsync(p, bytes, loc, 0, s);
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

static cudaError_t launch(const StencilArgs& a, int dtype, cudaStream_t s, PlanPrivate* p) {
    int path = 0;
    cudaError_t e = a.variant == V_XYWENOADVP ? launch_weno_adv(a, s)
                                             : launch_stencil_cfg(a, dtype, p->cfg < 0 ? 0 : p->cfg, s, &path);
    if (e == cudaSuccess) {
        ++p->launches;
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (path == 1) g_launches_tma.fetch_add(1, std::memory_order_relaxed);
    }
    return e;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Copies rows [r_begin, r_end) of tile t's input, in tile-local numbering, to dst. Rows below 0
// come from the tile's top halo rows, rows at or past nyTile from its bottom halo rows (the
// handle's boundaryTop/boundaryBottom pointers, as the reference's per-tile kernels read them).
static cudaError_t copy_tile_rows(const cuSten_t* h, int t, int r_begin, int r_end, char* dst, size_t row_bytes,
                                  int T, cudaStream_t s, unsigned long long* moved) {
    const int nyT = h->nyTile;
    while (r_begin < r_end) {
        const char* src;
        int seg_end;
        if (r_begin < 0) {
            src = reinterpret_cast<const char*>(h->boundaryTop[t]) + (size_t)(T + r_begin) * row_bytes;
            seg_end = r_end < 0 ? r_end : 0;
        } else if (r_begin < nyT) {
            src = reinterpret_cast<const char*>(h->dataInput[t]) + (size_t)r_begin * row_bytes;
            seg_end = r_end < nyT ? r_end : nyT;
        } else {
            src = reinterpret_cast<const char*>(h->boundaryBottom[t]) + (size_t)(r_begin - nyT) * row_bytes;
            seg_end = r_end;
        }
        const size_t bytes = (size_t)(seg_end - r_begin) * row_bytes;
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s);
        if (e != cudaSuccess) return e;
        *moved += bytes;
        dst += bytes;
        r_begin = seg_end;
    }
    return cudaSuccess;
}

// Untouched output columns of a non-periodic chunk: the first lw and the last rw 4-byte words of each of
// `rows` rows, read in place from device-accessible (pinned or registered) host memory into the output
// slot. One small gather per chunk instead of two strided copies of a few bytes per row, which the copy
// engines move one row at a time.
__global__ void stage_edge_columns_kernel(uint32_t* slot, const uint32_t* host, size_t row_words, int rows, int lw,
                                          int rw) {
    const int per_row = lw + rw;
    const long long total = (long long)rows * per_row;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / per_row;
        const int k = (int)(e - r * per_row);
        const size_t col = k < lw ? (size_t)k : row_words - (size_t)rw + (size_t)(k - lw);
        slot[(size_t)r * row_words + col] = host[(size_t)r * row_words + col];
    }
}

// Device address of host memory the GPU can read in place (pinned or registered), else null.
static const char* mapped_host(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? static_cast<const char*>(at.devicePointer) : nullptr;
}

// Host-resident fields: the rows of every tile stream through device staging slots in chunks.
// Chunk c copies its input rows and halo rows in on s_in, computes on s_comp and copies its output
// rows back on s_out; kStageSlots chunks are in flight, so the two copy directions and the
// kernels overlap. For the non-periodic variants the cells a Compute leaves untouched (the field's
// first L and last max(L, R) columns, its first T and last B rows) are copied in first, so that the
// whole chunk can be copied back unchanged.
static int compute_staged(cuSten_t* h, PlanPrivate* p, StencilArgs& a, cudaStream_t s_comp, cudaStream_t s_in,
                          cudaStream_t s_out) {
    const int esz = p->dtype == DT_F64 ? 8 : 4;
    const int nt = h->numTiles, nx = h->nx, ny = h->ny, nyT = h->nyTile;
    const int dir = variant_dir(p->variant);
    const bool periodic = variant_is_periodic(p->variant);
    const int T = p->T, B = p->B;
    const size_t row_bytes = (size_t)nx * esz;
    if (!p->stage) {
        // Chunks of about 32 MiB (custen_set_stage_chunk_bytes), a multiple of 32 rows where the tile
        // allows (the TMA kernel's tile height), and never shorter than a halo.
        const size_t target = g_stage_chunk_bytes.load();
        int rows = (int)std::max<size_t>(1, target / row_bytes);
        if (rows >= 32) rows -= rows % 32;
        rows = std::max(rows, std::max(T, B));
        rows = std::min(rows, nyT);
        const size_t in_bytes = align256((size_t)(T + rows + B) * row_bytes);
        const size_t out_bytes = align256((size_t)rows * row_bytes);
        // WENO advection also streams its two velocity fields
        const size_t slot = in_bytes + out_bytes * (p->variant == V_XYWENOADVP ? 3 : 1);
        const size_t coef_bytes = align256((size_t)std::max(p->ncoef, 1) * esz);
        CU_TRY(cudaMalloc(&p->stage, kStageSlots * slot + coef_bytes), "Allocating staging buffers");
        p->stage_slot_bytes = slot;
        p->stage_rows = rows;
    }
    if (!p->stage_events_ready) {
        for (int ev = 0; ev < 3 * kStageSlots; ++ev)
            CU_TRY(cudaEventCreateWithFlags(&p->stage_ev[ev], cudaEventDisableTiming), "Creating event");
        p->stage_events_ready = 1;
    }
    const int rows = p->stage_rows;
    const size_t slot_bytes = p->stage_slot_bytes;
    const size_t in_bytes = align256((size_t)(T + rows + B) * row_bytes);
    char* stage = static_cast<char*>(p->stage);
    char* coef_dev = stage + kStageSlots * slot_bytes;
    unsigned long long h2d = 0, d2h = 0;

    // Weights (or Fun coefficients) once per Compute: the kernels then read device memory only.
    // The copy waits for every kernel of the previous Compute that may still read the old ones.
    for (int k = 0; k < kStageSlots; ++k) CU_TRY(cudaStreamWaitEvent(s_in, p->stage_ev[3 * k + 1], 0), "Ordering");
    if (p->ncoef > 0 && a.coef != nullptr) {
        CU_TRY(cudaMemcpyAsync(coef_dev, a.coef, (size_t)p->ncoef * esz, cudaMemcpyDefault, s_in), "Copying weights");
        h2d += (size_t)p->ncoef * esz;
        a.coef = coef_dev;
    }
    const int wl = std::max(p->L, p->R);
    int c = 0;
    for (int t = 0; t < nt; ++t) {
        // untouched output columns are gathered by a kernel where the output tile is mapped host memory
        const char* out_mapped = (!periodic && dir != 1) ? mapped_host(h->dataOutput[t]) : nullptr;
        for (int r0 = 0; r0 < nyT; r0 += rows, ++c) {
            const int rc = std::min(rows, nyT - r0);
            const int k = c % kStageSlots;
            cudaEvent_t ev_in = p->stage_ev[3 * k], ev_kern = p->stage_ev[3 * k + 1], ev_out = p->stage_ev[3 * k + 2];
            char* in_slot = stage + (size_t)k * slot_bytes;
            char* out_slot = in_slot + in_bytes;
            char* u_slot = out_slot + align256((size_t)rows * row_bytes);
            char* v_slot = u_slot + align256((size_t)rows * row_bytes);
            const int gy0 = t * nyT + r0;
            const bool has_top = dir != 0 && T > 0 && (periodic || gy0 > 0);
            const bool has_bot = dir != 0 && B > 0 && (periodic || gy0 + rc < ny);
            // the slot is free once its previous kernel and its previous copy-out are done
            CU_TRY(cudaStreamWaitEvent(s_in, ev_kern, 0), "Ordering copy after kernel");
            CU_TRY(cudaStreamWaitEvent(s_in, ev_out, 0), "Ordering copy after copy-out");
            char* body = in_slot + (size_t)T * row_bytes;
            CU_TRY(copy_tile_rows(h, t, has_top ? r0 - T : r0, r0 + rc + (has_bot ? B : 0),
                                  has_top ? in_slot : body, row_bytes, T, s_in, &h2d),
                   "Copying input rows to the device");
            if (!periodic) {
                char* host_out = reinterpret_cast<char*>(h->dataOutput[t]) + (size_t)r0 * row_bytes;
                if (dir != 0) {
                    // field rows [0, T) and [ny - B, ny) that fall in this chunk
                    const int lo[2] = {0, ny - B}, hi[2] = {T, ny};
                    for (int q = 0; q < 2; ++q) {
                        const int a0 = std::max(lo[q], gy0), a1 = std::min(hi[q], gy0 + rc);
                        if (a1 <= a0) continue;
                        const size_t off = (size_t)(a0 - gy0) * row_bytes, bytes = (size_t)(a1 - a0) * row_bytes;
                        CU_TRY(cudaMemcpyAsync(out_slot + off, host_out + off, bytes, cudaMemcpyDefault, s_in),
                               "Copying untouched output rows");
                        h2d += bytes;
                    }
                }
                const int lw_words = p->L * esz / 4, rw_words = wl * esz / 4;
                if (dir != 1 && out_mapped != nullptr && lw_words + rw_words > 0) {
                    const long long words = (long long)rc * (lw_words + rw_words);
                    const int blocks = (int)std::min<long long>((words + 255) / 256, 1024);
                    stage_edge_columns_kernel<<<blocks, 256, 0, s_in>>>(
                        reinterpret_cast<uint32_t*>(out_slot),
                        reinterpret_cast<const uint32_t*>(out_mapped + (size_t)r0 * row_bytes), row_bytes / 4, rc,
                        lw_words, rw_words);
                    CU_TRY(cudaGetLastError(), "Copying untouched output columns");
                    h2d += (size_t)(lw_words + rw_words) * 4 * rc;
                } else if (dir != 1) {
                    if (p->L > 0) {
                        CU_TRY(cudaMemcpy2DAsync(out_slot, row_bytes, host_out, row_bytes, (size_t)p->L * esz, rc,
                                                 cudaMemcpyDefault, s_in),
                               "Copying untouched output columns");
                        h2d += (size_t)p->L * esz * rc;
                    }
                    if (wl > 0) {
                        const size_t off = (size_t)(nx - wl) * esz;
                        CU_TRY(cudaMemcpy2DAsync(out_slot + off, row_bytes, host_out + off, row_bytes, (size_t)wl * esz,
                                                 rc, cudaMemcpyDefault, s_in),
                               "Copying untouched output columns");
                        h2d += (size_t)wl * esz * rc;
                    }
                }
            }
            if (p->variant == V_XYWENOADVP) {
                const size_t off = (size_t)r0 * row_bytes, bytes = (size_t)rc * row_bytes;
                CU_TRY(cudaMemcpyAsync(u_slot, byte_ptr(h->uVel[t]) + off, bytes, cudaMemcpyDefault, s_in),
                       "Copying velocity rows to the device");
                CU_TRY(cudaMemcpyAsync(v_slot, byte_ptr(h->vVel[t]) + off, bytes, cudaMemcpyDefault, s_in),
                       "Copying velocity rows to the device");
                h2d += 2 * bytes;
                a.u = u_slot;
                a.v = v_slot;
            }
            CU_TRY(cudaEventRecord(ev_in, s_in), "Recording event");
            CU_TRY(cudaStreamWaitEvent(s_comp, ev_in, 0), "Ordering kernel after copy-in");
            a.in = body;
            a.out = out_slot;
            a.rows = rc;
            a.row0 = gy0;
            a.top = in_slot;
            a.bot = body + (size_t)rc * row_bytes;
            a.has_top = has_top;
            a.has_bot = has_bot;
            a.vec_ok = row_bytes % 16 == 0;
            CU_TRY(launch(a, p->dtype, s_comp, p), "Computing stencil chunk");
            CU_TRY(cudaEventRecord(ev_kern, s_comp), "Recording event");
            CU_TRY(cudaStreamWaitEvent(s_out, ev_kern, 0), "Ordering copy-out after kernel");
            char* host_out = reinterpret_cast<char*>(h->dataOutput[t]) + (size_t)r0 * row_bytes;
            CU_TRY(cudaMemcpyAsync(host_out, out_slot, (size_t)rc * row_bytes, cudaMemcpyDefault, s_out),
                   "Copying output rows to the host");
            d2h += (size_t)rc * row_bytes;
            CU_TRY(cudaEventRecord(ev_out, s_out), "Recording event");
        }
    }
    // Work issued later on the compute stream follows the last copy-out.
    for (int k = 0; k < kStageSlots; ++k)
        CU_TRY(cudaStreamWaitEvent(s_comp, p->stage_ev[3 * k + 2], 0), "Ordering compute after copies");
    g_h2d_bytes.fetch_add(h2d, std::memory_order_relaxed);
    g_d2h_bytes.fetch_add(d2h, std::memory_order_relaxed);
    return ST_OK;
}

int compute_plan(cuSten_t* h, int offload, cudaStream_t* explicit_stream) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    CU_TRY(cudaSetDevice(h->deviceNum), "Setting current device");
    cudaStream_t s = explicit_stream ? *explicit_stream : (p->use_user_stream ? p->user_stream : h->streams[0]);
    cudaStream_t copy_s = explicit_stream ? *explicit_stream : (p->use_user_stream ? p->user_stream : h->streams[1]);
    const int esz = p->dtype == DT_F64 ? 8 : 4;
    const int nt = h->numTiles, nx = h->nx, nyT = h->nyTile;
    const int dir = variant_dir(p->variant);
    const bool periodic = variant_is_periodic(p->variant);
    const size_t tile_bytes = (size_t)nx * nyT * esz;

    StencilArgs a;
    memset(&a, 0, sizeof(a));
    a.coef = variant_is_fun(p->variant) ? (const void*)h->coe : (const void*)h->weights;
    a.func = variant_is_fun(p->variant) ? (void*)h->devFunc : nullptr;
    a.nx = nx;
    a.L = p->L; a.R = p->R; a.T = p->T; a.B = p->B;
    a.H = p->H; a.V = p->V;
    a.ncoef = p->ncoef;
    a.variant = p->variant;
    a.bx = h->BLOCK_X;
    a.by = h->BLOCK_Y;
    a.nyTile = nyT;
    // a slab handle's tile is tile p->slab of p->slabs: the write rules and the halo rule take the
    // field-wide tile numbering, rows are numbered from the field's first row
    const int tile0 = p->slabs ? p->slab : 0, tiles_all = p->slabs ? p->slabs : nt;
    a.numTiles = tiles_all;
    a.wrap_x = periodic && dir != 1;
    if (variant_is_fun(p->variant) && g_fun_fusion.load(std::memory_order_relaxed)) {
        // The library's own c^3 - c functions (ids 1, 3, 5) with the window they read: cube each staged
        // value once, then apply the coefficients as plain weights (bit-identical, fewer FP64 operations).
        if (h->devFunc != p->fused_func) {
            p->fused_func = h->devFunc;
            const int id = custen_builtin_fun_id ? custen_builtin_fun_id(h->devFunc, p->dtype) : -1;
            p->fused_pre = (id == 1 && dir == 0 && p->L == 2 && p->R == 2 && p->ncoef == 5) ||
                           (id == 3 && dir == 1 && p->T == 2 && p->B == 2 && p->ncoef == 5) ||
                           (id == 5 && dir == 2 && p->ncoef == p->H * p->V);
        }
        a.pre = p->fused_pre;
    }
    if (p->variant == V_XYWENOADVP) {
        // the reference passes coeDx / coeDy from the handle at every Compute (2d_xyADVWENO_p_kernel.cu:479-480)
        a.cdx = h->coeDx;
        a.cdy = h->coeDy;
        a.coef = nullptr;
    }

    // Tiles contiguous and every interior halo pointer naming the neighbouring rows of that array?
    char* in0 = byte_ptr(h->dataInput[0]);
    char* out0 = byte_ptr(h->dataOutput[0]);
    const bool weno = p->variant == V_XYWENOADVP;
    bool contiguous = true;
    for (int t = 0; t < nt && contiguous; ++t) {
        if (byte_ptr(h->dataInput[t]) != in0 + t * tile_bytes) contiguous = false;
        if (byte_ptr(h->dataOutput[t]) != out0 + t * tile_bytes) contiguous = false;
        if (weno && (byte_ptr(h->uVel[t]) != byte_ptr(h->uVel[0]) + t * tile_bytes ||
                     byte_ptr(h->vVel[t]) != byte_ptr(h->vVel[0]) + t * tile_bytes))
            contiguous = false;
        if (dir != 0 && contiguous) {
            if (t > 0 && p->T > 0 &&
                byte_ptr(h->boundaryTop[t]) != in0 + ((long)t * nyT - p->T) * (long)nx * esz)
                contiguous = false;
            if (t < nt - 1 && p->B > 0 && byte_ptr(h->boundaryBottom[t]) != in0 + (long)(t + 1) * nyT * nx * esz)
                contiguous = false;
        }
    }

    const int kind = memory_kind(in0);
    const int kind_out = memory_kind(out0);
    p->mem_kind = kind;
    const bool row_aligned = ((size_t)nx * esz) % 16 == 0;

    auto fill_launch = [&](int t_first, int t_count) {
        a.in = h->dataInput[t_first];
        a.out = h->dataOutput[t_first];
        if (weno) {
            a.u = h->uVel[t_first];
            a.v = h->vVel[t_first];
        }
        a.rows = t_count * nyT;
        a.row0 = (tile0 + t_first) * nyT;
        const int t_last = t_first + t_count - 1;
        a.top = (dir != 0) ? (const void*)h->boundaryTop[t_first] : nullptr;
        a.bot = (dir != 0) ? (const void*)h->boundaryBottom[t_last] : nullptr;
        a.has_top = (dir != 0 && p->T > 0) && (periodic || tile0 + t_first > 0);
        a.has_bot = (dir != 0 && p->B > 0) && (periodic || tile0 + t_last < tiles_all - 1);
        a.vec_ok = row_aligned && aligned16(a.in) && aligned16(a.out) && (!a.has_top || aligned16(a.top)) &&
                   (!a.has_bot || aligned16(a.bot));
    };

    if (kind == 2 || kind_out == 2) {
        if (p->slabs) return fail_arg("slab handles take device or managed memory");
        // Pinned or system memory: stream the rows through device staging slots.
        cudaStream_t s_out = explicit_stream ? *explicit_stream
                                             : (p->use_user_stream ? p->user_stream : h->streams[2]);
        return compute_staged(h, p, a, s, copy_s, s_out);
    }
    if (kind != 1) {
        // Device-resident data: no copies. The first Compute picks the kernel configuration (autotune.cu).
        if (p->cfg < 0 && p->variant != V_XYWENOADVP) {
            fill_launch(0, contiguous ? nt : 1);
            p->cfg = choose_config(a, p->dtype, s, p->cfg == -2, 3);
        }
        if (contiguous) {
            fill_launch(0, nt);
            CU_TRY(launch(a, p->dtype, s, p), "Computing stencil");
        } else {
            for (int t = 0; t < nt; ++t) {
                fill_launch(t, 1);
                CU_TRY(launch(a, p->dtype, s, p), "Computing stencil tile");
            }
        }
        return ST_OK;
    }

    // Managed memory: stream the tiles through the GPU as the reference does
    // (cuSten/src/kernels/2d_x_p_kernel.cu:216-271): prefetch tile t+1 (and its halo rows) on the copy
    // stream while tile t computes; with HOST offload send each finished tile back to the host.
    // The ordering is expressed with events, so the host never blocks.
    const int dev = h->deviceNum;
    const size_t halo_top_bytes = (size_t)p->T * nx * esz, halo_bot_bytes = (size_t)p->B * nx * esz;
    CU_TRY(prefetch(a.coef, (size_t)p->ncoef * esz, dev, copy_s), "Prefetching weights");
    unsigned long long moved_in = 0, moved_out = 0;
    auto prefetch_tile = [&](int t) -> cudaError_t {
        moved_in += 2 * tile_bytes + (dir != 0 ? halo_top_bytes + halo_bot_bytes : 0);
        cudaError_t e = prefetch(h->dataInput[t], tile_bytes, dev, copy_s);
        if (e == cudaSuccess) e = prefetch(h->dataOutput[t], tile_bytes, dev, copy_s);
        if (e == cudaSuccess && weno) e = prefetch(h->uVel[t], tile_bytes, dev, copy_s);
        if (e == cudaSuccess && weno) e = prefetch(h->vVel[t], tile_bytes, dev, copy_s);
        if (weno) moved_in += 2 * tile_bytes;
        if (e == cudaSuccess && dir != 0 && halo_top_bytes) e = prefetch(h->boundaryTop[t], halo_top_bytes, dev, copy_s);
        if (e == cudaSuccess && dir != 0 && halo_bot_bytes) e = prefetch(h->boundaryBottom[t], halo_bot_bytes, dev, copy_s);
        if (e == cudaSuccess) e = cudaEventRecord(h->events[t & 1], copy_s);
        return e;
    };
    CU_TRY(prefetch_tile(0), "Prefetching tile");
    for (int t = 0; t < nt; ++t) {
        CU_TRY(cudaStreamWaitEvent(s, h->events[t & 1], 0), "Ordering tile after prefetch");
        fill_launch(t, 1);
        CU_TRY(launch(a, p->dtype, s, p), "Computing stencil tile");
        if (offload == HOST) {
            moved_out += 2 * tile_bytes;
            CU_TRY(prefetch(h->dataOutput[t], tile_bytes, -1, s), "Offloading output tile");
            CU_TRY(prefetch(h->dataInput[t], tile_bytes, -1, s), "Offloading input tile");
            if (weno) {
                moved_out += 2 * tile_bytes;
                CU_TRY(prefetch(h->uVel[t], tile_bytes, -1, s), "Offloading velocity tile");
                CU_TRY(prefetch(h->vVel[t], tile_bytes, -1, s), "Offloading velocity tile");
            }
        }
        if (t + 1 < nt) CU_TRY(prefetch_tile(t + 1), "Prefetching tile");
    }
    if (copy_s != s) {
        // Later work on the compute stream must also follow the last prefetch.
        CU_TRY(cudaEventRecord(h->events[0], copy_s), "Recording event");
        CU_TRY(cudaStreamWaitEvent(s, h->events[0], 0), "Ordering compute after copies");
    }
    g_h2d_bytes.fetch_add(moved_in, std::memory_order_relaxed);
    g_d2h_bytes.fetch_add(moved_out, std::memory_order_relaxed);
    return ST_OK;
}

}  // namespace custen

using namespace custen;

// ---------------------------------------------------------------------------------------------
// Reference C++ API (exit on error, as cuSten/src/util/error.cu:43-53 does)
// ---------------------------------------------------------------------------------------------

void checkError(const char* action) {
    cudaError_t error = cudaGetLastError();
    if (error != cudaSuccess) {
        printf("\nError while '%s': %s\nprogram terminated ...\n\n", action, cudaGetErrorString(error));
        exit(EXIT_FAILURE);
    }
}

static void exit_on(int st) {
    if (st != ST_OK) {
        printf("\n%s\nprogram terminated ...\n\n", g_last_error.c_str());
        exit(EXIT_FAILURE);
    }
}

// ---- X ----
void cuStenCreate2DXp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                      double* w, int numSten, int L, int R) {
    exit_on(create_plan(h, V_XP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, numSten, L, R, 1, 0, 0, numSten,
                        nullptr, numSten));
}
void cuStenCreate2DXnp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                       double* w, int numSten, int L, int R) {
    exit_on(create_plan(h, V_XNP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, numSten, L, R, 1, 0, 0, numSten,
                        nullptr, numSten));
}
void cuStenCreate2DXpFun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                         double* coe, int numSten, int L, int R, int numCoe, double* func) {
    exit_on(create_plan(h, V_XPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, L + R + 1, L, R, 1, 0, 0,
                        numCoe, func, numSten));
}
void cuStenCreate2DXnpFun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                          double* coe, int numSten, int L, int R, int numCoe, double* func) {
    exit_on(create_plan(h, V_XNPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, L + R + 1, L, R, 1, 0, 0,
                        numCoe, func, numSten));
}
// ---- Y ----
void cuStenCreate2DYp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                      double* w, int numSten, int T, int B) {
    exit_on(create_plan(h, V_YP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, 1, 0, 0, numSten, T, B, numSten,
                        nullptr, numSten));
}
void cuStenCreate2DYnp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                       double* w, int numSten, int T, int B) {
    exit_on(create_plan(h, V_YNP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, 1, 0, 0, numSten, T, B, numSten,
                        nullptr, numSten));
}
void cuStenCreate2DYpFun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                         double* coe, int numSten, int T, int B, int numCoe, double* func) {
    exit_on(create_plan(h, V_YPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, 1, 0, 0, T + B + 1, T, B,
                        numCoe, func, numSten));
}
void cuStenCreate2DYnpFun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                          double* coe, int numSten, int T, int B, double* func) {
    // kernel2DYnpFun copies numSten coefficients (2d_y_np_fun_kernel.cu:102).
    exit_on(create_plan(h, V_YNPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, 1, 0, 0, T + B + 1, T, B,
                        numSten, func, numSten));
}
// ---- XY ----
void cuStenCreate2DXYp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                       double* w, int Hs, int L, int R, int Vs, int T, int B) {
    exit_on(create_plan(h, V_XYP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, Hs, L, R, Vs, T, B, Hs * Vs,
                        nullptr, Hs * Vs));
}
void cuStenCreate2DXYnp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                        double* w, int Hs, int L, int R, int Vs, int T, int B) {
    exit_on(create_plan(h, V_XYNP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, Hs, L, R, Vs, T, B, Hs * Vs,
                        nullptr, Hs * Vs));
}
void cuStenCreate2DXYpFun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                          double* coe, int Hs, int L, int R, int Vs, int T, int B, double* func) {
    // kernel2DXYpFun copies numSten = H*V coefficients (2d_xy_p_fun_kernel.cu:114-118).
    exit_on(create_plan(h, V_XYPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, Hs, L, R, Vs, T, B, Hs * Vs,
                        func, Hs * Vs));
}
void cuStenCreate2DXYnpFun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                           double* coe, int Hs, int L, int R, int Vs, int T, int B, double* func) {
    exit_on(create_plan(h, V_XYNPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, Hs, L, R, Vs, T, B, Hs * Vs,
                        func, Hs * Vs));
}

#define CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(SUFFIX)                                                  \
    void cuStenSwap2D##SUFFIX(cuSten_t* h, double* dataInput) { exit_on(swap_plan(h, dataInput)); }  \
    void cuStenDestroy2D##SUFFIX(cuSten_t* h) { exit_on(destroy_plan(h)); }                          \
    void cuStenCompute2D##SUFFIX(cuSten_t* h, bool offload) { exit_on(compute_plan(h, offload ? 1 : 0, nullptr)); }

CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(Xp)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(Xnp)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XpFun)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XnpFun)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(Yp)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(Ynp)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(YpFun)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(YnpFun)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XYp)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XYnp)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XYpFun)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XYnpFun)
CUSTEN_DEFINE_SWAP_DESTROY_COMPUTE(XYWENOADVp)

// ---- XY WENO advection, periodic (cuSten_struct_functions.h:290-347, stencil_kernels.h:181-189) ----
void cuStenCreate2DXYWENOADVp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double dx, double dy,
                              double* u, double* v, double* out, double* in) {
    exit_on(create_weno_plan(h, dev, nt, nx, ny, bx, by, dx, dy, u, v, out, in));
}

// The reference library defines the XpFun compute under this misspelt name (2d_x_p_fun_kernel.cu:172).
void cuSenCompute2DXpFun(cuSten_t* h, bool offload) { exit_on(compute_plan(h, offload ? 1 : 0, nullptr)); }

// ---------------------------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

int custen_abi_version(void) { return 1; }
int custen_sizeof_handle(void) { return (int)sizeof(cuSten_t); }
const char* custen_last_error(void) { return g_last_error.c_str(); }
unsigned long long custen_kernel_launches(void) { return g_launches.load(); }
unsigned long long custen_kernel_launches_tma(void) { return g_launches_tma.load(); }
void custen_set_fun_fusion(int enable) { g_fun_fusion.store(enable ? 1 : 0); }
void custen_set_autotune(int mode) { set_autotune_mode(mode); }
void custen_set_tune_cache(const char* path) { set_tune_cache(path); }
int custen_tune_cache_path(char* buf, size_t len) {
    const std::string p = tune_cache_path();
    if (!buf || len == 0) return fail_arg("buffer is NULL");
    snprintf(buf, len, "%s", p.c_str());
    return ST_OK;
}
int custen_autotune(cuSten_t* h, int reps) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    if (p->variant == V_XYWENOADVP) return fail_arg("the WENO operator has a single kernel configuration");
    CU_TRY(cudaSetDevice(h->deviceNum), "Setting current device");
    if (memory_kind(h->dataInput[0]) != 0 || memory_kind(h->dataOutput[0]) != 0)
        return fail_arg("autotuning needs device-resident fields");
    (void)reps;
    p->cfg = -2;   // the next Compute tunes its launch geometry, whatever the mode and the cache hold
    return compute_plan(h, DEVICE, nullptr);
}
int custen_set_config(cuSten_t* h, int index) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    if (index < -1 || index >= kNumConfigs) return fail_arg("configuration index %d out of range", index);
    p->cfg = index;   // -1: choose again at the next Compute
    return ST_OK;
}
int custen_handle_config(const cuSten_t* h, char* name, size_t len) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    if (!name || len == 0) return fail_arg("buffer is NULL");
    snprintf(name, len, "%s", p->variant == V_XYWENOADVP ? "weno_tw64_th32" : config_name(p->dtype, p->cfg < 0 ? 0 : p->cfg));
    return ST_OK;
}
void custen_set_stage_chunk_bytes(size_t bytes) { g_stage_chunk_bytes.store(bytes ? bytes : (size_t)32 << 20); }
void custen_transfer_bytes(unsigned long long* h2d, unsigned long long* d2h) {
    if (h2d) *h2d = g_h2d_bytes.load();
    if (d2h) *d2h = g_d2h_bytes.load();
}

int custen_create(cuSten_t* h, int variant, int dtype, int dev, int nt, int nx, int ny, int bx, int by, void* out,
                  void* in, void* coef, int H, int L, int R, int V, int T, int B, int ncoef, void* func) {
    if (variant == V_XYWENOADVP)
        return fail_arg("the WENO advection stencil is created with custen_create_2d_xyweno_adv_p");
    const int dir = (variant >= 0 && variant < V_COUNT) ? variant_dir(variant) : 0;
    const int field = dir == 2 ? H * V : (dir == 0 ? H : V);
    return create_plan(h, variant, dtype, dev, nt, nx, ny, bx, by, out, in, coef, H, L, R, V, T, B, ncoef, func,
                       field);
}
int custen_create_slab(cuSten_t* h, int variant, int dtype, int dev, int slab, int num_slabs, int nx, int ny_slab,
                       int bx, int by, void* out, void* in, void* halo_top, void* halo_bottom, void* coef, int H, int L,
                       int R, int V, int T, int B, int ncoef, void* func) {
    if (variant == V_XYWENOADVP) return fail_arg("slab handles take the twelve weighted / Fun variants");
    if (num_slabs < 1 || slab < 0 || slab >= num_slabs)
        return fail_arg("slab %d of %d: the index must lie in [0, num_slabs)", slab, num_slabs);
    if (ny_slab < 1 || (long long)ny_slab * num_slabs > (1ll << 31) - 1) return fail_arg("slab rows out of range");
    const int dir = (variant >= 0 && variant < V_COUNT) ? variant_dir(variant) : 0;
    const bool periodic = variant >= 0 && variant < V_COUNT && variant_is_periodic(variant);
    if (dir != 0) {
        if (T > 0 && (periodic || slab > 0) && halo_top == nullptr)
            return fail_arg("slab %d reads %d halo rows above it: halo_top is NULL", slab, T);
        if (B > 0 && (periodic || slab < num_slabs - 1) && halo_bottom == nullptr)
            return fail_arg("slab %d reads %d halo rows below it: halo_bottom is NULL", slab, B);
    }
    const int field = dir == 2 ? H * V : (dir == 0 ? H : V);
    int st = create_plan(h, variant, dtype, dev, 1, nx, ny_slab, bx, by, out, in, coef, H, L, R, V, T, B, ncoef, func,
                         field);
    if (st != ST_OK) return st;
    PlanPrivate* p = priv_of(h);
    p->slab = slab;
    p->slabs = num_slabs;
    h->ny = ny_slab * num_slabs;
    if (dir != 0) {
        h->boundaryTop[0] = static_cast<double*>(halo_top);
        h->boundaryBottom[0] = static_cast<double*>(halo_bottom);
    }
    return ST_OK;
}
int custen_compute(cuSten_t* h, int offload) { return compute_plan(h, offload, nullptr); }
int custen_compute_group(cuSten_t* const* handles, int count, int offload, void* stream) {
    if (count < 0 || (count > 0 && handles == nullptr)) return fail_arg("custen_compute_group: no handles");
    for (int k = 0; k < count; ++k) {
        if (!priv_of(handles[k])) return fail_arg("custen_compute_group: handle %d was not created by this library", k);
        for (int j = 0; j < k; ++j)
            if (handles[j] == handles[k]) return fail_arg("custen_compute_group: handle %d appears twice", k);
        if (handles[k]->deviceNum != handles[0]->deviceNum)
            return fail_arg("custen_compute_group: handle %d is on device %d, handle 0 on device %d", k,
                            handles[k]->deviceNum, handles[0]->deviceNum);
    }
    if (count == 0) return ST_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CU_TRY(cudaSetDevice(handles[0]->deviceNum), "Setting current device");
    // fork: every handle's first stream follows the work already queued on `stream`
    CU_TRY(cudaEventRecord(handles[0]->events[1], s), "Recording the group's fork event");
    for (int k = 0; k < count; ++k)
        CU_TRY(cudaStreamWaitEvent(handles[k]->streams[0], handles[0]->events[1], 0), "Ordering a group member");
    // each handle's Compute, all of its work on its own first stream
    for (int k = 0; k < count; ++k) {
        cudaStream_t hs = handles[k]->streams[0];
        const int st = compute_plan(handles[k], offload, &hs);
        if (st != ST_OK) return st;
    }
    // join: later work on `stream` follows every member
    for (int k = 0; k < count; ++k) {
        CU_TRY(cudaEventRecord(handles[k]->events[0], handles[k]->streams[0]), "Recording a group member's end");
        CU_TRY(cudaStreamWaitEvent(s, handles[k]->events[0], 0), "Joining the group");
    }
    return ST_OK;
}
int custen_compute_on_stream(cuSten_t* h, int offload, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return compute_plan(h, offload, &s);
}
int custen_swap(cuSten_t* h, void* in) { return swap_plan(h, in); }
int custen_destroy(cuSten_t* h) { return destroy_plan(h); }
int custen_set_stream(cuSten_t* h, void* stream) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    p->user_stream = static_cast<cudaStream_t>(stream);
    p->use_user_stream = stream != nullptr;
    return ST_OK;
}
int custen_handle_variant(const cuSten_t* h, int* variant, int* dtype) {
    PlanPrivate* p = priv_of(h);
    if (!p) return fail_arg("cuSten handle was not created by this library (or was destroyed)");
    if (variant) *variant = p->variant;
    if (dtype) *dtype = p->dtype;
    return ST_OK;
}

int custen_create_2d_xp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                        double* w, int numSten, int L, int R) {
    return create_plan(h, V_XP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, numSten, L, R, 1, 0, 0, numSten,
                       nullptr, numSten);
}
int custen_create_2d_xnp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                         double* w, int numSten, int L, int R) {
    return create_plan(h, V_XNP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, numSten, L, R, 1, 0, 0, numSten,
                       nullptr, numSten);
}
int custen_create_2d_xp_fun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out,
                            double* in, double* coe, int numSten, int L, int R, int numCoe, double* func) {
    return create_plan(h, V_XPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, L + R + 1, L, R, 1, 0, 0,
                       numCoe, func, numSten);
}
int custen_create_2d_xnp_fun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out,
                             double* in, double* coe, int numSten, int L, int R, int numCoe, double* func) {
    return create_plan(h, V_XNPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, L + R + 1, L, R, 1, 0, 0,
                       numCoe, func, numSten);
}
int custen_create_2d_yp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                        double* w, int numSten, int T, int B) {
    return create_plan(h, V_YP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, 1, 0, 0, numSten, T, B, numSten,
                       nullptr, numSten);
}
int custen_create_2d_ynp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                         double* w, int numSten, int T, int B) {
    return create_plan(h, V_YNP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, 1, 0, 0, numSten, T, B, numSten,
                       nullptr, numSten);
}
int custen_create_2d_yp_fun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out,
                            double* in, double* coe, int numSten, int T, int B, int numCoe, double* func) {
    return create_plan(h, V_YPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, 1, 0, 0, T + B + 1, T, B,
                       numCoe, func, numSten);
}
int custen_create_2d_ynp_fun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out,
                             double* in, double* coe, int numSten, int T, int B, double* func) {
    return create_plan(h, V_YNPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, 1, 0, 0, T + B + 1, T, B,
                       numSten, func, numSten);
}
int custen_create_2d_xyp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                         double* w, int Hs, int L, int R, int Vs, int T, int B) {
    return create_plan(h, V_XYP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, Hs, L, R, Vs, T, B, Hs * Vs,
                       nullptr, Hs * Vs);
}
int custen_create_2d_xynp(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out, double* in,
                          double* w, int Hs, int L, int R, int Vs, int T, int B) {
    return create_plan(h, V_XYNP, DT_F64, dev, nt, nx, ny, bx, by, out, in, w, Hs, L, R, Vs, T, B, Hs * Vs,
                       nullptr, Hs * Vs);
}
int custen_create_2d_xyp_fun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out,
                             double* in, double* coe, int Hs, int L, int R, int Vs, int T, int B, double* func) {
    return create_plan(h, V_XYPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, Hs, L, R, Vs, T, B, Hs * Vs,
                       func, Hs * Vs);
}
int custen_create_2d_xynp_fun(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double* out,
                              double* in, double* coe, int Hs, int L, int R, int Vs, int T, int B, double* func) {
    return create_plan(h, V_XYNPFUN, DT_F64, dev, nt, nx, ny, bx, by, out, in, coe, Hs, L, R, Vs, T, B, Hs * Vs,
                       func, Hs * Vs);
}

int custen_create_2d_xyweno_adv_p(cuSten_t* h, int dev, int nt, int nx, int ny, int bx, int by, double dx, double dy,
                                  double* u, double* v, double* out, double* in) {
    return create_weno_plan(h, dev, nt, nx, ny, bx, by, dx, dy, u, v, out, in);
}

int custen_device_error(unsigned int* flags, int clear) {
    if (flags == nullptr) return fail_arg("flags pointer is NULL");
    CU_TRY(cudaMemcpyFromSymbol(flags, g_custen_device_error, sizeof(unsigned int)), "Reading device error flags");
    if (clear) {
        unsigned int z = 0;
        CU_TRY(cudaMemcpyToSymbol(g_custen_device_error, &z, sizeof(z)), "Clearing device error flags");
    }
    return ST_OK;
}

int custen_malloc_managed(void** ptr, size_t bytes) {
    CU_TRY(cudaMallocManaged(ptr, bytes), "Allocating managed memory");
    return ST_OK;
}
int custen_malloc_device(void** ptr, size_t bytes) {
    CU_TRY(cudaMalloc(ptr, bytes), "Allocating device memory");
    return ST_OK;
}
int custen_malloc_host(void** ptr, size_t bytes) {
    CU_TRY(cudaMallocHost(ptr, bytes), "Allocating pinned host memory");
    return ST_OK;
}
int custen_free(void* ptr) {
    CU_TRY(cudaFree(ptr), "Freeing memory");
    return ST_OK;
}
int custen_free_host(void* ptr) {
    CU_TRY(cudaFreeHost(ptr), "Freeing pinned host memory");
    return ST_OK;
}
int custen_memcpy(void* dst, const void* src, size_t bytes) {
    CU_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault), "Copying memory");
    return ST_OK;
}
int custen_memset(void* ptr, int value, size_t bytes) {
    CU_TRY(cudaMemset(ptr, value, bytes), "Setting memory");
    return ST_OK;
}
int custen_device_synchronize(void) {
    CU_TRY(cudaDeviceSynchronize(), "Synchronising device");
    return ST_OK;
}
int custen_set_device(int device) {
    CU_TRY(cudaSetDevice(device), "Setting current device");
    return ST_OK;
}

}  // extern "C"
