/*
 * custen_gb300.h -- C-ABI (extern "C") entry points of the GB300 cuSten rebuild.
 *
 * Every function returns 0 on success and a non-zero status otherwise (1: CUDA error, 2: invalid
 * argument, 3: unsupported); custen_last_error() returns the message of the last failure on the
 * calling thread. No function exits the process. Plain pointers and sizes only.
 *
 * The handle is the reference's own 200-byte cuSten_t (include/cuSten.h), allocated by the caller.
 * Each create entry point takes the argument list of the reference function it mirrors (cited
 * below, paths inside the cuSten project) and fills the handle exactly as the C++ drop-in API does;
 * custen_create with dtype CUSTEN_F32 takes float data and runs the FP32 kernels (the precision
 * variant; the reference is FP64 only). Compute / swap / destroy dispatch on the
 * variant recorded in the handle, so one entry point each replaces the reference's per-variant
 * cuStenCompute2D* / cuStenSwap2D* / cuStenDestroy2D* functions.
 */
#ifndef CUSTEN_GB300_H
#define CUSTEN_GB300_H

#include <stddef.h>
#include "cuSten.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Variant codes (the twelve operators of cuSten/src/kernels/stencil_kernels.h:52-183). */
enum {
    CUSTEN_XP = 0, CUSTEN_XNP = 1, CUSTEN_XPFUN = 2, CUSTEN_XNPFUN = 3,
    CUSTEN_YP = 4, CUSTEN_YNP = 5, CUSTEN_YPFUN = 6, CUSTEN_YNPFUN = 7,
    CUSTEN_XYP = 8, CUSTEN_XYNP = 9, CUSTEN_XYPFUN = 10, CUSTEN_XYNPFUN = 11,
    CUSTEN_XYWENOADVP = 12   /* created by custen_create_2d_xyweno_adv_p only */
};
enum { CUSTEN_F64 = 0, CUSTEN_F32 = 1 };

/* ---- library information ---- */
int custen_abi_version(void);                 /* increments when an entry point changes */
int custen_sizeof_handle(void);               /* sizeof(cuSten_t): 200 on LP64 */
const char* custen_last_error(void);
unsigned long long custen_kernel_launches(void);   /* kernels launched by this library so far */
unsigned long long custen_kernel_launches_tma(void);   /* of which used the TMA-staged stencil kernel */
/* Bytes Compute has moved host -> device and device -> host since the library was loaded (managed
 * prefetches and the staged copies of pinned / system-memory fields). No reference counterpart. */
void custen_transfer_bytes(unsigned long long* h2d, unsigned long long* d2h);
/* Fields in pinned or system memory are streamed through device staging slots in chunks of about
 * `bytes` (0: the default, 32 MiB); applies to handles whose first such Compute comes later. */
void custen_set_stage_chunk_bytes(size_t bytes);
/* Fun variants whose device function is one of the library's c^3 - c functions (custen_builtin_function
 * ids 1, 3, 5, with the window that function reads) run as c^3 - c once per input value followed by the
 * coefficients as plain weights: bit-identical results, fewer FP64 operations. enable = 0 sends them
 * through the indirect call like any user function. Default 1. No reference counterpart. */
void custen_set_fun_fusion(int enable);
/* At most `max_ctas` CTAs per persistent (TMA-staged) stencil launch; 0 (the default) lifts the cap.
 * Results do not depend on it: a lower cap makes each CTA walk more tiles through its shared-memory
 * ring, which lets small fields exercise stage reuse. No reference counterpart. */
void custen_set_max_ctas(int max_ctas);
/* ---- autotuner (no reference counterpart) ----
 * The stencil kernels come in several tile configurations (tile width / height, rows per thread, vector
 * width: the role of BLOCK_X / BLOCK_Y); all compute identical values. A handle's first Compute on
 * device-resident fields picks one: mode 0 looks the launch geometry up in the JSON cache and uses the
 * default when absent (default mode); mode 1 also tunes absent geometries (times every configuration on
 * that launch) and stores the result; mode 2 always tunes. The environment variable CUSTEN_AUTOTUNE sets
 * the initial mode; the cache file is custen_set_tune_cache's path, else CUSTEN_TUNE_CACHE, else
 * $HOME/.cache/custen_gb300/tune.json. custen_autotune tunes one handle now. */
void custen_set_autotune(int mode);
void custen_set_tune_cache(const char* path);
int custen_tune_cache_path(char* buf, size_t len);
int custen_autotune(cuSten_t* h, int reps);
int custen_handle_config(const cuSten_t* h, char* name, size_t len);
/* Pin a handle to configuration `index` (0 .. 4; -1: choose again at the next Compute). */
int custen_set_config(cuSten_t* h, int index);

/* Which shipped function (0..5) `f` is on the current device, or -1. */
int custen_builtin_fun_id(const void* f, int dtype);

/* ---- handle life cycle: generic form ----
 * H/L/R: window width and extents in x; V/T/B in y. X variants: V=1, T=B=0; Y variants: H=1, L=R=0.
 * ncoef: number of weights/coefficients read per Compute. func: device function pointer (Fun). */
int custen_create(cuSten_t* h, int variant, int dtype, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X,
                  int BLOCK_Y, void* dataOutput, void* dataInput, void* coef, int H, int L, int R, int V, int T,
                  int B, int ncoef, void* func);
/* A handle over one y-slab of a field split across several owners (processes, GPUs): the slab is tile
 * `slab` of `num_slabs` tiles of ny_slab rows each, the numTiles layout of the reference
 * (custenCreateDestroy2DYp.cu:182-216) with each tile in its own allocation. halo_top holds the T rows above
 * the slab and halo_bottom the B rows below it (periodic variants wrap around the field); the caller fills
 * them before each Compute, e.g. from the neighbouring slabs' edge rows (custen_gb300.slabs). Either may be
 * NULL where the variant never reads it (non-periodic variants: above slab 0, below the last slab). The
 * non-periodic write rules are those of tile `slab` of the whole field, so the slabs together give exactly
 * the single-handle result with numTiles = num_slabs. Swap exchanges in and out and keeps the halo buffers.
 * Device or managed memory. */
int custen_create_slab(cuSten_t* h, int variant, int dtype, int deviceNum, int slab, int num_slabs, int nx,
                       int ny_slab, int BLOCK_X, int BLOCK_Y, void* dataOutput, void* dataInput, void* halo_top,
                       void* halo_bottom, void* coef, int H, int L, int R, int V, int T, int B, int ncoef,
                       void* func);
int custen_compute(cuSten_t* h, int offload);                       /* cuStenCompute2D*(h, offload) */
int custen_compute_on_stream(cuSten_t* h, int offload, void* stream); /* same, all work on `stream` */
/* One Compute of each of `count` distinct handles, free to run at the same time: each handle's work runs
 * on its own first stream, after the work already queued on `stream` and before any work queued on
 * `stream` later. Use it for independent operators (e.g. several derivatives of one field into separate
 * outputs): on small fields one launch's tail then overlaps the next launch. All handles and `stream`
 * belong to one device. Handles that write a buffer another member reads must not be grouped. The reference computes one handle per call
 * (stencil_kernels.h:52-183); this has no counterpart there. */
int custen_compute_group(cuSten_t* const* handles, int count, int offload, void* stream);
int custen_swap(cuSten_t* h, void* dataInput);                      /* cuStenSwap2D*(h, dataInput) */
int custen_destroy(cuSten_t* h);                                    /* cuStenDestroy2D*(h) */
int custen_set_stream(cuSten_t* h, void* stream);   /* later Computes run on `stream` (NULL: own streams) */
int custen_handle_variant(const cuSten_t* h, int* variant, int* dtype);

/* ---- per-variant create, FP64, reference argument lists ---- */
/* cuSten_struct_functions.h:184-198 */
int custen_create_2d_xp(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                        double* dataOutput, double* dataInput, double* weights, int numSten, int numStenLeft,
                        int numStenRight);
/* :67-81 */
int custen_create_2d_xnp(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                         double* dataOutput, double* dataInput, double* weights, int numSten, int numStenLeft,
                         int numStenRight);
/* :242-266 */
int custen_create_2d_xp_fun(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                            double* dataOutput, double* dataInput, double* coe, int numSten, int numStenLeft,
                            int numStenRight, int numCoe, double* func);
/* :125-141 */
int custen_create_2d_xnp_fun(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                             double* dataOutput, double* dataInput, double* coe, int numSten, int numStenLeft,
                             int numStenRight, int numCoe, double* func);
/* :742-756 */
int custen_create_2d_yp(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                        double* dataOutput, double* dataInput, double* weights, int numSten, int numStenTop,
                        int numStenBottom);
/* :626-640 */
int custen_create_2d_ynp(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                         double* dataOutput, double* dataInput, double* weights, int numSten, int numStenTop,
                         int numStenBottom);
/* :801-817 */
int custen_create_2d_yp_fun(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                            double* dataOutput, double* dataInput, double* coe, int numSten, int numStenTop,
                            int numStenBottom, int numCoe, double* func);
/* :684-699 (no numCoe; numSten coefficients are read) */
int custen_create_2d_ynp_fun(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                             double* dataOutput, double* dataInput, double* coe, int numSten, int numStenTop,
                             int numStenBottom, double* func);
/* :500-517 */
int custen_create_2d_xyp(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                         double* dataOutput, double* dataInput, double* weights, int numStenHoriz, int numStenLeft,
                         int numStenRight, int numStenVert, int numStenTop, int numStenBottom);
/* :371-388 */
int custen_create_2d_xynp(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                          double* dataOutput, double* dataInput, double* weights, int numStenHoriz, int numStenLeft,
                          int numStenRight, int numStenVert, int numStenTop, int numStenBottom);
/* :564-582 */
int custen_create_2d_xyp_fun(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                             double* dataOutput, double* dataInput, double* coe, int numStenHoriz, int numStenLeft,
                             int numStenRight, int numStenVert, int numStenTop, int numStenBottom, double* func);
/* :435-453 */
int custen_create_2d_xynp_fun(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                              double* dataOutput, double* dataInput, double* coe, int numStenHoriz, int numStenLeft,
                              int numStenRight, int numStenVert, int numStenTop, int numStenBottom, double* func);

/* WENO5 advection, periodic: cuStenCreate2DXYWENOADVp (cuSten_struct_functions.h:290-324); computed by
 * custen_compute like every other handle (cuStenCompute2DXYWENOADVp, stencil_kernels.h:181-189), swapped
 * with custen_swap, destroyed with custen_destroy. */
int custen_create_2d_xyweno_adv_p(cuSten_t* h, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X,
                                  int BLOCK_Y, double dx, double dy, double* u, double* v, double* dataOutput,
                                  double* dataInput);

/* ---- device functions shipped with the library for the Fun variants ----
 * id 0: X  (d[l-1] - 2 d[l] + d[l+1]) * coe[0]
 *         (the user function of the reference example examples/src/2d_x_np_fun.cu:49-51)
 * id 1: X  sum_k coe[k] * (d^3 - d) over the window l-L..l+R, L = R = 2 (5 coefficients)
 * id 2: Y  sum_k coe[k] * d[l + (k-4)*jump], 9 coefficients (examples/src/2d_y_p_fun.cu:49-60)
 * id 3: Y  sum_k coe[k] * (d^3 - d) over rows l-2..l+2 (5 coefficients)
 * id 4: XY sum_{j,i} coe[j*H+i] * d[tl + j*jump + i] (examples/src/2d_xy_p_fun.cu:58-80)
 * id 5: XY sum_{j,i} coe[j*H+i] * (d^3 - d) (the Cahn-Hilliard nonLinRHS,
 *         cuPentCahnADI/src/cuPentCahnADI.cu:164-190)
 * All use explicit fused multiply-adds in a fixed order, so their results are reproducible on the
 * host. `dtype` selects the double or float version. */
int custen_builtin_function(int id, int dtype, void** func);

/* ---- measurement ----
 * Sustained FMA rate of this GPU (FMA per second, 8 independent chains per thread, all SMs), the
 * compute-roofline denominator of the FP64 stencils. No counterpart in the reference. */
int custen_probe_fma_rate(int dtype, double* fma_per_s);

/* Device-side error flags raised by kernels instead of trapping (bit 0: a bounded mbarrier wait of a
 * TMA-staged kernel expired; the kernel then returned early. bit 1, in the checked build of the library
 * only: a kernel index outside the extent it must stay in; that access was skipped). Synchronous;
 * clear != 0 resets them. No counterpart in the reference (its kernels have no waits or checks). */
int custen_device_error(unsigned int* flags, int clear);
/* Self-test of that failure path: one CTA waits, with the stencil kernels' bounded wait limited to
 * `rounds` try_wait rounds (1 .. 2^22), on an mbarrier nothing arrives on; the wait gives up, bit 0 is
 * raised and the kernel returns. *flags receives the flags afterwards (left set). No copy fails and
 * nothing traps; the context stays usable. */
int custen_selftest_wait_expiry(long long rounds, unsigned int* flags);

/* ---- batched pentadiagonal systems (cuPentBatch, cuPentCahnADI/src/cuPentBatch.cu) ----
 * Interleaved layout: element (row i, system s) of each diagonal and of b at [i * batch + s]; ds, dl
 * two / one below the main diagonal d, du, dw one / two above (ds[0..1], dl[0], du[m-1], dw[m-2..m-1]
 * zero). Device pointers; asynchronous on `stream` (NULL: the default stream). m >= 4.
 * custen_pent_factor_batch   -- pentFactorBatch (:35-113), in place, bit-identical to the reference kernel
 * custen_pent_solve_batch    -- pentSolveBatch (:119-198) with those factors, b overwritten by x,
 *                               bit-identical to the reference kernel
 * custen_pent_invert_pivots  -- d <- 1 / d after the factorisation (no reference counterpart)
 * custen_pent_solve_batch_rcp -- the solve with inverted pivots: multiplications instead of divisions,
 *                               rounding within about one unit in the last place per row of the reference */
int custen_pent_factor_batch(double* ds, double* dl, double* d, double* du, double* dw, int m, int batch,
                             void* stream);
int custen_pent_solve_batch(const double* ds, const double* dl, const double* d, const double* du, const double* dw,
                            double* b, int m, int batch, void* stream);
int custen_pent_invert_pivots(double* d, int m, int batch, void* stream);
int custen_pent_solve_batch_rcp(const double* ds, const double* dl, const double* rd, const double* du,
                                const double* dw, double* b, int m, int batch, void* stream);
const char* custen_pent_last_error(void);
/* Rows of loads issued ahead of the recurrence (2, 4 or 8) in the factorisation (which = 0), the exact
 * solve (1) and the inverted-pivot solve (2); results do not depend on it. */
int custen_pent_set_depth(int which, int rows);

/* ---- Cahn-Hilliard ADI solver: batches of periodic grids of different sizes ----
 * The method of cuPentCahnADI (cuPentCahnADI/src/cuPentCahnADI.cu:197-627 with BatchHyper.cu and
 * cuPentBatch.cu): D = 1, gamma, dt = dt_factor * dx, domain [0, lx)^2, BDF2 / ADI with cyclic
 * pentadiagonal sweeps. Grid sizes n: multiples of 32, at least 64. lx may be NULL (2 pi each).
 * rhs_dtype CUSTEN_F32 computes the explicit stencil terms in FP32 (precision variant); the solves,
 * updates and mass sums stay FP64. State arrays are n*n doubles, host or device pointers. */
const char* custen_ch_last_error(void);
int custen_ch_batch_create(void** batch, int nsims, const int* n, const double* lx, double gamma, double dt_factor,
                           int rhs_dtype, void* stream);
int custen_ch_batch_set_state(void* batch, int sim, const double* c_cur, const double* c_old);
int custen_ch_batch_get_state(void* batch, int sim, double* c_cur, double* c_old);
int custen_ch_batch_step(void* batch, int steps, int use_graph);   /* asynchronous */
int custen_ch_batch_synchronize(void* batch);
int custen_ch_batch_mean(void* batch, int sim, double* mean);     /* compensated FP64 sum */
unsigned long long custen_ch_batch_launches(void* batch);
/* Kernel configuration of the batch's steps (warps per right-hand-side CTA, rows per y-sweep batch):
 * custen_ch_batch_autotune times every configuration over `steps` steps of the batch itself, restores
 * the fields, and keeps the fastest; results do not depend on it. No reference counterpart. */
int custen_ch_batch_autotune(void* batch, int steps, char* name, size_t len);
int custen_ch_batch_config(void* batch, char* name, size_t len);
int custen_ch_batch_set_config(void* batch, int index);   /* 0 .. 21; -1: the default */
/* Checkpoint / resume of one grid through an HDF5 snapshot (the format below): save writes "c" = cCurr,
 * "c_old" = cOld and "t" = time; load takes "c" (must be n x n), "c_old" if present (else cCurr, as the
 * reference starts) and returns "t" in *time (NaN when absent, as in the reference's own snapshots).
 * A resumed grid continues bit for bit as if never stopped. */
int custen_ch_batch_save(void* batch, int sim, const char* path, double time);
int custen_ch_batch_load(void* batch, int sim, const char* path, double* time);
int custen_ch_batch_destroy(void* batch);

/* ---- HDF5 snapshot files (host only; no HDF5 library needed) ----
 * The file the reference solver writes (Print_Out, cuPentCahnADI/src/cuPentCahnADI.cu:103-140): an
 * HDF5 file (superblock version 0, as the HDF5 library writes with default properties) whose root group
 * holds two-dimensional datasets of IEEE little-endian doubles in contiguous storage; the reference's
 * file holds one, "c", with dims {nx, ny}. custen_h5_write writes 1 to 8 datasets (dims[2i], dims[2i+1]
 * of dataset i; names without '/'). custen_h5_read reads one dataset of such a file, or of any HDF5
 * file with version-0/1 superblock, old-style groups and contiguous float32/float64 data; it stores
 * the dims (rank 1 gives {d0, 1}) and, when out is not NULL, the values (capacity in doubles). */
int custen_h5_write(const char* path, int count, const char* const* names, const double* const* data,
                    const long long* dims);
int custen_h5_read(const char* path, const char* name, double* out, long long capacity, long long* dims);
const char* custen_h5_last_error(void);

/* ---- Cahn-Hilliard serving: request loop with continuous batching ----
 * Requests (n, steps, c0 or a seed for c0 ~ U(-0.1, 0.1), arrival time) are queued, then run()
 * admits arrived requests first-come first-served within the HBM budget, advances every resident
 * grid together a chunk of steps at a time (one launch per kernel for all grids), retires finished
 * grids and admits new arrivals between chunks. Times are seconds on the server clock of run().
 * No counterpart in the reference (its driver runs one simulation per process). */
const char* custen_ch_server_last_error(void);
int custen_ch_server_create(void** server, double hbm_budget_bytes, int rhs_dtype, double gamma, double dt_factor,
                            int chunk_steps, int keep_results);
int custen_ch_server_submit(void* server, int n, double lx, int steps, const double* c0, unsigned long long seed,
                            double arrival, int* request_id);
int custen_ch_server_run(void* server);
int custen_ch_server_result(void* server, int request_id, double* c_out, double* arrival, double* admit_t,
                            double* done_t, double* mean0, double* mean_end);
int custen_ch_server_stats(void* server, double* makespan, long long* total_steps, double* total_point_steps,
                           int* max_active, double* peak_bytes, unsigned long long* launches);
/* Failure isolation: a request whose admission fails (device allocation or upload) is marked failed
 * (state 3; custen_ch_server_result returns 3 and the reason) and the run continues with the others; a
 * request that can never fit the budget is rejected by submit. custen_ch_server_request_state: 0
 * pending, 1 resident, 2 done, 3 failed. custen_ch_server_inject_failure is a test hook: kind 1 makes
 * the request's admission allocation fail as cudaMallocAsync would on an exhausted device (a fake of
 * the failing call on the host; nothing reaches the GPU). */
int custen_ch_server_request_state(void* server, int request_id, int* state);
/* Checkpoint / resume in the server. custen_ch_server_set_snapshots (before run): every `every` steps
 * the request's state goes to dir/cahn_hilliard_<time %0.10f>.nc -- the reference's Print_Out file
 * (cuPentCahnADI.cu:103-140, 585-595: dataset "c", time accumulated by dt per step) plus "c_old" and
 * "t"; a failed write fails the request. custen_ch_server_submit_snapshot queues a request resumed
 * from such a file (n and cCurr from "c", cOld from "c_old" or cCurr, time from "t" or 0), which then
 * continues bit for bit; lx <= 0 means 2 pi. */
int custen_ch_server_set_snapshots(void* server, int request_id, int every, const char* dir);
int custen_ch_server_submit_snapshot(void* server, const char* path, double lx, int steps, double arrival,
                                     int* request_id);
int custen_ch_server_snapshots_written(void* server, int request_id, int* count);
int custen_ch_server_inject_failure(void* server, int request_id, int kind);
int custen_ch_server_destroy(void* server);

/* One Cahn-Hilliard step of one n x n grid that allocates nothing: for callers that cannot allocate
 * device memory (a plug-in inside an application that owns all device memory, or a loop that must
 * never enter cudaMalloc / cudaFree, which synchronise the device). Its work buffers live in a
 * library-owned static device array sized for n <= 256 (about 532 KiB, held by every GPU that loads
 * the library until exit); larger n is rejected with status 2. c_old and c_cur are the previous two
 * fields, c_new receives the next (it may be the c_old buffer, not the c_cur buffer); all three are
 * device-accessible n*n doubles. The first call on a device looks up the array's device address, so
 * make it before any stream capture. Calls share the array: calls that overlap on the GPU race.
 * No counterpart in the reference. */
int custen_ch_step_noalloc(const double* c_old, const double* c_cur, double* c_new, int n, double lx, double gamma,
                           double dt_factor, void* stream);

/* ---- memory helpers for hosts without a CUDA runtime binding ---- */
int custen_malloc_managed(void** ptr, size_t bytes);
int custen_malloc_device(void** ptr, size_t bytes);
int custen_malloc_host(void** ptr, size_t bytes);    /* pinned */
int custen_free(void* ptr);
int custen_free_host(void* ptr);
int custen_memcpy(void* dst, const void* src, size_t bytes);   /* cudaMemcpyDefault, synchronous */
int custen_memset(void* ptr, int value, size_t bytes);
int custen_device_synchronize(void);
int custen_set_device(int device);

#ifdef __cplusplus
}
#endif

#endif /* CUSTEN_GB300_H */
