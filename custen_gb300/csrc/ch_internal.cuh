// Shared declarations of the Cahn-Hilliard ADI kernels (ch_solver.cu) for the batch and server hosts.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace custen {
namespace ch {

constexpr int BLK = 32;   // rows / columns per work item; n must be a multiple of 32

// Per-grid descriptor (device).
struct GridDev {
    double* buf[2];       // the two field buffers: cCurr = buf[parity], cOld = buf[parity ^ 1]
    double* tmp;          // n x n work field (rhs, then the x-sweep solution)
    double* ends;         // 2 n values: the x sweep's last two unknowns of every row
    double* hbuf;         // n x n h of the two-pass right-hand side (batch only; null elsewhere)
    const double* tab;    // solver table for n (layout below)
    int n;
    int pad;
};

// Table layout for one n (m = n - 2), all double:
//   [0, m) ds  [m, 2m) dl  [2m, 3m) rd = 1/diag  [3m, 4m) du  [4m, 5m) dw   (factored, zero-padded:
//   ds[0] = ds[1] = dl[0] = 0, du[m-1] = 0, dw[m-2] = dw[m-1] = 0)
//   [5m, 6m) inv1  [6m, 7m) inv2   border columns of the cyclic correction
//   [7m, 7m+4) omega  [7m+4, 7m+8) a, b, d, e  [7m+8, 7m+33) linear 5x5 weights  [7m+33, 7m+42) the
//   non-linear 3x3 weights
__host__ __device__ inline int tab_size(int n) { return 7 * (n - 2) + 42; }

struct Item {
    int grid;
    int block;   // K1: 32 x 32 block index (row-major over the grid); K2: row block; K3: column block
};

__global__ void ch_xsolve_kernel(const GridDev* __restrict__ grids, const Item* __restrict__ items, int n_items,
                                 unsigned int* counter);
__global__ void ch_mass_kernel(const double* __restrict__ f, long long count, double* out);

// Kernel configuration of a step: warps per right-hand-side CTA (1, 2, 4), rows per batch of the y
// sweep (16, 32; with pipelined sweeps also the x sweep's columns per chunk), and whether the sweeps
// copy the next chunk into shared memory while the current one runs (pipe 1; pipe 2: the x sweep takes
// x_chunk-column chunks with its table entries in registers; pipe 3: both sweeps hold their table
// entries in registers, the y sweep in y_chunk-row batches). Every configuration computes the same values; the
// batch tuner times them.
struct ChConfig {
    int rhs_warps;
    int y_chunk;
    int pipe;
    int x_chunk;     // columns per chunk of the register-table x sweep (pipe 2, 3): 8 or 16
    int rhs_split;   // 1: the right-hand side in two passes through GridDev::hbuf (batches only); 2: the same
                     // with pass 2 pipelined (cp.async double buffer)
    int ysplit;      // 1: the y sweep's correction and update as element-wise kernels around the recurrences
                     // (pipe 3 only; for batches with few lines per SM)
};
constexpr ChConfig kChDefault{4, 8, 3, 16, 0};   // configuration 12; needs no h buffer (server, one-grid step)
constexpr int kChBatchDefault = 20;             // batches (they allocate the h buffer): two-pass right-hand side,
                                                // pass 2 pipelined, 8 warps per CTA
constexpr int kChConfigs = 22;
constexpr int kChSplitConfig = 21;             // configuration 20 with the split y sweep
constexpr int kChCounters = 4;   // work counters per step (zeroed before it)
ChConfig ch_config(int index);   // 0 .. kChConfigs-1
int ch_launches_per_step(const ChConfig& c);
void config_name(const ChConfig& c, char* name, size_t len);

// One step of every grid of a work list: right-hand side (one or two passes), x sweep, y sweep (3 or 4
// launches on s). counters: kChCounters zeroed work counters.
cudaError_t launch_ch_step(const ChConfig& c, bool rhs_fp32, const GridDev* grids, const Item* items_rhs, int n_rhs,
                           const Item* items_rows, int n_rows, int parity, unsigned int* counters, int sms,
                           cudaStream_t s);

// Solver table of an n x n grid (tab_size(n) doubles) built on the host.
std::vector<double> build_table(int n, double lx, double gamma, double dt_factor);

}  // namespace ch
}  // namespace custen
