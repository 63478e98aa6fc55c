// Cahn-Hilliard ADI solver on sm_103a: one time step of many periodic grids of different sizes.
//
// Scheme of the reference solver (cuPentCahnADI/src/cuPentCahnADI.cu:528-596, and its CPU twin
// cuPentSpeedUp/serialCahnADITiming/serialCahnADI.c:1010-1047), per grid of n x n points:
//   cBar = 2 cCurr - cOld
//   rhs  = Lin5x5(cBar) + Nl3x3(cCurr^3 - cCurr) - (2/3)(cCurr - cOld)
//   (1 + s Dx4)(1 + s Dy4) delta = rhs   -- two cyclic pentadiagonal sweeps, x then y, each solved as
//       the (n-2) x (n-2) banded block (pre-factored, cuPentBatch.cu:35-198) plus the 2 x 2 Schur
//       complement on the last two unknowns (BatchHyper.cu:195-259, 421-514)
//   cNew = cBar + delta;  cOld <- cCurr;  cCurr <- cNew
//
// GB300 shape: FP64 FMAs (about 2 per clock per SM) bound this solver, not HBM, so the kernels
// minimise FP64 operations (about 32 per point and step, against about 100 in the reference: the two
// explicit stencils as two 5-point Laplacians, cBar and c^3 - c computed once per point, divisions
// replaced by reciprocals) and keep every SM sub-partition busy:
//   K1 ch_rhs_kernel     -- right-hand side, 32 x 32 blocks, lane = column, all points in parallel.
//   K2 ch_xsolve_kernel  -- x sweep, one warp per 32 rows (lane = row) walking 32-column chunks
//                           transposed through shared memory; leaves the banded solution y and the
//                           two corner values of every row.
//   K3 ch_ysolve_kernel  -- y sweep, one warp per 32 columns (lane = column, coalesced), applying the
//                           x sweep's rank-2 correction as it reads, then cNew = cBar + delta written
//                           over cOld (the two field buffers swap roles every step).
// Each kernel is persistent over a work list that covers all grids (largest first, claimed through
// an atomic counter), so grids of different sizes share one launch. A step is three launches (four with
// the two-pass right-hand side, six with the split y sweep as well); pairs of steps are captured in a CUDA
// graph.
//
// The sweeps come in three forms, all computing the same values (ChConfig, tuned per batch):
// staged through registers (the kernels K2/K3 below), pipelined (the next chunk copied into shared
// memory with cp.async while the current one runs), and pipelined with the chunk's table entries held
// in registers by every lane (no per-element shuffles; the default, configuration 12).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/custen_gb300.h"
#include "ch_internal.cuh"
#include "checked.cuh"

namespace custen {
namespace ch {

// ------------------------------------------------------------------------------------------------
// K1: right-hand side
// ------------------------------------------------------------------------------------------------
// T = double: FP64 arithmetic; T = float: the FP32 precision variant (cBar, c^3 - c, the inner Laplacian
// and h in FP32 from inputs and coefficients rounded to float; the outer Laplacian of the FP32 h values
// and the time-derivative term summed in FP64, which keeps the mass conserved to FP64 rounding).
//
// The reference's two explicit stencils are the 13-point biharmonic sigma_lin * [-1; -2 8 -2; -1 8 -20
// 8 -1; ...] on cBar and the 5-point Laplacian sigma_nl * [1; 1 -4 1; 1] on c^3 - c
// (cuPentCahnADI.cu:463-467, 509-513). The biharmonic is the 5-point Laplacian applied twice, so
//   Lin(cBar) + Nl(g) = Lap(h),   h = sigma_nl * g - sigma_lin * Lap(cBar),
// with Lap the unit-weight 5-point Laplacian (N + S + W + E - 4 C). The kernel evaluates that form:
// about 16 FP64 operations per point instead of 24 for the two stencils taken separately. The sums are
// the same mathematically; their rounding differs from the reference's weight-by-weight chain at the
// level of one rounding per term, far inside the solver's 1e-10 parity bar.
// NW warps per CTA share one 32 x 32 work item: shared memory limits residency to a few CTAs per SM, so
// more warps per CTA give the FP64 pipe more warps to issue from (the tuned choice, ChConfig).
//
// The constant factors 2, -4 and -2/3 are read from device memory into registers once per thread: an
// FP64 FMA that takes a literal or a kernel parameter as an operand issues about 19% slower on GB300
// (507 against 602-628 G FMA/s measured) than one whose operands are all registers. The values, and
// so the results, are the same as with literals.
__device__ double g_rhs_factors[3] = {2.0, -4.0, -2.0 / 3.0};

template <typename T, int NW>
__global__ void __launch_bounds__(NW * BLK) ch_rhs_kernel(const GridDev* __restrict__ grids,
                                                          const Item* __restrict__ items, int n_items, int parity,
                                                          unsigned int* counter) {
    __shared__ T cb[36][37];        // cBar over the block and a 2-point halo
    __shared__ T hh[34][35];        // sigma_nl * (c^3 - c), then h, over the block and a 1-point halo
    __shared__ double dco[32][33];  // cCurr - cOld at the block's points (FP64 in both variants)
    __shared__ int s_item;
    constexpr int NT = NW * BLK;
    const int tid = threadIdx.x;
    const int lane = tid & (BLK - 1), warp = tid / BLK;
    const volatile double* factors = g_rhs_factors;
    const T two = (T)factors[0], m_four = (T)factors[1];
    const double m_four_d = factors[1], m_two_thirds_d = factors[2];
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        // selects rather than gd.buf[parity]: a run-time index would put the descriptor in local memory
        const double* cur = parity ? gd.buf[1] : gd.buf[0];
        const double* old = parity ? gd.buf[0] : gd.buf[1];
        const double* tab = gd.tab;
        const int bpr = n / BLK;
        const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
        // sigma_lin and sigma_nl, exactly: the far weight of the biharmonic is -sigma_lin, the north weight
        // of the Laplacian sigma_nl (the table stores the weights as pattern * sigma)
        const T s_lin = (T)(-tab[7 * m + 8 + 2]);
        const T s_nl = (T)tab[7 * m + 33 + 1];
        // stage the 36 x 36 window (periodic wrap)
#pragma unroll 4
        for (int e = tid; e < 36 * 36; e += NT) {
            const int r = e / 36, c = e - r * 36;
            int gy = y0 - 2 + r, gx = x0 - 2 + c;
            gy = gy < 0 ? gy + n : (gy >= n ? gy - n : gy);
            gx = gx < 0 ? gx + n : (gx >= n ? gx - n : gx);
            const double cv = cur[(size_t)gy * n + gx];
            const double ov = old[(size_t)gy * n + gx];
            const T c32 = (T)cv, o32 = (T)ov;
            cb[r][c] = fma(two, c32, -o32);
            if (r >= 1 && r < 35 && c >= 1 && c < 35) hh[r - 1][c - 1] = s_nl * fma(c32 * c32, c32, -c32);
            if (r >= 2 && r < 34 && c >= 2 && c < 34) dco[r - 2][c - 2] = cv - ov;
        }
        __syncthreads();
        // h = sigma_nl * g - sigma_lin * Lap(cBar) over the 34 x 34 block + halo
#pragma unroll 4
        for (int e = tid; e < 34 * 34; e += NT) {
            const int r = e / 34, c = e - r * 34;
            const T lap = fma(m_four, cb[r + 1][c + 1], (cb[r][c + 1] + cb[r + 2][c + 1]) + (cb[r + 1][c] + cb[r + 1][c + 2]));
            hh[r][c] = fma(-s_lin, lap, hh[r][c]);
        }
        __syncthreads();
        // rhs = Lap(h) - (2/3)(cCurr - cOld)  (findRHS, cuPentCahnADI.cu:72-86); lane = column. Summed in
        // FP64 in both variants: over FP32 values of h (the precision variant) the FP64 sums are exact, so
        // the discrete Laplacian sums to zero over the periodic grid and the mass is conserved to FP64
        // rounding, as in the FP64 variant.
        const int j = lane;
        double* out = gd.tmp + (size_t)y0 * n + x0 + j;
#pragma unroll 4
        for (int rr = warp; rr < BLK; rr += NW) {
            const double lap = fma(m_four_d, (double)hh[rr + 1][j + 1],
                                   ((double)hh[rr][j + 1] + (double)hh[rr + 2][j + 1]) +
                                       ((double)hh[rr + 1][j] + (double)hh[rr + 1][j + 2]));
            if (!in_bounds((long long)(y0 + rr) * n + x0 + j, 0, (long long)n * n)) continue;
            out[(size_t)rr * n] = fma(m_two_thirds_d, dco[rr][j], lap);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------
// K1 in two passes (batch configurations with rhs_split): h is formed once per point and kept in the
// grid's h buffer, so that no block recomputes its neighbours' halo values of h (K1 above forms cBar
// on a 2-point halo and h on a 1-point halo of every block: about 16.3 FP64 operations per point;
// the two passes take about 15.1). The expressions and their order are those of K1, so the results
// are the same bit for bit.
// ------------------------------------------------------------------------------------------------
// Pass 1: h = sigma_nl * (c^3 - c) - sigma_lin * Lap(cBar), cBar over the block and a 1-point halo.
template <typename T, int NW>
__global__ void __launch_bounds__(NW * BLK) ch_h_kernel(const GridDev* __restrict__ grids,
                                                        const Item* __restrict__ items, int n_items, int parity,
                                                        unsigned int* counter) {
    __shared__ T cb[34][35];
    __shared__ T gg[32][33];   // sigma_nl * (c^3 - c)
    __shared__ int s_item;
    constexpr int NT = NW * BLK;
    const int tid = threadIdx.x;
    const volatile double* factors = g_rhs_factors;
    const T two = (T)factors[0], m_four = (T)factors[1];
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* cur = parity ? gd.buf[1] : gd.buf[0];
        const double* old = parity ? gd.buf[0] : gd.buf[1];
        const double* tab = gd.tab;
        const int bpr = n / BLK;
        const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
        const T s_lin = (T)(-tab[7 * m + 8 + 2]);
        const T s_nl = (T)tab[7 * m + 33 + 1];
#pragma unroll 4
        for (int e = tid; e < 34 * 34; e += NT) {
            const int r = e / 34, c = e - r * 34;
            int gy = y0 - 1 + r, gx = x0 - 1 + c;
            gy = gy < 0 ? gy + n : (gy >= n ? gy - n : gy);
            gx = gx < 0 ? gx + n : (gx >= n ? gx - n : gx);
            const double cv = cur[(size_t)gy * n + gx];
            const double ov = old[(size_t)gy * n + gx];
            const T c32 = (T)cv, o32 = (T)ov;
            cb[r][c] = fma(two, c32, -o32);
            if (r >= 1 && r < 33 && c >= 1 && c < 33) gg[r - 1][c - 1] = s_nl * fma(c32 * c32, c32, -c32);
        }
        __syncthreads();
#pragma unroll 4
        for (int e = tid; e < 32 * 32; e += NT) {
            const int r = e / 32, c = e - r * 32;
            const T lap = fma(m_four, cb[r + 1][c + 1], (cb[r][c + 1] + cb[r + 2][c + 1]) + (cb[r + 1][c] + cb[r + 1][c + 2]));
            const long long q = (long long)(y0 + r) * n + x0 + c;
            if (in_bounds(q, 0, (long long)n * n)) gd.hbuf[q] = (double)fma(-s_lin, lap, gg[r][c]);
        }
        __syncthreads();
    }
}

// Pass 2: rhs = Lap(h) - (2/3)(cCurr - cOld) (findRHS, cuPentCahnADI.cu:72-86), h over the block and a
// 1-point halo from the h buffer.
template <typename T, int NW>
__global__ void __launch_bounds__(NW * BLK) ch_rhs2_kernel(const GridDev* __restrict__ grids,
                                                           const Item* __restrict__ items, int n_items, int parity,
                                                           unsigned int* counter) {
    __shared__ T hh[34][35];
    __shared__ T dco[32][33];
    __shared__ int s_item;
    constexpr int NT = NW * BLK;
    const int tid = threadIdx.x;
    const int lane = tid & (BLK - 1), warp = tid / BLK;
    const volatile double* factors = g_rhs_factors;
    const T m_four = (T)factors[1], m_two_thirds = (T)factors[2];
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n;
        const double* cur = parity ? gd.buf[1] : gd.buf[0];
        const double* old = parity ? gd.buf[0] : gd.buf[1];
        const int bpr = n / BLK;
        const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
#pragma unroll 4
        for (int e = tid; e < 34 * 34; e += NT) {
            const int r = e / 34, c = e - r * 34;
            int gy = y0 - 1 + r, gx = x0 - 1 + c;
            gy = gy < 0 ? gy + n : (gy >= n ? gy - n : gy);
            gx = gx < 0 ? gx + n : (gx >= n ? gx - n : gx);
            hh[r][c] = (T)gd.hbuf[(size_t)gy * n + gx];
            if (r >= 1 && r < 33 && c >= 1 && c < 33) {
                const T c32 = (T)cur[(size_t)gy * n + gx], o32 = (T)old[(size_t)gy * n + gx];
                dco[r - 1][c - 1] = c32 - o32;
            }
        }
        __syncthreads();
        const int j = lane;
        double* out = gd.tmp + (size_t)y0 * n + x0 + j;
#pragma unroll 4
        for (int rr = warp; rr < BLK; rr += NW) {
            const T lap = fma(m_four, hh[rr + 1][j + 1], (hh[rr][j + 1] + hh[rr + 2][j + 1]) + (hh[rr + 1][j] + hh[rr + 1][j + 2]));
            if (!in_bounds((long long)(y0 + rr) * n + x0 + j, 0, (long long)n * n)) continue;
            out[(size_t)rr * n] = (double)fma(m_two_thirds, dco[rr][j], lap);
        }
        __syncthreads();
    }
}

// cp.async helpers (8-byte copies into shared memory, grouped, waited on by group count)
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Pass 2, pipelined (configurations with rhs_split = 2): the same expressions as ch_rhs2_kernel<double>,
// so the same results, with the next work item's h window and cCurr / cOld blocks copied into the other
// half of a shared-memory double buffer (cp.async) while the current item computes. ch_rhs2_kernel waits
// on its loads (long-scoreboard stalls about 22 warps per issue at 32 grids of 512^2, FP64 pipe 68% busy);
// here they are in flight during the previous item's arithmetic. The buffer is dynamic shared memory:
// kRhs2PipeWords doubles per half, so four CTAs fit an SM; with 8 warps per CTA (configuration 20, the
// batch default) a step of the 512-grid batch takes 8.54 ms against 8.72 with ch_rhs2_kernel
// (configuration 17); with 4 warps per CTA, 16 warps per SM hide too little and it takes 8.74.
constexpr int kRhs2H = 34 * 35, kRhs2C = 32 * 33;
constexpr int kRhs2PipeWords = kRhs2H + 2 * kRhs2C;
constexpr size_t kRhs2PipeBytes = 2 * kRhs2PipeWords * sizeof(double);

template <int NW>
__device__ __forceinline__ void rhs2_issue(double* buf, const GridDev& gd, const Item& item, int parity, int tid) {
    constexpr int NT = NW * BLK;
    const int n = gd.n;
    const double* cur = parity ? gd.buf[1] : gd.buf[0];
    const double* old = parity ? gd.buf[0] : gd.buf[1];
    const int bpr = n / BLK;
    const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
    double* hh = buf;
    double* cu = buf + kRhs2H;
    double* ol = cu + kRhs2C;
    for (int e = tid; e < 34 * 34; e += NT) {
        const int r = e / 34, c = e - r * 34;
        int gy = y0 - 1 + r, gx = x0 - 1 + c;
        gy = gy < 0 ? gy + n : (gy >= n ? gy - n : gy);
        gx = gx < 0 ? gx + n : (gx >= n ? gx - n : gx);
        cp_async8(hh + r * 35 + c, gd.hbuf + (size_t)gy * n + gx);
    }
    for (int e = tid; e < 32 * 32; e += NT) {
        const int r = e >> 5, c = e & 31;
        const size_t q = (size_t)(y0 + r) * n + x0 + c;
        cp_async8(cu + r * 33 + c, cur + q);
        cp_async8(ol + r * 33 + c, old + q);
    }
}

template <int NW>
__global__ void __launch_bounds__(NW * BLK) ch_rhs2_pipe_kernel(const GridDev* __restrict__ grids,
                                                                const Item* __restrict__ items, int n_items,
                                                                int parity, unsigned int* counter) {
    extern __shared__ __align__(16) double rhs2_smem[];
    __shared__ int s_next[2];
    const int tid = threadIdx.x;
    const int lane = tid & (BLK - 1), warp = tid / BLK;
    const volatile double* factors = g_rhs_factors;
    const double m_four = factors[1], m_two_thirds = factors[2];
    if (tid == 0) s_next[1] = (int)atomicAdd(counter, 1u);
    __syncthreads();
    int it_cur = s_next[1];
    if (it_cur < n_items) rhs2_issue<NW>(rhs2_smem, grids[items[it_cur].grid], items[it_cur], parity, tid);
    cp_async_commit();
    for (int k = 0;; ++k) {
        if (it_cur >= n_items) break;   // uniform: every thread read the same claim
        if (tid == 0) s_next[k & 1] = (int)atomicAdd(counter, 1u);
        __syncthreads();   // the claim is visible; every thread is done with the other half of the buffer
        const int it_next = s_next[k & 1];
        if (it_next < n_items)
            rhs2_issue<NW>(rhs2_smem + ((k + 1) & 1) * kRhs2PipeWords, grids[items[it_next].grid], items[it_next],
                           parity, tid);
        cp_async_commit();
        cp_async_wait<1>();   // this thread's copies of the current item have landed
        __syncthreads();      // and every other thread's
        const double* hh = rhs2_smem + (k & 1) * kRhs2PipeWords;
        const double* cu = hh + kRhs2H;
        const double* ol = cu + kRhs2C;
        const Item item = items[it_cur];
        const GridDev gd = grids[item.grid];
        const int n = gd.n;
        const int bpr = n / BLK;
        const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
        const int j = lane;
        double* out = gd.tmp + (size_t)y0 * n + x0 + j;
#pragma unroll 4
        for (int rr = warp; rr < BLK; rr += NW) {
            const double lap = fma(m_four, hh[(rr + 1) * 35 + j + 1],
                                   (hh[rr * 35 + j + 1] + hh[(rr + 2) * 35 + j + 1]) +
                                       (hh[(rr + 1) * 35 + j] + hh[(rr + 1) * 35 + j + 2]));
            const double dco = cu[rr * 33 + j] - ol[rr * 33 + j];
            if (!in_bounds((long long)(y0 + rr) * n + x0 + j, 0, (long long)n * n)) continue;
            out[(size_t)rr * n] = fma(m_two_thirds, dco, lap);
        }
        it_cur = it_next;
    }
    cp_async_wait<0>();
}

// ------------------------------------------------------------------------------------------------
// K2: x sweep (lane = row), 32-column chunks through shared memory
// ------------------------------------------------------------------------------------------------
// The recurrences are latency chains of FP64 operations; everything else is taken off their path:
// the 32 solver-table entries of a chunk are loaded once, coalesced (lane k holds entry k), and
// broadcast with shuffles as the chain walks the chunk, and a chunk's 32 x 32 field values are all
// in flight before the chain starts.
__global__ void __launch_bounds__(BLK) ch_xsolve_kernel(const GridDev* __restrict__ grids,
                                                        const Item* __restrict__ items, int n_items,
                                                        unsigned int* counter) {
    __shared__ double blk[BLK][BLK + 1];
    __shared__ int s_item;
    const int lane = threadIdx.x;
    const unsigned FULL = 0xffffffffu;
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        double* rows = gd.tmp + (size_t)item.block * BLK * n;   // 32 rows, stride n
        const int nchunk = n / BLK;
        // forward elimination of the banded (n-2) x (n-2) block, row = lane
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        for (int ch = 0; ch < nchunk; ++ch) {
            const int cx = ch * BLK;
            const int il = cx + lane;
            const double tds = il < m ? ds[il] : 0.0, tdl = il < m ? dl[il] : 0.0, trd = il < m ? rd[il] : 0.0;
            double v[BLK];
#pragma unroll
            for (int rr = 0; rr < BLK; ++rr) v[rr] = rows[(size_t)rr * n + il];
#pragma unroll
            for (int rr = 0; rr < BLK; ++rr) blk[rr][lane] = v[rr];
            __syncwarp();
#pragma unroll
            for (int k = 0; k < BLK; ++k) {
                const int i = cx + k;
                const double x = blk[lane][k];
                const double a_s = __shfl_sync(FULL, tds, k), a_l = __shfl_sync(FULL, tdl, k);
                const double a_r = __shfl_sync(FULL, trd, k);
                if (i < m) {
                    double t = fma(-a_s, b2, x);
                    t = fma(-a_l, b1, t);
                    t *= a_r;
                    b2 = b1;
                    b1 = t;
                    blk[lane][k] = t;
                } else if (i == m) {
                    r2 = x;
                } else {
                    r1 = x;
                }
            }
            __syncwarp();
#pragma unroll
            for (int rr = 0; rr < BLK; ++rr)
                if (in_bounds((long long)(item.block * BLK + rr) * n + il, 0, (long long)n * n))
                    rows[(size_t)rr * n + il] = blk[rr][lane];
            __syncwarp();
        }
        // backward substitution, chunks in reverse
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        for (int ch = nchunk - 1; ch >= 0; --ch) {
            const int cx = ch * BLK;
            const int il = cx + lane;
            const double tdu = il < m ? du[il] : 0.0, tdw = il < m ? dw[il] : 0.0;
            double v[BLK];
#pragma unroll
            for (int rr = 0; rr < BLK; ++rr) v[rr] = rows[(size_t)rr * n + il];
#pragma unroll
            for (int rr = 0; rr < BLK; ++rr) blk[rr][lane] = v[rr];
            __syncwarp();
#pragma unroll
            for (int k = BLK - 1; k >= 0; --k) {
                const int i = cx + k;
                const double a_u = __shfl_sync(FULL, tdu, k), a_w = __shfl_sync(FULL, tdw, k);
                if (i < m) {
                    double y = fma(-a_u, f1, blk[lane][k]);
                    y = fma(-a_w, f2, y);
                    f2 = f1;
                    f1 = y;
                    blk[lane][k] = y;
                    if (i == 0) y0v = y;
                    if (i == 1) y1v = y;
                    if (i == m - 2) ym2 = y;
                    if (i == m - 1) ym1 = y;
                }
            }
            __syncwarp();
#pragma unroll
            for (int rr = 0; rr < BLK; ++rr)
                if (in_bounds((long long)(item.block * BLK + rr) * n + il, 0, (long long)n * n))
                    rows[(size_t)rr * n + il] = blk[rr][lane];
            __syncwarp();
        }
        // the last two unknowns through the 2 x 2 Schur complement (BatchHyper.cu:195-227)
        const double* om = tab + 7 * m;
        const double a = om[4], b = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + b * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        double* row = rows + (size_t)lane * n;
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        row[n - 2] = x2;
        row[n - 1] = x1;
        // kept apart as well: the y sweep overwrites columns n-2 and n-1 of tmp while other warps still
        // need them for the rank-2 correction
        const int gy = item.block * BLK + lane;
        if (in_bounds(2 * gy + 1, 0, 2 * n)) {
            gd.ends[2 * gy] = x2;
            gd.ends[2 * gy + 1] = x1;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// K3: y sweep (lane = column) + the update
// ------------------------------------------------------------------------------------------------
// Rows are taken 32 at a time: the batch's field values are loaded into registers first (32 loads
// in flight per lane) and the batch's table entries / row ends are loaded coalesced and broadcast
// with shuffles, so the FP64 recurrence does not wait on memory.
// CH rows per batch (16 or 32): the three CH-deep register arrays of the update set the register use,
// hence how many warps fit on an SM (the tuned choice, ChConfig).
template <int CH>
__global__ void __launch_bounds__(BLK) ch_ysolve_kernel(const GridDev* __restrict__ grids,
                                                        const Item* __restrict__ items, int n_items, int parity,
                                                        unsigned int* counter) {
    __shared__ int s_item;
    const int lane = threadIdx.x;
    const unsigned FULL = 0xffffffffu;
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        const double* inv1 = tab + 5 * m;
        const double* inv2 = tab + 6 * m;
        const int x = item.block * BLK + lane;
        double* t = gd.tmp;
        const double* ends = gd.ends;
        // x sweep's rank-2 correction for this column (BatchHyper.cu:233-259): applied on read
        const bool corr = x < m;
        const double cx1 = corr ? inv1[x] : 0.0;
        const double cx2 = corr ? inv2[x] : 0.0;
        const int nb = n / CH;
        // forward elimination along y
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        for (int bb = 0; bb < nb; ++bb) {
            const int yb = bb * CH, yl = yb + lane;
            const double tds = yl < m ? ds[yl] : 0.0, tdl = yl < m ? dl[yl] : 0.0, trd = yl < m ? rd[yl] : 0.0;
            const double e2 = yl < n ? ends[2 * yl] : 0.0, e1 = yl < n ? ends[2 * yl + 1] : 0.0;
            double v[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) v[k] = t[(size_t)(yb + k) * n + x];
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const int y = yb + k;
                const double c2 = __shfl_sync(FULL, e2, k), c1 = __shfl_sync(FULL, e1, k);
                const double a_s = __shfl_sync(FULL, tds, k), a_l = __shfl_sync(FULL, tdl, k);
                const double a_r = __shfl_sync(FULL, trd, k);
                const double val = corr ? fma(-cx1, c2, fma(-cx2, c1, v[k])) : v[k];
                if (y < m) {
                    double w = fma(-a_s, b2, val);
                    w = fma(-a_l, b1, w);
                    w *= a_r;
                    b2 = b1;
                    b1 = w;
                    v[k] = w;
                } else if (y == m) {
                    r2 = val;
                } else {
                    r1 = val;
                }
            }
#pragma unroll
            for (int k = 0; k < CH; ++k)
                if (yb + k < m && in_bounds((long long)(yb + k) * n + x, 0, (long long)n * n))
                    t[(size_t)(yb + k) * n + x] = v[k];
        }
        // backward substitution
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        for (int bb = nb - 1; bb >= 0; --bb) {
            const int yb = bb * CH, yl = yb + lane;
            const double tdu = yl < m ? du[yl] : 0.0, tdw = yl < m ? dw[yl] : 0.0;
            double v[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) v[k] = (yb + k < m) ? t[(size_t)(yb + k) * n + x] : 0.0;
#pragma unroll
            for (int k = CH - 1; k >= 0; --k) {
                const int y = yb + k;
                const double a_u = __shfl_sync(FULL, tdu, k), a_w = __shfl_sync(FULL, tdw, k);
                if (y < m) {
                    double w = fma(-a_u, f1, v[k]);
                    w = fma(-a_w, f2, w);
                    f2 = f1;
                    f1 = w;
                    v[k] = w;
                    if (y == m - 1) ym1 = w;
                    if (y == m - 2) ym2 = w;
                    if (y == 1) y1v = w;
                    if (y == 0) y0v = w;
                }
            }
#pragma unroll
            for (int k = 0; k < CH; ++k)
                if (yb + k < m && in_bounds((long long)(yb + k) * n + x, 0, (long long)n * n))
                    t[(size_t)(yb + k) * n + x] = v[k];
        }
        const double* om = tab + 7 * m;
        const double a = om[4], b = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + b * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        // cNew = cBar + delta over cOld (cuPentCahnADI.cu:58-69, 89-100)
        const double two = ((const volatile double*)g_rhs_factors)[0];   // register operand, as in K1
        const double* cur = parity ? gd.buf[1] : gd.buf[0];
        double* old = parity ? gd.buf[0] : gd.buf[1];
        for (int bb = 0; bb < nb; ++bb) {
            const int yb = bb * CH, yl = yb + lane;
            const double ti1 = yl < m ? inv1[yl] : 0.0, ti2 = yl < m ? inv2[yl] : 0.0;
            double v[CH], cv[CH], ov[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const size_t q = (size_t)(yb + k) * n + x;
                v[k] = (yb + k < m) ? t[q] : 0.0;
                cv[k] = cur[q];
                ov[k] = old[q];
            }
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const int y = yb + k;
                const double a1 = __shfl_sync(FULL, ti1, k), a2 = __shfl_sync(FULL, ti2, k);
                double dlt;
                if (y < m) dlt = fma(-a1, x2, fma(-a2, x1, v[k]));
                else dlt = (y == m) ? x2 : x1;
                const double cbar = fma(two, cv[k], -ov[k]);
                if (in_bounds((long long)y * n + x, 0, (long long)n * n)) old[(size_t)y * n + x] = cbar + dlt;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------------
// K2 / K3, pipelined: the same sweeps with the field values of chunk c+1 copied into shared memory
// (cp.async, double buffered) while the recurrence runs over chunk c
// ------------------------------------------------------------------------------------------------
// The recurrences are latency-bound: a warp's chain issues one dependent FP64 operation at a time, so
// the FP64 pipe stays busy only while other warps have work. In the kernels above a chunk's loads start
// when its chain is about to run, and the values they stage in registers (32 per lane) limit the warps
// per SM. Here the loads of the next chunk are in flight during the current chain, they occupy no
// registers, and the table entries of the next chunk are read one chunk ahead. The arithmetic, its order
// and so every result are those of the kernels above.

// x sweep (lane = row) over XC-column chunks. Each lane copies, and later writes back, the elements
// e = lane + 32 j of a chunk (row e / XC, column e % XC): one row segment (XC = 32) or two (XC = 16) per
// instruction, coalesced; a lane reads back in the backward pass exactly what it stored in the forward
// pass, so program order alone orders those accesses.
template <int XC>
__global__ void __launch_bounds__(BLK) ch_xsolve_pipe_kernel(const GridDev* __restrict__ grids,
                                                             const Item* __restrict__ items, int n_items,
                                                             unsigned int* counter) {
    __shared__ double blk[2][BLK][XC + 1];
    __shared__ int s_item;
    const int lane = threadIdx.x;
    const unsigned FULL = 0xffffffffu;
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        double* rows = gd.tmp + (size_t)item.block * BLK * n;   // 32 rows, stride n
        const int nchunk = n / XC;
        // element e = lane + 32 j sits at row j * RPI + lr, column lc of the chunk
        constexpr int RPI = BLK / XC;
        const int lr = lane / XC, lc = lane % XC;
        const size_t step = (size_t)RPI * n;
        auto issue = [&](int c, int b) {
            const double* src = rows + (size_t)lr * n + c * XC + lc;
#pragma unroll 4
            for (int j = 0; j < XC; ++j, src += step) cp_async8(&blk[b][j * RPI + lr][lc], src);
            cp_async_commit();
        };
        auto write_back = [&](int c, int b) {
            double* dst = rows + (size_t)lr * n + c * XC + lc;
#pragma unroll 4
            for (int j = 0; j < XC; ++j, dst += step)
                if (in_bounds(dst - gd.tmp, 0, (long long)n * n)) *dst = blk[b][j * RPI + lr][lc];
        };
        // forward elimination of the banded (n-2) x (n-2) block
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        issue(0, 0);
        double tds = lane < m ? ds[lane] : 0.0, tdl = lane < m ? dl[lane] : 0.0, trd = lane < m ? rd[lane] : 0.0;
        for (int c = 0; c < nchunk; ++c) {
            const int b = c & 1, cx = c * XC;
            double nds = 0.0, ndl = 0.0, nrd = 0.0;
            if (c + 1 < nchunk) {
                issue(c + 1, b ^ 1);
                const int il = cx + XC + lane;
                if (il < m && lane < XC) { nds = ds[il]; ndl = dl[il]; nrd = rd[il]; }
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < XC; ++k) {
                const int i = cx + k;
                const double x = blk[b][lane][k];
                const double a_s = __shfl_sync(FULL, tds, k), a_l = __shfl_sync(FULL, tdl, k);
                const double a_r = __shfl_sync(FULL, trd, k);
                if (i < m) {
                    double t = fma(-a_s, b2, x);
                    t = fma(-a_l, b1, t);
                    t *= a_r;
                    b2 = b1;
                    b1 = t;
                    blk[b][lane][k] = t;
                } else if (i == m) {
                    r2 = x;
                } else {
                    r1 = x;
                }
            }
            __syncwarp();
            write_back(c, b);
            __syncwarp();   // buffer b is refilled next iteration
            tds = nds; tdl = ndl; trd = nrd;
        }
        // backward substitution, chunks in reverse
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        issue(nchunk - 1, 0);
        int il0 = (nchunk - 1) * XC + lane;
        double tdu = (il0 < m && lane < XC) ? du[il0] : 0.0, tdw = (il0 < m && lane < XC) ? dw[il0] : 0.0;
        for (int j = 0; j < nchunk; ++j) {
            const int c = nchunk - 1 - j, b = j & 1, cx = c * XC;
            double ndu = 0.0, ndw = 0.0;
            if (c > 0) {
                issue(c - 1, b ^ 1);
                const int il = cx - XC + lane;
                if (il < m && lane < XC) { ndu = du[il]; ndw = dw[il]; }
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncwarp();
#pragma unroll
            for (int k = XC - 1; k >= 0; --k) {
                const int i = cx + k;
                const double a_u = __shfl_sync(FULL, tdu, k), a_w = __shfl_sync(FULL, tdw, k);
                if (i < m) {
                    double y = fma(-a_u, f1, blk[b][lane][k]);
                    y = fma(-a_w, f2, y);
                    f2 = f1;
                    f1 = y;
                    blk[b][lane][k] = y;
                    if (i == 0) y0v = y;
                    if (i == 1) y1v = y;
                    if (i == m - 2) ym2 = y;
                    if (i == m - 1) ym1 = y;
                }
            }
            __syncwarp();
            write_back(c, b);
            __syncwarp();
            tdu = ndu; tdw = ndw;
        }
        // the last two unknowns through the 2 x 2 Schur complement (BatchHyper.cu:195-227)
        const double* om = tab + 7 * m;
        const double a = om[4], b = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + b * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        double* row = rows + (size_t)lane * n;
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        row[n - 2] = x2;
        row[n - 1] = x1;
        const int gy = item.block * BLK + lane;
        if (in_bounds(2 * gy + 1, 0, 2 * n)) {
            gd.ends[2 * gy] = x2;
            gd.ends[2 * gy + 1] = x1;
        }
    }
}

// The same x sweep with XC-column chunks (8 or 16) whose table entries every lane holds in registers, read with
// uniform (broadcast) loads when the chunk starts and before its field copies are awaited: the chain
// then takes no shuffle. The arithmetic is that of the kernels above.
template <int XC>
__global__ void __launch_bounds__(BLK) ch_xsolve_pipe_rt_kernel(const GridDev* __restrict__ grids,
                                                                const Item* __restrict__ items, int n_items,
                                                                unsigned int* counter) {
    constexpr int RPI = BLK / XC;
    __shared__ double blk[2][BLK][XC + 1];
    __shared__ int s_item;
    const int lane = threadIdx.x;
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        double* rows = gd.tmp + (size_t)item.block * BLK * n;
        const int nchunk = n / XC;
        const int lr = lane / XC, lc = lane % XC;
        const size_t step = (size_t)RPI * n;
        auto issue = [&](int c, int b) {
            const double* src = rows + (size_t)lr * n + c * XC + lc;
#pragma unroll 4
            for (int j = 0; j < XC; ++j, src += step) cp_async8(&blk[b][j * RPI + lr][lc], src);
            cp_async_commit();
        };
        auto write_back = [&](int c, int b) {
            double* dst = rows + (size_t)lr * n + c * XC + lc;
#pragma unroll 4
            for (int j = 0; j < XC; ++j, dst += step)
                if (in_bounds(dst - gd.tmp, 0, (long long)n * n)) *dst = blk[b][j * RPI + lr][lc];
        };
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        issue(0, 0);
        for (int c = 0; c < nchunk; ++c) {
            const int b = c & 1, cx = c * XC;
            double ts[XC], tl[XC], tr[XC];
#pragma unroll
            for (int k = 0; k < XC; ++k) {
                const bool in = cx + k < m;
                ts[k] = in ? __ldg(ds + cx + k) : 0.0;
                tl[k] = in ? __ldg(dl + cx + k) : 0.0;
                tr[k] = in ? __ldg(rd + cx + k) : 0.0;
            }
            if (c + 1 < nchunk) {
                issue(c + 1, b ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < XC; ++k) {
                const int i = cx + k;
                const double x = blk[b][lane][k];
                if (i < m) {
                    double t = fma(-ts[k], b2, x);
                    t = fma(-tl[k], b1, t);
                    t *= tr[k];
                    b2 = b1;
                    b1 = t;
                    blk[b][lane][k] = t;
                } else if (i == m) {
                    r2 = x;
                } else {
                    r1 = x;
                }
            }
            __syncwarp();
            write_back(c, b);
            __syncwarp();
        }
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        issue(nchunk - 1, 0);
        for (int j = 0; j < nchunk; ++j) {
            const int c = nchunk - 1 - j, b = j & 1, cx = c * XC;
            double tu[XC], tw[XC];
#pragma unroll
            for (int k = 0; k < XC; ++k) {
                const bool in = cx + k < m;
                tu[k] = in ? __ldg(du + cx + k) : 0.0;
                tw[k] = in ? __ldg(dw + cx + k) : 0.0;
            }
            if (c > 0) {
                issue(c - 1, b ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncwarp();
#pragma unroll
            for (int k = XC - 1; k >= 0; --k) {
                const int i = cx + k;
                if (i < m) {
                    double y = fma(-tu[k], f1, blk[b][lane][k]);
                    y = fma(-tw[k], f2, y);
                    f2 = f1;
                    f1 = y;
                    blk[b][lane][k] = y;
                    if (i == 0) y0v = y;
                    if (i == 1) y1v = y;
                    if (i == m - 2) ym2 = y;
                    if (i == m - 1) ym1 = y;
                }
            }
            __syncwarp();
            write_back(c, b);
            __syncwarp();
        }
        const double* om = tab + 7 * m;
        const double a = om[4], bq = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + bq * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        double* row = rows + (size_t)lane * n;
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        row[n - 2] = x2;
        row[n - 1] = x1;
        const int gy = item.block * BLK + lane;
        if (in_bounds(2 * gy + 1, 0, 2 * n)) {
            gd.ends[2 * gy] = x2;
            gd.ends[2 * gy + 1] = x1;
        }
    }
}

// y sweep (lane = column) with CH-row batches copied one batch ahead. Each lane reads only its own
// column, which it copied itself, so no warp barrier is needed around the buffers; results are stored
// to global memory as the chain produces them. The update runs in register batches of 8 rows.
template <int CH>
__global__ void __launch_bounds__(BLK) ch_ysolve_pipe_kernel(const GridDev* __restrict__ grids,
                                                             const Item* __restrict__ items, int n_items, int parity,
                                                             unsigned int* counter) {
    __shared__ double vb[2][CH][BLK];
    __shared__ int s_item;
    constexpr int UD = 8;
    const int lane = threadIdx.x;
    const unsigned FULL = 0xffffffffu;
    const double two = ((const volatile double*)g_rhs_factors)[0];
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        const double* inv1 = tab + 5 * m;
        const double* inv2 = tab + 6 * m;
        const int x = item.block * BLK + lane;
        double* t = gd.tmp;
        const double* ends = gd.ends;
        const bool corr = x < m;
        const double cx1 = corr ? inv1[x] : 0.0;
        const double cx2 = corr ? inv2[x] : 0.0;
        const int nb = n / CH;
        auto issue = [&](int bb, int b, bool below_m) {
            const int yb = bb * CH;
            const double* src = t + (size_t)yb * n + x;
#pragma unroll 4
            for (int k = 0; k < CH; ++k, src += n)
                if (!below_m || yb + k < m) cp_async8(&vb[b][k][lane], src);
            cp_async_commit();
        };
        // forward elimination along y
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        issue(0, 0, false);
        double tds = 0.0, tdl = 0.0, trd = 0.0, e2 = 0.0, e1 = 0.0;
        if (lane < CH) {
            if (lane < m) { tds = ds[lane]; tdl = dl[lane]; trd = rd[lane]; }
            e2 = ends[2 * lane];
            e1 = ends[2 * lane + 1];
        }
        for (int bb = 0; bb < nb; ++bb) {
            const int b = bb & 1, yb = bb * CH;
            double nds = 0.0, ndl = 0.0, nrd = 0.0, ne2 = 0.0, ne1 = 0.0;
            if (bb + 1 < nb) {
                issue(bb + 1, b ^ 1, false);
                const int yl = yb + CH + lane;
                if (lane < CH) {
                    if (yl < m) { nds = ds[yl]; ndl = dl[yl]; nrd = rd[yl]; }
                    ne2 = ends[2 * yl];
                    ne1 = ends[2 * yl + 1];
                }
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const int y = yb + k;
                const double c2 = __shfl_sync(FULL, e2, k), c1 = __shfl_sync(FULL, e1, k);
                const double a_s = __shfl_sync(FULL, tds, k), a_l = __shfl_sync(FULL, tdl, k);
                const double a_r = __shfl_sync(FULL, trd, k);
                const double vk = vb[b][k][lane];
                const double val = corr ? fma(-cx1, c2, fma(-cx2, c1, vk)) : vk;
                if (y < m) {
                    double w = fma(-a_s, b2, val);
                    w = fma(-a_l, b1, w);
                    w *= a_r;
                    b2 = b1;
                    b1 = w;
                    if (in_bounds((long long)y * n + x, 0, (long long)n * n)) t[(size_t)y * n + x] = w;
                } else if (y == m) {
                    r2 = val;
                } else {
                    r1 = val;
                }
            }
            tds = nds; tdl = ndl; trd = nrd; e2 = ne2; e1 = ne1;
        }
        // backward substitution (rows below m only; the lane re-reads what it stored above)
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        issue(nb - 1, 0, true);
        int yl0 = (nb - 1) * CH + lane;
        double tdu = (lane < CH && yl0 < m) ? du[yl0] : 0.0, tdw = (lane < CH && yl0 < m) ? dw[yl0] : 0.0;
        for (int j = 0; j < nb; ++j) {
            const int bb = nb - 1 - j, b = j & 1, yb = bb * CH;
            double ndu = 0.0, ndw = 0.0;
            if (bb > 0) {
                issue(bb - 1, b ^ 1, true);
                const int yl = yb - CH + lane;
                if (lane < CH && yl < m) { ndu = du[yl]; ndw = dw[yl]; }
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int k = CH - 1; k >= 0; --k) {
                const int y = yb + k;
                const double a_u = __shfl_sync(FULL, tdu, k), a_w = __shfl_sync(FULL, tdw, k);
                if (y < m) {
                    double w = fma(-a_u, f1, vb[b][k][lane]);
                    w = fma(-a_w, f2, w);
                    f2 = f1;
                    f1 = w;
                    if (in_bounds((long long)y * n + x, 0, (long long)n * n)) t[(size_t)y * n + x] = w;
                    if (y == m - 1) ym1 = w;
                    if (y == m - 2) ym2 = w;
                    if (y == 1) y1v = w;
                    if (y == 0) y0v = w;
                }
            }
            tdu = ndu; tdw = ndw;
        }
        const double* om = tab + 7 * m;
        const double a = om[4], b = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + b * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        // cNew = cBar + delta over cOld (cuPentCahnADI.cu:58-69, 89-100)
        const double* cur = parity ? gd.buf[1] : gd.buf[0];
        double* old = parity ? gd.buf[0] : gd.buf[1];
        for (int yb = 0; yb < n; yb += UD) {
            const int yl = yb + (lane & (UD - 1));
            const double ti1 = yl < m ? inv1[yl] : 0.0, ti2 = yl < m ? inv2[yl] : 0.0;
            double v[UD], cv[UD], ov[UD];
#pragma unroll
            for (int k = 0; k < UD; ++k) {
                const size_t q = (size_t)(yb + k) * n + x;
                v[k] = (yb + k < m) ? t[q] : 0.0;
                cv[k] = cur[q];
                ov[k] = old[q];
            }
#pragma unroll
            for (int k = 0; k < UD; ++k) {
                const int y = yb + k;
                const double a1 = __shfl_sync(FULL, ti1, k), a2 = __shfl_sync(FULL, ti2, k);
                double dlt;
                if (y < m) dlt = fma(-a1, x2, fma(-a2, x1, v[k]));
                else dlt = (y == m) ? x2 : x1;
                const double cbar = fma(two, cv[k], -ov[k]);
                if (in_bounds((long long)y * n + x, 0, (long long)n * n)) old[(size_t)y * n + x] = cbar + dlt;
            }
        }
    }
}

// The same y sweep with the batch's table entries (pivots, multipliers, x-sweep row ends, update
// factors) held in registers by every lane, read with uniform loads before the batch's copies are
// awaited: the chain takes no shuffle. The arithmetic is that of the kernels above.
template <int CH>
__global__ void __launch_bounds__(BLK) ch_ysolve_pipe_rt_kernel(const GridDev* __restrict__ grids,
                                                             const Item* __restrict__ items, int n_items, int parity,
                                                             unsigned int* counter) {
    __shared__ double vb[2][CH][BLK];
    __shared__ int s_item;
    constexpr int UD = 8;
    const int lane = threadIdx.x;
    const double two = ((const volatile double*)g_rhs_factors)[0];
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        const double* inv1 = tab + 5 * m;
        const double* inv2 = tab + 6 * m;
        const int x = item.block * BLK + lane;
        double* t = gd.tmp;
        const double* ends = gd.ends;
        const bool corr = x < m;
        const double cx1 = corr ? inv1[x] : 0.0;
        const double cx2 = corr ? inv2[x] : 0.0;
        const int nb = n / CH;
        auto issue = [&](int bb, int b, bool below_m) {
            const int yb = bb * CH;
            const double* src = t + (size_t)yb * n + x;
#pragma unroll 4
            for (int k = 0; k < CH; ++k, src += n)
                if (!below_m || yb + k < m) cp_async8(&vb[b][k][lane], src);
            cp_async_commit();
        };
        // forward elimination along y
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        issue(0, 0, false);
        for (int bb = 0; bb < nb; ++bb) {
            const int b = bb & 1, yb = bb * CH;
            double ts[CH], tl[CH], tr[CH], te2[CH], te1[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const bool in = yb + k < m;
                ts[k] = in ? __ldg(ds + yb + k) : 0.0;
                tl[k] = in ? __ldg(dl + yb + k) : 0.0;
                tr[k] = in ? __ldg(rd + yb + k) : 0.0;
                te2[k] = ends[2 * (yb + k)];
                te1[k] = ends[2 * (yb + k) + 1];
            }
            if (bb + 1 < nb) {
                issue(bb + 1, b ^ 1, false);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const int y = yb + k;
                const double c2 = te2[k], c1 = te1[k];
                const double a_s = ts[k], a_l = tl[k];
                const double a_r = tr[k];
                const double vk = vb[b][k][lane];
                const double val = corr ? fma(-cx1, c2, fma(-cx2, c1, vk)) : vk;
                if (y < m) {
                    double w = fma(-a_s, b2, val);
                    w = fma(-a_l, b1, w);
                    w *= a_r;
                    b2 = b1;
                    b1 = w;
                    if (in_bounds((long long)y * n + x, 0, (long long)n * n)) t[(size_t)y * n + x] = w;
                } else if (y == m) {
                    r2 = val;
                } else {
                    r1 = val;
                }
            }
        }
        // backward substitution (rows below m only; the lane re-reads what it stored above)
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        issue(nb - 1, 0, true);
        for (int j = 0; j < nb; ++j) {
            const int bb = nb - 1 - j, b = j & 1, yb = bb * CH;
            double tu[CH], tw[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const bool in = yb + k < m;
                tu[k] = in ? __ldg(du + yb + k) : 0.0;
                tw[k] = in ? __ldg(dw + yb + k) : 0.0;
            }
            if (bb > 0) {
                issue(bb - 1, b ^ 1, true);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int k = CH - 1; k >= 0; --k) {
                const int y = yb + k;
                const double a_u = tu[k], a_w = tw[k];
                if (y < m) {
                    double w = fma(-a_u, f1, vb[b][k][lane]);
                    w = fma(-a_w, f2, w);
                    f2 = f1;
                    f1 = w;
                    if (in_bounds((long long)y * n + x, 0, (long long)n * n)) t[(size_t)y * n + x] = w;
                    if (y == m - 1) ym1 = w;
                    if (y == m - 2) ym2 = w;
                    if (y == 1) y1v = w;
                    if (y == 0) y0v = w;
                }
            }
        }
        const double* om = tab + 7 * m;
        const double a = om[4], b = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + b * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        // cNew = cBar + delta over cOld (cuPentCahnADI.cu:58-69, 89-100)
        const double* cur = parity ? gd.buf[1] : gd.buf[0];
        double* old = parity ? gd.buf[0] : gd.buf[1];
        for (int yb = 0; yb < n; yb += UD) {
            double i1[UD], i2[UD];
#pragma unroll
            for (int k = 0; k < UD; ++k) {
                const bool in = yb + k < m;
                i1[k] = in ? __ldg(inv1 + yb + k) : 0.0;
                i2[k] = in ? __ldg(inv2 + yb + k) : 0.0;
            }
            double v[UD], cv[UD], ov[UD];
#pragma unroll
            for (int k = 0; k < UD; ++k) {
                const size_t q = (size_t)(yb + k) * n + x;
                v[k] = (yb + k < m) ? t[q] : 0.0;
                cv[k] = cur[q];
                ov[k] = old[q];
            }
#pragma unroll
            for (int k = 0; k < UD; ++k) {
                const int y = yb + k;
                const double a1 = i1[k], a2 = i2[k];
                double dlt;
                if (y < m) dlt = fma(-a1, x2, fma(-a2, x1, v[k]));
                else dlt = (y == m) ? x2 : x1;
                const double cbar = fma(two, cv[k], -ov[k]);
                if (in_bounds((long long)y * n + x, 0, (long long)n * n)) old[(size_t)y * n + x] = cbar + dlt;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------------
// K3 split in three (configurations with ysplit): for batches too small to fill the GPU with line warps.
// ch_xcorr_kernel applies the x sweep's rank-2 correction to the work field, ch_ysolve_split_kernel runs
// the y recurrences alone and leaves each column's two cyclic unknowns in GridDev::ends, and
// ch_update_kernel forms cNew = cBar + delta. The expressions are those of ch_ysolve_pipe_rt_kernel, so
// the results are the same bit for bit. A warp's FP64 instruction holds its sub-partition's FP64 pipe for
// 64 cycles however few lanes it has, so a column's time in the y sweep is its warp's FP64 instruction
// count: 5 per element here against 11 in the fused kernel, while the correction and the update spread
// over every SM as element-wise kernels.
// ------------------------------------------------------------------------------------------------
// One 32 x 32 block of a grid per CTA (the right-hand side's work list): t[y][x] -= inv1[x] x2(y) +
// inv2[x] x1(y) for the columns x < n - 2 of the block's rows, as fma(-inv1, x2, fma(-inv2, x1, t)).
__global__ void __launch_bounds__(256) ch_xcorr_kernel(const GridDev* __restrict__ grids,
                                                       const Item* __restrict__ items) {
    const Item item = items[blockIdx.x];
    const GridDev gd = grids[item.grid];
    const int n = gd.n, m = n - 2;
    const int bpr = n / BLK;
    const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
    const int x = x0 + (threadIdx.x & (BLK - 1));
    if (x >= m) return;
    const double cx1 = gd.tab[5 * m + x], cx2 = gd.tab[6 * m + x];
    for (int r = threadIdx.x / BLK; r < BLK; r += blockDim.x / BLK) {
        const int y = y0 + r;
        const long long q = (long long)y * n + x;
        if (!in_bounds(q, 0, (long long)n * n)) continue;
        gd.tmp[q] = fma(-cx1, gd.ends[2 * y], fma(-cx2, gd.ends[2 * y + 1], gd.tmp[q]));
    }
}

// One 32 x 32 block per CTA: cNew = cBar + delta written over cOld (cuPentCahnADI.cu:58-69, 89-100), delta
// from the banded y solution in the work field and the column's cyclic unknowns in GridDev::ends.
__global__ void __launch_bounds__(256) ch_update_kernel(const GridDev* __restrict__ grids,
                                                        const Item* __restrict__ items, int parity) {
    const Item item = items[blockIdx.x];
    const GridDev gd = grids[item.grid];
    const int n = gd.n, m = n - 2;
    const int bpr = n / BLK;
    const int y0 = (item.block / bpr) * BLK, x0 = (item.block % bpr) * BLK;
    const int x = x0 + (threadIdx.x & (BLK - 1));
    const double two = ((const volatile double*)g_rhs_factors)[0];
    const double x2 = gd.ends[2 * x], x1 = gd.ends[2 * x + 1];
    const double* cur = parity ? gd.buf[1] : gd.buf[0];
    double* old = parity ? gd.buf[0] : gd.buf[1];
    for (int r = threadIdx.x / BLK; r < BLK; r += blockDim.x / BLK) {
        const int y = y0 + r;
        const long long q = (long long)y * n + x;
        double dlt;
        if (y < m) dlt = fma(-gd.tab[5 * m + y], x2, fma(-gd.tab[6 * m + y], x1, gd.tmp[q]));
        else dlt = (y == m) ? x2 : x1;
        const double cbar = fma(two, cur[q], -old[q]);
        if (in_bounds(q, 0, (long long)n * n)) old[q] = cbar + dlt;
    }
}

template <int CH>
__global__ void __launch_bounds__(BLK) ch_ysolve_split_kernel(const GridDev* __restrict__ grids,
                                                             const Item* __restrict__ items, int n_items, int parity,
                                                             unsigned int* counter) {
    __shared__ double vb[2][CH][BLK];
    __shared__ int s_item;
    const int lane = threadIdx.x;
    for (;;) {
        if (lane == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncwarp();
        const int it = s_item;
        __syncwarp();
        if (it >= n_items) break;
        const Item item = items[it];
        const GridDev gd = grids[item.grid];
        const int n = gd.n, m = n - 2;
        const double* tab = gd.tab;
        const double* ds = tab;
        const double* dl = tab + m;
        const double* rd = tab + 2 * m;
        const double* du = tab + 3 * m;
        const double* dw = tab + 4 * m;
        const int x = item.block * BLK + lane;
        double* t = gd.tmp;
        const int nb = n / CH;
        auto issue = [&](int bb, int b, bool below_m) {
            const int yb = bb * CH;
            const double* src = t + (size_t)yb * n + x;
#pragma unroll 4
            for (int k = 0; k < CH; ++k, src += n)
                if (!below_m || yb + k < m) cp_async8(&vb[b][k][lane], src);
            cp_async_commit();
        };
        // forward elimination along y
        double b1 = 0.0, b2 = 0.0, r2 = 0.0, r1 = 0.0;
        issue(0, 0, false);
        for (int bb = 0; bb < nb; ++bb) {
            const int b = bb & 1, yb = bb * CH;
            double ts[CH], tl[CH], tr[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const bool in = yb + k < m;
                ts[k] = in ? __ldg(ds + yb + k) : 0.0;
                tl[k] = in ? __ldg(dl + yb + k) : 0.0;
                tr[k] = in ? __ldg(rd + yb + k) : 0.0;
            }
            if (bb + 1 < nb) {
                issue(bb + 1, b ^ 1, false);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const int y = yb + k;
                const double a_s = ts[k], a_l = tl[k];
                const double a_r = tr[k];
                const double vk = vb[b][k][lane];
                const double val = vk;   // corrected by ch_xcorr_kernel
                if (y < m) {
                    double w = fma(-a_s, b2, val);
                    w = fma(-a_l, b1, w);
                    w *= a_r;
                    b2 = b1;
                    b1 = w;
                    if (in_bounds((long long)y * n + x, 0, (long long)n * n)) t[(size_t)y * n + x] = w;
                } else if (y == m) {
                    r2 = val;
                } else {
                    r1 = val;
                }
            }
        }
        // backward substitution (rows below m only; the lane re-reads what it stored above)
        double f1 = 0.0, f2 = 0.0, y0v = 0.0, y1v = 0.0, ym2 = 0.0, ym1 = 0.0;
        issue(nb - 1, 0, true);
        for (int j = 0; j < nb; ++j) {
            const int bb = nb - 1 - j, b = j & 1, yb = bb * CH;
            double tu[CH], tw[CH];
#pragma unroll
            for (int k = 0; k < CH; ++k) {
                const bool in = yb + k < m;
                tu[k] = in ? __ldg(du + yb + k) : 0.0;
                tw[k] = in ? __ldg(dw + yb + k) : 0.0;
            }
            if (bb > 0) {
                issue(bb - 1, b ^ 1, true);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int k = CH - 1; k >= 0; --k) {
                const int y = yb + k;
                const double a_u = tu[k], a_w = tw[k];
                if (y < m) {
                    double w = fma(-a_u, f1, vb[b][k][lane]);
                    w = fma(-a_w, f2, w);
                    f2 = f1;
                    f1 = w;
                    if (in_bounds((long long)y * n + x, 0, (long long)n * n)) t[(size_t)y * n + x] = w;
                    if (y == m - 1) ym1 = w;
                    if (y == m - 2) ym2 = w;
                    if (y == 1) y1v = w;
                    if (y == 0) y0v = w;
                }
            }
        }
        const double* om = tab + 7 * m;
        const double a = om[4], b = om[5], d = om[6], e = om[7];
        const double nx2 = r2 - (e * y0v + a * ym2 + b * ym1);
        const double nx1 = r1 - (d * y0v + e * y1v + a * ym1);
        const double x2 = om[0] * nx2 + om[1] * nx1;
        const double x1 = om[2] * nx2 + om[3] * nx1;
        // the column's two cyclic unknowns, for ch_update_kernel (the x sweep's row ends were consumed
        // by ch_xcorr_kernel, so their buffer is free)
        gd.ends[2 * x] = x2;
        gd.ends[2 * x + 1] = x1;
    }
}

int ch_launches_per_step(const ChConfig& c) { return 3 + (c.rhs_split ? 1 : 0) + (c.ysplit ? 2 : 0); }

ChConfig ch_config(int index) {
    // {warps per right-hand-side CTA, y-sweep rows per batch, sweep kind, x-sweep columns per chunk (kinds 2,
    // 3), two-pass right-hand side}
    static const ChConfig tab[kChConfigs] = {
        {1, 32, 0, 16}, {2, 32, 0, 16}, {4, 32, 0, 16}, {1, 16, 0, 16}, {2, 16, 0, 16}, {4, 16, 0, 16},
        {2, 16, 1, 16}, {4, 16, 1, 16}, {2, 32, 1, 16}, {4, 32, 1, 16}, {4, 16, 2, 16}, {4, 32, 2, 16},
        {4, 8, 3, 16},  {4, 16, 3, 16}, {4, 8, 3, 8},   {4, 4, 3, 8},   {4, 4, 3, 16},
        {4, 8, 3, 16, 1}, {2, 8, 3, 16, 1}, {4, 8, 3, 16, 2}, {8, 8, 3, 16, 2}, {8, 8, 3, 16, 2, 1}};
    return tab[(index >= 0 && index < kChConfigs) ? index : 0];
}

void config_name(const ChConfig& c, char* name, size_t len) {
    if (c.pipe >= 2)
        snprintf(name, len, "rhs_warps%d%s_ychunk%d_pipe_regtab%s_xchunk%d%s", c.rhs_warps,
                 c.rhs_split == 2 ? "_2pass_pipe" : (c.rhs_split ? "_2pass" : ""),
                 c.y_chunk, c.pipe == 3 ? "_xy" : "", c.x_chunk, c.ysplit ? "_ysplit" : "");
    else
        snprintf(name, len, "rhs_warps%d_ychunk%d%s", c.rhs_warps, c.y_chunk, c.pipe ? "_pipe" : "");
}

// The two passes of the split right-hand side; pass 2 claims work through the step's fourth counter.
// Pass 2 runs in FP64 in both variants: the precision variant's h buffer holds FP32 values, whose FP64
// Laplacian is exact, so its mass is conserved to FP64 rounding (the one-pass kernel does the same).
// Pass 2 pipelined: dynamic shared memory beyond 48 KB, allowed once per device and kernel.
template <int NW>
static cudaError_t launch_rhs2_pipe(int grid, const GridDev* g, const Item* it, int n, int parity, unsigned int* ctr,
                                    cudaStream_t s) {
    static std::atomic<int> ready[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!ready[dev].load(std::memory_order_acquire)) {
        cudaError_t e = cudaFuncSetAttribute(ch_rhs2_pipe_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kRhs2PipeBytes);
        if (e != cudaSuccess) return e;
        ready[dev].store(1, std::memory_order_release);
    }
    ch_rhs2_pipe_kernel<NW><<<grid, NW * BLK, kRhs2PipeBytes, s>>>(g, it, n, parity, ctr);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_rhs2(int nw, int grid, const GridDev* g, const Item* it, int n, int parity,
                               unsigned int* ctr, cudaStream_t s, bool pipe, int sms) {
    if (pipe) {   // four CTAs per SM fit the double buffer
        const int gp = std::max(1, std::min(n, sms * 4));
        if (nw == 8) {
            ch_h_kernel<T, 8><<<grid, 8 * BLK, 0, s>>>(g, it, n, parity, ctr);
            return launch_rhs2_pipe<8>(gp, g, it, n, parity, ctr + 3, s);
        }
        if (nw == 4) {
            ch_h_kernel<T, 4><<<grid, 4 * BLK, 0, s>>>(g, it, n, parity, ctr);
            return launch_rhs2_pipe<4>(gp, g, it, n, parity, ctr + 3, s);
        }
        ch_h_kernel<T, 2><<<grid, 2 * BLK, 0, s>>>(g, it, n, parity, ctr);
        return launch_rhs2_pipe<2>(gp, g, it, n, parity, ctr + 3, s);
    }
    if (nw == 4) {
        ch_h_kernel<T, 4><<<grid, 4 * BLK, 0, s>>>(g, it, n, parity, ctr);
        ch_rhs2_kernel<double, 4><<<grid, 4 * BLK, 0, s>>>(g, it, n, parity, ctr + 3);
    } else {
        ch_h_kernel<T, 2><<<grid, 2 * BLK, 0, s>>>(g, it, n, parity, ctr);
        ch_rhs2_kernel<double, 2><<<grid, 2 * BLK, 0, s>>>(g, it, n, parity, ctr + 3);
    }
    return cudaGetLastError();
}

template <typename T>
static void launch_rhs(int nw, int grid, const GridDev* g, const Item* it, int n, int parity, unsigned int* ctr,
                       cudaStream_t s) {
    switch (nw) {
    case 1: ch_rhs_kernel<T, 1><<<grid, BLK, 0, s>>>(g, it, n, parity, ctr); break;
    case 4: ch_rhs_kernel<T, 4><<<grid, 4 * BLK, 0, s>>>(g, it, n, parity, ctr); break;
    default: ch_rhs_kernel<T, 2><<<grid, 2 * BLK, 0, s>>>(g, it, n, parity, ctr); break;
    }
}

cudaError_t launch_ch_step(const ChConfig& c, bool rhs_fp32, const GridDev* grids, const Item* items_rhs, int n_rhs,
                           const Item* items_rows, int n_rows, int parity, unsigned int* counters, int sms,
                           cudaStream_t s) {
    // persistent grids over the work lists; CTAs beyond the resident ones find the lists empty
    const int g1 = std::max(1, std::min(n_rhs, sms * 32 / c.rhs_warps));
    const int g23 = std::max(1, std::min(n_rows, sms * 16));
    if (c.rhs_split) {
        const cudaError_t e2 =
            rhs_fp32 ? launch_rhs2<float>(c.rhs_warps, g1, grids, items_rhs, n_rhs, parity, counters, s,
                                          c.rhs_split == 2, sms)
                     : launch_rhs2<double>(c.rhs_warps, g1, grids, items_rhs, n_rhs, parity, counters, s,
                                           c.rhs_split == 2, sms);
        if (e2 != cudaSuccess) return e2;
    } else if (rhs_fp32) {
        launch_rhs<float>(c.rhs_warps, g1, grids, items_rhs, n_rhs, parity, counters, s);
    } else {
        launch_rhs<double>(c.rhs_warps, g1, grids, items_rhs, n_rhs, parity, counters, s);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (c.pipe) {
        // 64-100 registers and 8-17 KB of shared memory per one-warp CTA: up to 32 CTAs per SM
        const int gp = std::max(1, std::min(n_rows, sms * 32));
        if (c.ysplit) {   // x sweep, x correction, y recurrences, update (register-table sweeps, 8-row y batches)
            if (c.x_chunk == 8) ch_xsolve_pipe_rt_kernel<8><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
            else ch_xsolve_pipe_rt_kernel<16><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            ch_xcorr_kernel<<<n_rhs, 256, 0, s>>>(grids, items_rhs);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            ch_ysolve_split_kernel<8><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            ch_update_kernel<<<n_rhs, 256, 0, s>>>(grids, items_rhs, parity);
            return cudaGetLastError();
        }
        if (c.pipe >= 2 && c.x_chunk == 8)
            ch_xsolve_pipe_rt_kernel<8><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
        else if (c.pipe >= 2)
            ch_xsolve_pipe_rt_kernel<16><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
        else if (c.y_chunk == 32) ch_xsolve_pipe_kernel<32><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
        else ch_xsolve_pipe_kernel<16><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (c.pipe == 3 && c.y_chunk == 4)
            ch_ysolve_pipe_rt_kernel<4><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
        else if (c.pipe == 3 && c.y_chunk == 8)
            ch_ysolve_pipe_rt_kernel<8><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
        else if (c.pipe == 3)
            ch_ysolve_pipe_rt_kernel<16><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
        else if (c.y_chunk == 32)
            ch_ysolve_pipe_kernel<32><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
        else ch_ysolve_pipe_kernel<16><<<gp, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
        return cudaGetLastError();
    }
    ch_xsolve_kernel<<<g23, BLK, 0, s>>>(grids, items_rows, n_rows, counters + 1);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (c.y_chunk == 32) ch_ysolve_kernel<32><<<g23, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
    else ch_ysolve_kernel<16><<<g23, BLK, 0, s>>>(grids, items_rows, n_rows, parity, counters + 2);
    return cudaGetLastError();
}

// Compensated (Neumaier) sum of one grid, one CTA of 256 threads; combined with a two-sum tree.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& err) {
    s = a + b;
    const double bb = s - a;
    err = (a - (s - bb)) + (b - bb);
}

__global__ void __launch_bounds__(256) ch_mass_kernel(const double* __restrict__ f, long long count, double* out) {
    __shared__ double ss[256], sc[256];
    double s = 0.0, c = 0.0;
    for (long long k = threadIdx.x; k < count; k += blockDim.x) {
        double t, e;
        two_sum(s, f[k], t, e);
        s = t;
        c += e;
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            double t, e;
            two_sum(ss[threadIdx.x], ss[threadIdx.x + w], t, e);
            ss[threadIdx.x] = t;
            sc[threadIdx.x] += sc[threadIdx.x + w] + e;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = ss[0] + sc[0];
}

// ------------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------------

// Solver table for an n x n grid of side lx with D = 1, gamma, dt = dt_factor * dx (the reference
// defaults are gamma = 0.01, dt = 0.1 dx: cuPentCahnADI.cu:204-221), written into t (tab_size(n)
// doubles) with `work` (7 * (n - 2) doubles) as scratch.
static void fill_table(double* t, double* work, int n, double lx, double gamma, double dt_factor) {
    const int m = n - 2;
    const double D = 1.0, dx = lx / n, dt = dt_factor * dx;
    const double sl = 2.0 * dt * D * gamma / (3.0 * (dx * dx * dx * dx));
    const double a = sl, b = -4 * sl, c = 1 + 6 * sl, d = -4 * sl, e = sl;
    double *ds = work, *dl = work + m, *dg = work + 2 * m, *du = work + 3 * m, *dw = work + 4 * m;
    double *inv1 = work + 5 * m, *inv2 = work + 6 * m;
    for (int i = 0; i < m; ++i) {
        ds[i] = (i > 1) ? a : 0.0;
        dl[i] = (i > 0) ? b : 0.0;
        dg[i] = c;
        du[i] = (i < m - 1) ? d : 0.0;
        dw[i] = (i < m - 2) ? e : 0.0;
    }
    // in-place factorisation of the banded block (cuPentBatch.cu:35-113)
    du[0] = du[0] / dg[0];
    dw[0] = dw[0] / dg[0];
    dg[1] = dg[1] - dl[1] * du[0];
    du[1] = (du[1] - dl[1] * dw[0]) / dg[1];
    dw[1] = dw[1] / dg[1];
    for (int i = 2; i < m; ++i) {
        dl[i] = dl[i] - ds[i] * du[i - 2];
        dg[i] = dg[i] - ds[i] * dw[i - 2] - dl[i] * du[i - 1];
        if (i < m - 2) dw[i] = dw[i] / dg[i];
        if (i < m - 1) du[i] = (du[i] - dl[i] * dw[i - 1]) / dg[i];
    }
    auto solve = [&](double* x) {
        x[0] = x[0] / dg[0];
        x[1] = (x[1] - dl[1] * x[0]) / dg[1];
        for (int i = 2; i < m; ++i) x[i] = (x[i] - ds[i] * x[i - 2] - dl[i] * x[i - 1]) / dg[i];
        x[m - 2] = x[m - 2] - du[m - 2] * x[m - 1];
        for (int i = m - 3; i >= 0; --i) x[i] = x[i] - du[i] * x[i + 1] - dw[i] * x[i + 2];
    };
    // border columns and omega (BatchHyper.cu:421-514)
    for (int i = 0; i < m; ++i) inv1[i] = inv2[i] = 0.0;
    inv1[0] = a; inv1[m - 2] = e; inv1[m - 1] = d;
    inv2[0] = b; inv2[1] = a; inv2[m - 1] = e;
    solve(inv1);
    solve(inv2);
    const double z11 = e * inv1[0] + a * inv1[m - 2] + b * inv1[m - 1];
    const double z12 = e * inv2[0] + a * inv2[m - 2] + b * inv2[m - 1];
    const double z21 = d * inv1[0] + e * inv1[1] + a * inv1[m - 1];
    const double z22 = d * inv2[0] + e * inv2[1] + a * inv2[m - 1];
    const double y11 = c - z11, y12 = d - z12, y21 = b - z21, y22 = c - z22;
    const double det = 1.0 / (y11 * y22 - y21 * y12);
    for (int k = 0; k < tab_size(n); ++k) t[k] = 0.0;
    for (int i = 0; i < m; ++i) {
        t[i] = (i > 1) ? ds[i] : 0.0;
        t[m + i] = (i > 0) ? dl[i] : 0.0;
        t[2 * m + i] = 1.0 / dg[i];
        t[3 * m + i] = (i < m - 1) ? du[i] : 0.0;
        t[4 * m + i] = (i < m - 2) ? dw[i] : 0.0;
        t[5 * m + i] = inv1[i];
        t[6 * m + i] = inv2[i];
    }
    double* om = &t[7 * m];
    om[0] = y22 * det;
    om[1] = -y12 * det;
    om[2] = -y21 * det;
    om[3] = y11 * det;
    om[4] = a; om[5] = b; om[6] = d; om[7] = e;
    static const double wl[25] = {0, 0, -1, 0, 0, 0, -2, 8, -2, 0, -1, 8, -20, 8, -1, 0, -2, 8, -2, 0, 0, 0, -1, 0, 0};
    static const double wn[9] = {0, 1, 0, 1, -4, 1, 0, 1, 0};
    const double snl = (dt / 3.0) * D * (2.0 / (dx * dx));
    for (int k = 0; k < 25; ++k) t[7 * m + 8 + k] = wl[k] * sl;
    for (int k = 0; k < 9; ++k) t[7 * m + 33 + k] = wn[k] * snl;
}

std::vector<double> build_table(int n, double lx, double gamma, double dt_factor) {
    std::vector<double> t(tab_size(n)), work(7 * (n - 2));
    fill_table(t.data(), work.data(), n, lx, gamma, dt_factor);
    return t;
}

struct Batch {
    int device = 0;
    int rhs_fp32 = 0;
    int parity = 0;   // cCurr = buf[parity]
    long long steps_done = 0;
    std::vector<int> n;
    std::vector<double> lx;
    std::vector<GridDev> grids_h;
    std::vector<double*> allocs;
    std::vector<std::pair<std::string, double*>> tables;   // key "n/lx/gamma/dtf" -> device table
    GridDev* grids_d = nullptr;
    Item* items_rhs = nullptr;
    Item* items_rows = nullptr;   // K2 and K3 share the per-grid block lists (row / column blocks)
    int n_items_rhs = 0, n_items_rows = 0;
    unsigned int* counters = nullptr;   // 3 counters per step of a captured pair
    double* mass_d = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};   // pair of steps starting at parity 0 / 1
    int sms = 0;
    int cfg = -1;   // ch_config index; -1: kChBatchDefault
    unsigned long long launches = 0;
};

// The default: configuration 20, or with fewer 32-line warps than FP64 sub-partitions (4 per SM) its split
// y sweep (configuration 21), which a warp's FP64 instruction count bounds there (a 2048^2 grid alone: 1.32
// against 1.87 ms per step). Both compute the same values.
static ChConfig batch_config(const Batch* b) {
    if (b->cfg >= 0) return ch_config(b->cfg);
    return ch_config(b->n_items_rows < 4 * b->sms ? kChSplitConfig : kChBatchDefault);
}

static thread_local std::string g_ch_err;
static int ch_fail(cudaError_t e, const char* what) {
    g_ch_err = std::string("Error while '") + what + "': " + cudaGetErrorString(e);
    cudaGetLastError();
    return 1;
}
static int ch_fail_arg(const std::string& msg) {
    g_ch_err = msg;
    return 2;
}
#define CH_TRY(x, what)                             \
    do {                                            \
        cudaError_t _e = (x);                       \
        if (_e != cudaSuccess) return ch_fail(_e, what); \
    } while (0)

static int enqueue_step(Batch* b, int parity, int slot) {
    unsigned int* ctr = b->counters + kChCounters * slot;
    CH_TRY(cudaMemsetAsync(ctr, 0, kChCounters * sizeof(unsigned int), b->stream), "Resetting work counters");
    CH_TRY(launch_ch_step(batch_config(b), b->rhs_fp32 != 0, b->grids_d, b->items_rhs, b->n_items_rhs, b->items_rows,
                          b->n_items_rows, parity, ctr, b->sms, b->stream),
           "Launching a step");
    return 0;
}

static int capture_pairs(Batch* b) {
    for (int p = 0; p < 2; ++p) {
        if (b->graph_exec[p]) continue;
        cudaGraph_t g;
        CH_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "Beginning graph capture");
        int st = enqueue_step(b, p, 0);
        if (st == 0) st = enqueue_step(b, p ^ 1, 1);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (st != 0) return st;
        CH_TRY(e, "Ending graph capture");
        e = cudaGraphInstantiate(&b->graph_exec[p], g, 0);
        cudaGraphDestroy(g);
        CH_TRY(e, "Instantiating graph");
    }
    return 0;
}

// ------------------------------------------------------------------------------------------------
// Allocation-free single-grid step (custen_ch_step_noalloc)
// ------------------------------------------------------------------------------------------------
// Some callers cannot allocate device memory at all: a plug-in running inside a host application
// that owns every device allocation through its own budgeted pool, or a latency-critical loop that
// must never enter cudaMalloc / cudaFree (they synchronise the device). For them one step of one
// grid runs with all of its work buffers in this file-scope array: the right-hand side / x-sweep
// field, the row ends, the solver table, the descriptor, the work lists and the work counters.
// Maximum grid: kNoAllocMaxN x kNoAllocMaxN. Every GPU that loads the library holds the array
// (about 532 KiB) until the process exits.
constexpr int kNoAllocMaxN = 256;
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kNoAllocTmpOff = 0;
constexpr size_t kNoAllocEndsOff = align256(kNoAllocTmpOff + sizeof(double) * kNoAllocMaxN * kNoAllocMaxN);
constexpr size_t kNoAllocTabOff = align256(kNoAllocEndsOff + sizeof(double) * 2 * kNoAllocMaxN);
constexpr int kNoAllocTabLen = 7 * (kNoAllocMaxN - 2) + 42;
constexpr size_t kNoAllocGridOff = align256(kNoAllocTabOff + sizeof(double) * kNoAllocTabLen);
constexpr int kNoAllocBlocks = (kNoAllocMaxN / BLK) * (kNoAllocMaxN / BLK);
constexpr int kNoAllocRows = kNoAllocMaxN / BLK;
constexpr size_t kNoAllocRhsOff = align256(kNoAllocGridOff + sizeof(GridDev));
constexpr size_t kNoAllocRowsOff = align256(kNoAllocRhsOff + sizeof(Item) * kNoAllocBlocks);
constexpr size_t kNoAllocCtrOff = align256(kNoAllocRowsOff + sizeof(Item) * kNoAllocRows);
constexpr size_t kNoAllocBytes = align256(kNoAllocCtrOff + kChCounters * sizeof(unsigned int));

static __device__ __align__(256) unsigned char g_ch_noalloc_scratch[kNoAllocBytes];

// Device address of the array for each device, taken once with that device current. In host code the
// array's name is only a host-side stand-in, never a device address.
static std::atomic<unsigned char*> g_noalloc_base[64] = {};

}  // namespace ch
}  // namespace custen

using namespace custen::ch;

extern "C" {

const char* custen_ch_last_error(void) { return g_ch_err.c_str(); }

int custen_ch_batch_create(void** out, int nsims, const int* n, const double* lx, double gamma, double dt_factor,
                           int rhs_dtype, void* stream) {
    if (!out || nsims < 1 || !n) return ch_fail_arg("invalid arguments");
    for (int s = 0; s < nsims; ++s)
        if (n[s] < 64 || n[s] % BLK != 0) return ch_fail_arg("grid sizes must be multiples of 32, at least 64");
    Batch* b = new Batch();
    cudaGetDevice(&b->device);
    b->rhs_fp32 = rhs_dtype == CUSTEN_F32;
    if (stream) {
        b->stream = static_cast<cudaStream_t>(stream);
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete b; return ch_fail(e, "Creating stream"); }
        b->own_stream = true;
    }
    auto cleanup_fail = [&](int st) {
        for (double* p : b->allocs) cudaFree(p);
        for (auto& t : b->tables) cudaFree(t.second);
        if (b->own_stream) cudaStreamDestroy(b->stream);
        delete b;
        return st;
    };
    b->n.assign(n, n + nsims);
    b->lx.resize(nsims);
    for (int s = 0; s < nsims; ++s) b->lx[s] = lx ? lx[s] : 2.0 * M_PI;
    b->grids_h.resize(nsims);
    for (int s = 0; s < nsims; ++s) {
        const int ns = n[s];
        char key[128];
        snprintf(key, sizeof(key), "%d/%.17g/%.17g/%.17g", ns, b->lx[s], gamma, dt_factor);
        double* tab = nullptr;
        for (auto& t : b->tables)
            if (t.first == key) tab = t.second;
        if (!tab) {
            std::vector<double> h = build_table(ns, b->lx[s], gamma, dt_factor);
            cudaError_t e = cudaMalloc(&tab, h.size() * sizeof(double));
            if (e != cudaSuccess) return cleanup_fail(ch_fail(e, "Allocating solver table"));
            e = cudaMemcpy(tab, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cleanup_fail(ch_fail(e, "Uploading solver table"));
            b->tables.push_back({key, tab});
        }
        GridDev g{};
        const size_t bytes = (size_t)ns * ns * sizeof(double);
        for (int k = 0; k < 5; ++k) {   // cCurr / cOld, tmp, row ends, h of the two-pass right-hand side
            double* p = nullptr;
            cudaError_t e = cudaMalloc(&p, k == 3 ? 2 * ns * sizeof(double) : bytes);
            if (e != cudaSuccess) return cleanup_fail(ch_fail(e, "Allocating grid fields"));
            b->allocs.push_back(p);
            if (k < 2) g.buf[k] = p; else if (k == 2) g.tmp = p; else if (k == 3) g.ends = p; else g.hbuf = p;
        }
        g.tab = tab;
        g.n = ns;
        b->grids_h[s] = g;
    }
    // work lists, largest grids first
    std::vector<int> order(nsims);
    for (int s = 0; s < nsims; ++s) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
    std::vector<Item> rhs, rows;
    for (int s : order) {
        const int bpr = n[s] / BLK;
        for (int k = 0; k < bpr * bpr; ++k) rhs.push_back({s, k});
        for (int k = 0; k < bpr; ++k) rows.push_back({s, k});
    }
    b->n_items_rhs = (int)rhs.size();
    b->n_items_rows = (int)rows.size();
    cudaError_t e = cudaMalloc(&b->grids_d, nsims * sizeof(GridDev));
    if (e == cudaSuccess) e = cudaMemcpy(b->grids_d, b->grids_h.data(), nsims * sizeof(GridDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->items_rhs, rhs.size() * sizeof(Item));
    if (e == cudaSuccess) e = cudaMemcpy(b->items_rhs, rhs.data(), rhs.size() * sizeof(Item), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->items_rows, rows.size() * sizeof(Item));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->items_rows, rows.data(), rows.size() * sizeof(Item), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->counters, 2 * kChCounters * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&b->mass_d, sizeof(double));
    if (e != cudaSuccess) return cleanup_fail(ch_fail(e, "Allocating work lists"));
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    *out = b;
    return 0;
}

int custen_ch_batch_set_state(void* h, int sim, const double* c_cur, const double* c_old) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || sim < 0 || sim >= (int)b->n.size() || !c_cur) return ch_fail_arg("invalid arguments");
    const size_t bytes = (size_t)b->n[sim] * b->n[sim] * sizeof(double);
    GridDev& g = b->grids_h[sim];
    CH_TRY(cudaMemcpyAsync(g.buf[b->parity], c_cur, bytes, cudaMemcpyDefault, b->stream), "Uploading cCurr");
    CH_TRY(cudaMemcpyAsync(g.buf[b->parity ^ 1], c_old ? c_old : c_cur, bytes, cudaMemcpyDefault, b->stream),
           "Uploading cOld");
    CH_TRY(cudaStreamSynchronize(b->stream), "Synchronising upload");
    return 0;
}

int custen_ch_batch_get_state(void* h, int sim, double* c_cur, double* c_old) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || sim < 0 || sim >= (int)b->n.size()) return ch_fail_arg("invalid arguments");
    const size_t bytes = (size_t)b->n[sim] * b->n[sim] * sizeof(double);
    GridDev& g = b->grids_h[sim];
    if (c_cur) CH_TRY(cudaMemcpyAsync(c_cur, g.buf[b->parity], bytes, cudaMemcpyDefault, b->stream), "Reading cCurr");
    if (c_old)
        CH_TRY(cudaMemcpyAsync(c_old, g.buf[b->parity ^ 1], bytes, cudaMemcpyDefault, b->stream), "Reading cOld");
    CH_TRY(cudaStreamSynchronize(b->stream), "Synchronising read");
    return 0;
}

// Snapshot of one grid in the reference's HDF5 format (Print_Out, cuPentCahnADI.cu:103-140): dataset
// "c" = cCurr (n x n doubles), plus "c_old" = cOld and "t" = the time (1 x 1), which a resume needs
// and a reader of the reference's files ignores.
int custen_ch_batch_save(void* h, int sim, const char* path, double time) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || sim < 0 || sim >= (int)b->n.size() || !path) return ch_fail_arg("invalid arguments");
    const long long n = b->n[sim];
    std::vector<double> cur((size_t)(n * n)), old((size_t)(n * n));
    const int rc = custen_ch_batch_get_state(h, sim, cur.data(), old.data());
    if (rc) return rc;
    const char* names[3] = {"c", "c_old", "t"};
    const double* data[3] = {cur.data(), old.data(), &time};
    const long long dims[6] = {n, n, n, n, 1, 1};
    if (custen_h5_write(path, 3, names, data, dims)) return ch_fail_arg(std::string("Writing the snapshot: ") + custen_h5_last_error());
    return 0;
}

// Resume one grid from a snapshot: "c" (required, n x n) becomes cCurr; cOld is "c_old" when present,
// else cCurr too, as the reference starts from its initial condition (cuPentCahnADI.cu:295-305).
// *time receives "t", or NaN when the file has none (the reference's own snapshots).
int custen_ch_batch_load(void* h, int sim, const char* path, double* time) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || sim < 0 || sim >= (int)b->n.size() || !path) return ch_fail_arg("invalid arguments");
    const long long n = b->n[sim];
    long long dims[2] = {0, 0};
    if (custen_h5_read(path, "c", nullptr, 0, dims)) return ch_fail_arg(std::string("Reading the snapshot: ") + custen_h5_last_error());
    if (dims[0] != n || dims[1] != n)
        return ch_fail_arg("snapshot grid is " + std::to_string(dims[0]) + " x " + std::to_string(dims[1]) +
                           ", grid " + std::to_string(sim) + " is " + std::to_string(n) + " x " + std::to_string(n));
    std::vector<double> cur((size_t)(n * n)), old;
    if (custen_h5_read(path, "c", cur.data(), n * n, dims)) return ch_fail_arg(std::string("Reading the snapshot: ") + custen_h5_last_error());
    long long od[2] = {0, 0};
    if (custen_h5_read(path, "c_old", nullptr, 0, od) == 0) {
        if (od[0] != n || od[1] != n) return ch_fail_arg("snapshot c_old does not match c");
        old.resize((size_t)(n * n));
        if (custen_h5_read(path, "c_old", old.data(), n * n, od))
            return ch_fail_arg(std::string("Reading the snapshot: ") + custen_h5_last_error());
    }
    double t = std::nan("");
    long long td[2];
    if (custen_h5_read(path, "t", nullptr, 0, td) == 0 && td[0] * td[1] == 1) custen_h5_read(path, "t", &t, 1, td);
    if (time) *time = t;
    return custen_ch_batch_set_state(h, sim, cur.data(), old.empty() ? nullptr : old.data());
}

// Advance every grid by `steps` steps; asynchronous on the batch's stream (graph replays for pairs of
// steps, plain launches for an odd remainder) unless use_graph == 0.
int custen_ch_batch_step(void* h, int steps, int use_graph) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || steps < 0) return ch_fail_arg("invalid arguments");
    cudaSetDevice(b->device);
    int left = steps;
    const int per_step = ch_launches_per_step(batch_config(b));   // kernel launches in one step
    if (use_graph && left >= 2) {
        int st = capture_pairs(b);
        if (st) return st;
        while (left >= 2) {
            CH_TRY(cudaGraphLaunch(b->graph_exec[b->parity], b->stream), "Launching step graph");
            b->launches += 2 * per_step;
            left -= 2;
            b->steps_done += 2;
        }
    }
    while (left > 0) {
        int st = enqueue_step(b, b->parity, 0);
        if (st) return st;
        b->launches += per_step;
        b->parity ^= 1;
        --left;
        ++b->steps_done;
    }
    return 0;
}

int custen_ch_batch_synchronize(void* h) {
    Batch* b = static_cast<Batch*>(h);
    CH_TRY(cudaStreamSynchronize(b->stream), "Synchronising batch");
    return 0;
}

// Mean of a grid's cCurr with a compensated FP64 sum (device side).
int custen_ch_batch_mean(void* h, int sim, double* mean) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || sim < 0 || sim >= (int)b->n.size() || !mean) return ch_fail_arg("invalid arguments");
    const long long count = (long long)b->n[sim] * b->n[sim];
    ch_mass_kernel<<<1, 256, 0, b->stream>>>(b->grids_h[sim].buf[b->parity], count, b->mass_d);
    CH_TRY(cudaGetLastError(), "Launching mass sum");
    double s = 0.0;
    CH_TRY(cudaMemcpyAsync(&s, b->mass_d, sizeof(double), cudaMemcpyDeviceToHost, b->stream), "Reading mass");
    CH_TRY(cudaStreamSynchronize(b->stream), "Synchronising mass");
    *mean = s / (double)count;
    return 0;
}

unsigned long long custen_ch_batch_launches(void* h) { return static_cast<Batch*>(h)->launches; }

// One step of one n x n grid (n a multiple of 32, 64 <= n <= 256) without any device allocation.
// c_old, c_cur: the two previous fields; c_new receives the next one (it may be the c_old buffer,
// not the c_cur buffer). All three are device-accessible n*n double arrays. The first call on a
// device looks up the scratch array's device address (make it before any stream capture). Calls
// share the array: two calls that overlap on the GPU (different streams, no ordering) race.
int custen_ch_step_noalloc(const double* c_old, const double* c_cur, double* c_new, int n, double lx, double gamma,
                           double dt_factor, void* stream) {
    if (!c_old || !c_cur || !c_new) return ch_fail_arg("custen_ch_step_noalloc: NULL field pointer");
    if (n < 64 || n % BLK != 0) return ch_fail_arg("custen_ch_step_noalloc: n must be a multiple of 32, at least 64");
    if (n > kNoAllocMaxN) {
        char msg[160];
        snprintf(msg, sizeof(msg), "custen_ch_step_noalloc: n = %d exceeds the allocation-free maximum of %d", n,
                 kNoAllocMaxN);
        return ch_fail_arg(msg);
    }
    if (c_new == c_cur) return ch_fail_arg("custen_ch_step_noalloc: c_new must not be the c_cur buffer");
    int dev = 0;
    CH_TRY(cudaGetDevice(&dev), "Querying the current device");
    if (dev < 0 || dev >= 64) return ch_fail_arg("custen_ch_step_noalloc: device index out of range");
    unsigned char* base = g_noalloc_base[dev].load(std::memory_order_acquire);
    if (base == nullptr) {   // the same address whichever thread looks it up first
        void* p = nullptr;
        CH_TRY(cudaGetSymbolAddress(&p, g_ch_noalloc_scratch), "Looking up the scratch array's device address");
        base = static_cast<unsigned char*>(p);
        g_noalloc_base[dev].store(base, std::memory_order_release);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // host-side inputs in stack buffers (no heap either)
    double tab[kNoAllocTabLen];
    double work[7 * (kNoAllocMaxN - 2)];
    fill_table(tab, work, n, lx, gamma, dt_factor);
    GridDev g{};
    g.buf[0] = const_cast<double*>(c_cur);
    g.buf[1] = c_new;
    g.tmp = reinterpret_cast<double*>(base + kNoAllocTmpOff);
    g.ends = reinterpret_cast<double*>(base + kNoAllocEndsOff);
    g.tab = reinterpret_cast<const double*>(base + kNoAllocTabOff);
    g.n = n;
    const int bpr = n / BLK;
    Item rhs[kNoAllocBlocks], rows[kNoAllocRows];
    for (int k = 0; k < bpr * bpr; ++k) rhs[k] = Item{0, k};
    for (int k = 0; k < bpr; ++k) rows[k] = Item{0, k};

    const size_t bytes = (size_t)n * n * sizeof(double);
    // the update is written over the "old" buffer: start it from c_old
    if (c_new != c_old) CH_TRY(cudaMemcpyAsync(c_new, c_old, bytes, cudaMemcpyDefault, s), "Copying c_old");
    CH_TRY(cudaMemcpyAsync(base + kNoAllocTabOff, tab, sizeof(double) * tab_size(n), cudaMemcpyHostToDevice, s),
           "Uploading the solver table");
    CH_TRY(cudaMemcpyAsync(base + kNoAllocGridOff, &g, sizeof(g), cudaMemcpyHostToDevice, s),
           "Uploading the grid descriptor");
    CH_TRY(cudaMemcpyAsync(base + kNoAllocRhsOff, rhs, sizeof(Item) * bpr * bpr, cudaMemcpyHostToDevice, s),
           "Uploading the work list");
    CH_TRY(cudaMemcpyAsync(base + kNoAllocRowsOff, rows, sizeof(Item) * bpr, cudaMemcpyHostToDevice, s),
           "Uploading the work list");
    // the work counters must start at zero on every call (the array keeps the previous call's values)
    unsigned int* ctr = reinterpret_cast<unsigned int*>(base + kNoAllocCtrOff);
    CH_TRY(cudaMemsetAsync(ctr, 0, kChCounters * sizeof(unsigned int), s), "Clearing the work counters");
    const GridDev* gd = reinterpret_cast<const GridDev*>(base + kNoAllocGridOff);
    const Item* it_rhs = reinterpret_cast<const Item*>(base + kNoAllocRhsOff);
    const Item* it_rows = reinterpret_cast<const Item*>(base + kNoAllocRowsOff);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    CH_TRY(launch_ch_step(kChDefault, false, gd, it_rhs, bpr * bpr, it_rows, bpr, 0, ctr, sms, s), "Launching the step");
    return 0;
}

// Kernel configuration of a batch: time every configuration (ch_config) over `steps` steps of the
// batch itself, then restore the fields it started from, so tuning changes no result. Writes the
// chosen configuration's name to `name`. No reference counterpart.
int custen_ch_batch_autotune(void* h, int steps, char* name, size_t len) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || steps < 1) return ch_fail_arg("invalid arguments");
    CH_TRY(cudaSetDevice(b->device), "Setting device");
    size_t total = 0;
    for (const auto& g : b->grids_h) total += (size_t)g.n * g.n;
    double* save = nullptr;
    CH_TRY(cudaMalloc(&save, 2 * total * sizeof(double)), "Allocating the saved state");
    auto copy_state = [&](bool to_save) -> cudaError_t {
        size_t off = 0;
        for (const auto& g : b->grids_h) {
            const size_t bytes = (size_t)g.n * g.n * sizeof(double);
            for (int k = 0; k < 2; ++k) {
                double* dev = g.buf[k];
                double* sv = save + off;
                cudaError_t e = cudaMemcpyAsync(to_save ? sv : dev, to_save ? dev : sv, bytes,
                                                cudaMemcpyDeviceToDevice, b->stream);
                if (e != cudaSuccess) return e;
                off += (size_t)g.n * g.n;
            }
        }
        return cudaSuccess;
    };
    const int parity0 = b->parity;
    const long long done0 = b->steps_done;
    const unsigned long long launches0 = b->launches;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = copy_state(true);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    int best = -1;
    float best_ms = 0.f;
    for (int c = 0; c < kChConfigs && err == cudaSuccess; ++c) {
        b->cfg = c;
        for (int p = 0; p < 2; ++p)
            if (b->graph_exec[p]) {
                cudaGraphExecDestroy(b->graph_exec[p]);
                b->graph_exec[p] = nullptr;
            }
        if (custen_ch_batch_step(h, 2, 1) != 0) break;   // warm-up, graph capture
        cudaEventRecord(e0, b->stream);
        if (custen_ch_batch_step(h, steps, 1) != 0) break;
        cudaEventRecord(e1, b->stream);
        if ((err = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (best < 0 || ms < best_ms) {
            best = c;
            best_ms = ms;
        }
        if ((err = copy_state(false)) != cudaSuccess) break;
        b->parity = parity0;
        b->steps_done = done0;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (err == cudaSuccess) err = cudaStreamSynchronize(b->stream);
    cudaFree(save);
    b->parity = parity0;
    b->steps_done = done0;
    b->launches = launches0;
    for (int p = 0; p < 2; ++p)
        if (b->graph_exec[p]) {
            cudaGraphExecDestroy(b->graph_exec[p]);
            b->graph_exec[p] = nullptr;
        }
    if (err != cudaSuccess) return ch_fail(err, "Tuning the batch");
    if (best < 0) return 1;
    b->cfg = best;
    if (name && len) {
        const ChConfig c = ch_config(best);
        config_name(c, name, len);
    }
    return 0;
}

int custen_ch_batch_set_config(void* h, int index) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || index < -1 || index >= kChConfigs) return ch_fail_arg("invalid arguments");
    CH_TRY(cudaStreamSynchronize(b->stream), "Synchronising the batch");
    b->cfg = index;
    for (int p = 0; p < 2; ++p)
        if (b->graph_exec[p]) {
            cudaGraphExecDestroy(b->graph_exec[p]);
            b->graph_exec[p] = nullptr;
        }
    return 0;
}

int custen_ch_batch_config(void* h, char* name, size_t len) {
    Batch* b = static_cast<Batch*>(h);
    if (!b || !name || !len) return ch_fail_arg("invalid arguments");
    const ChConfig c = batch_config(b);
    config_name(c, name, len);
    return 0;
}

int custen_ch_batch_destroy(void* h) {
    Batch* b = static_cast<Batch*>(h);
    if (!b) return 0;
    cudaStreamSynchronize(b->stream);
    for (int p = 0; p < 2; ++p)
        if (b->graph_exec[p]) cudaGraphExecDestroy(b->graph_exec[p]);
    for (double* p : b->allocs) cudaFree(p);
    for (auto& t : b->tables) cudaFree(t.second);
    cudaFree(b->grids_d);
    cudaFree(b->items_rhs);
    cudaFree(b->items_rows);
    cudaFree(b->counters);
    cudaFree(b->mass_d);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return 0;
}

}  // extern "C"


