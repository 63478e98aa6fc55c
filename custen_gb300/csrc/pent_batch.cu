// Batched pentadiagonal factorisation and solve over the interleaved layout of cuPentBatch
// (cuPentCahnADI/src/cuPentBatch.cu): element (row i, system s) of every diagonal and of the
// right-hand side lives at [i * batch + s]; ds / dl are the diagonals two and one below the main one
// (ds[0], ds[1], dl[0] zero), du / dw one and two above (du[m-1], dw[m-2], dw[m-1] zero).
//
// pent_factor: in place, the reference's pentFactorBatch (:35-113) -- the same expressions in the same
// order, so every factor is bit-identical to the reference kernel's on the same GPU.
// pent_solve: the reference's pentSolveBatch (:119-198), bit-identical as well.
// pent_invert_pivots / pent_solve_rcp: the fast variant this library's ADI solver uses -- pivots
// inverted once, the solve multiplies instead of dividing (rounding differs from the reference by about
// one unit in the last place per row).
//
// GB300 shape: one thread per system, coalesced across systems (the layout's purpose). The per-row
// recurrence is a dependent chain, so each thread issues the loads of the next KR rows before the chain
// consumes them, and keeps the rows the chain refers back to in registers instead of re-reading them.
// With divisions (about 10 FP64 operations each) the exact variants are FP64-bound; the reciprocal
// variant is bound by HBM.
#include <cuda_runtime.h>

#include <atomic>

#include <algorithm>
#include <cstdio>
#include <string>

#include "../../include/custen_gb300.h"

namespace custen {
namespace pent {
namespace {

constexpr int kThreads = 128;

// KR: rows whose loads are issued ahead of the dependent chain.
template <int KR>
__global__ void __launch_bounds__(kThreads) factor_kernel(double* __restrict__ ds, double* __restrict__ dl,
                                                          double* __restrict__ d, double* __restrict__ du,
                                                          double* __restrict__ dw, int m, int batch) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= batch) return;
    const size_t B = (size_t)batch;
    // row 0
    double d0 = d[s];
    double du0 = du[s] / d0;
    double dw0 = dw[s] / d0;
    du[s] = du0;
    dw[s] = dw0;
    // row 1
    size_t r = B + s;
    const double dl1 = dl[r];
    double d1 = d[r] - dl1 * du0;
    double du1 = (du[r] - dl1 * dw0) / d1;
    double dw1 = dw[r] / d1;
    d[r] = d1;
    du[r] = du1;
    dw[r] = dw1;
    // interior rows 2 .. m-3 (cuPentBatch.cu:75-80); (du, dw) of the two previous rows stay in registers
    // (duP2, dwP2 = row i-2; duP1, dwP1 = row i-1)
    double duP2 = du0, dwP2 = dw0, duP1 = du1, dwP1 = dw1;
    for (int i0 = 2; i0 < m - 2; i0 += KR) {
        double vs[KR], vl[KR], vd[KR], vu[KR], vw[KR];
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int i = i0 + k;
            if (i < m - 2) {
                const size_t q = (size_t)i * B + s;
                vs[k] = ds[q];
                vl[k] = dl[q];
                vd[k] = d[q];
                vu[k] = du[q];
                vw[k] = dw[q];
            }
        }
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int i = i0 + k;
            if (i >= m - 2) break;
            const size_t q = (size_t)i * B + s;
            const double l = vl[k] - vs[k] * duP2;
            const double dd = vd[k] - vs[k] * dwP2 - l * duP1;
            const double ww = vw[k] / dd;
            const double uu = (vu[k] - l * dwP1) / dd;
            dl[q] = l;
            d[q] = dd;
            dw[q] = ww;
            du[q] = uu;
            duP2 = duP1;
            dwP2 = dwP1;
            duP1 = uu;
            dwP1 = ww;
        }
    }
    // second last row (:86-92): no dw
    {
        const size_t q = (size_t)(m - 2) * B + s;
        const double l = dl[q] - ds[q] * duP2;
        const double dd = d[q] - ds[q] * dwP2 - l * duP1;
        const double uu = (du[q] - l * dwP1) / dd;
        dl[q] = l;
        d[q] = dd;
        du[q] = uu;
        duP2 = duP1;
        dwP2 = dwP1;
        duP1 = uu;
    }
    // last row (:94-99): dl and d only
    {
        const size_t q = (size_t)(m - 1) * B + s;
        const double l = dl[q] - ds[q] * duP2;
        dl[q] = l;
        d[q] = d[q] - ds[q] * dwP2 - l * duP1;
    }
}

template <int KR>
__global__ void __launch_bounds__(kThreads) solve_kernel(const double* __restrict__ ds, const double* __restrict__ dl,
                                                         const double* __restrict__ d, const double* __restrict__ du,
                                                         const double* __restrict__ dw, double* __restrict__ b, int m,
                                                         int batch, int rcp) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= batch) return;
    const size_t B = (size_t)batch;
    // forward substitution (cuPentBatch.cu:153-171)
    double b0 = rcp ? b[s] * d[s] : b[s] / d[s];
    b[s] = b0;
    double b1 = rcp ? (b[B + s] - dl[B + s] * b0) * d[B + s] : (b[B + s] - dl[B + s] * b0) / d[B + s];
    b[B + s] = b1;
    double p2 = b0, p1 = b1;
    for (int i0 = 2; i0 < m; i0 += KR) {
        double vs[KR], vl[KR], vd[KR], vb[KR];
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int i = i0 + k;
            if (i < m) {
                const size_t q = (size_t)i * B + s;
                vs[k] = ds[q];
                vl[k] = dl[q];
                vd[k] = d[q];
                vb[k] = b[q];
            }
        }
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int i = i0 + k;
            if (i >= m) break;
            const double t = vb[k] - vs[k] * p2 - vl[k] * p1;
            const double v = rcp ? t * vd[k] : t / vd[k];
            b[(size_t)i * B + s] = v;
            p2 = p1;
            p1 = v;
        }
    }
    // backward substitution (:178-196); rows m-1 and m-2 first
    double a1 = p1;                                   // row m-1
    double a0 = b[(size_t)(m - 2) * B + s] - du[(size_t)(m - 2) * B + s] * a1;   // row m-2
    b[(size_t)(m - 2) * B + s] = a0;
    // a0 = row i+1, a1 = row i+2
    double n1 = a0, n2 = a1;
    for (int i0 = m - 3; i0 >= 0; i0 -= KR) {
        double vu[KR], vw[KR], vb[KR];
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int i = i0 - k;
            if (i >= 0) {
                const size_t q = (size_t)i * B + s;
                vu[k] = du[q];
                vw[k] = dw[q];
                vb[k] = b[q];
            }
        }
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            const int i = i0 - k;
            if (i < 0) break;
            const double v = vb[k] - vu[k] * n1 - vw[k] * n2;
            b[(size_t)i * B + s] = v;
            n2 = n1;
            n1 = v;
        }
    }
}

__global__ void __launch_bounds__(kThreads) invert_kernel(double* __restrict__ d, size_t count) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < count; q += (size_t)gridDim.x * blockDim.x)
        d[q] = 1.0 / d[q];
}

thread_local std::string g_err;
std::atomic<int> g_kr[3] = {8, 2, 2};   // prefetch depth: factor, exact solve, inverted-pivot solve (measured best)

template <typename F2, typename F4, typename F8>
void by_depth(int kr, F2 f2, F4 f4, F8 f8) {
    if (kr <= 2) f2();
    else if (kr <= 4) f4();
    else f8();
}

int check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    g_err = std::string("Error while '") + what + "': " + cudaGetErrorString(e);
    cudaGetLastError();
    return 1;
}

int check_args(const void* a, const void* b, const void* c, const void* dd, const void* e, int m, int batch) {
    if (!a || !b || !c || !dd || !e) {
        g_err = "diagonal pointers must not be NULL";
        return 2;
    }
    if (m < 4 || batch < 1) {
        g_err = "need m >= 4 unknowns and batch >= 1 systems";
        return 2;
    }
    return 0;
}

}  // namespace
}  // namespace pent
}  // namespace custen

using namespace custen::pent;

extern "C" {

const char* custen_pent_last_error(void) { return g_err.c_str(); }

// Prefetch depth (rows of loads issued ahead of the chain: 2, 4 or 8) of the factorisation (which = 0),
// the exact solve (1) and the inverted-pivot solve (2). Results do not depend on it.
int custen_pent_set_depth(int which, int rows) {
    if (which < 0 || which > 2 || (rows != 2 && rows != 4 && rows != 8)) {
        g_err = "invalid prefetch depth";
        return 2;
    }
    g_kr[which] = rows;
    return 0;
}

int custen_pent_factor_batch(double* ds, double* dl, double* d, double* du, double* dw, int m, int batch,
                             void* stream) {
    if (int st = check_args(ds, dl, d, du, dw, m, batch)) return st;
    const int blocks = (batch + kThreads - 1) / kThreads;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    by_depth(
        g_kr[0], [&] { factor_kernel<2><<<blocks, kThreads, 0, st>>>(ds, dl, d, du, dw, m, batch); },
        [&] { factor_kernel<4><<<blocks, kThreads, 0, st>>>(ds, dl, d, du, dw, m, batch); },
        [&] { factor_kernel<8><<<blocks, kThreads, 0, st>>>(ds, dl, d, du, dw, m, batch); });
    return check(cudaGetLastError(), "Launching the batched factorisation");
}

int custen_pent_solve_batch(const double* ds, const double* dl, const double* d, const double* du, const double* dw,
                            double* b, int m, int batch, void* stream) {
    if (int st = check_args(ds, dl, d, du, dw, m, batch)) return st;
    if (!b) {
        g_err = "right-hand side pointer must not be NULL";
        return 2;
    }
    const int blocks = (batch + kThreads - 1) / kThreads;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    by_depth(
        g_kr[1], [&] { solve_kernel<2><<<blocks, kThreads, 0, st>>>(ds, dl, d, du, dw, b, m, batch, 0); },
        [&] { solve_kernel<4><<<blocks, kThreads, 0, st>>>(ds, dl, d, du, dw, b, m, batch, 0); },
        [&] { solve_kernel<8><<<blocks, kThreads, 0, st>>>(ds, dl, d, du, dw, b, m, batch, 0); });
    return check(cudaGetLastError(), "Launching the batched solve");
}

int custen_pent_invert_pivots(double* d, int m, int batch, void* stream) {
    if (!d || m < 4 || batch < 1) {
        g_err = "invalid arguments";
        return 2;
    }
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    invert_kernel<<<sms * 8, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(d, (size_t)m * batch);
    return check(cudaGetLastError(), "Inverting the pivots");
}

int custen_pent_solve_batch_rcp(const double* ds, const double* dl, const double* rd, const double* du,
                                const double* dw, double* b, int m, int batch, void* stream) {
    if (int st = check_args(ds, dl, rd, du, dw, m, batch)) return st;
    if (!b) {
        g_err = "right-hand side pointer must not be NULL";
        return 2;
    }
    const int blocks = (batch + kThreads - 1) / kThreads;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    by_depth(
        g_kr[2], [&] { solve_kernel<2><<<blocks, kThreads, 0, st>>>(ds, dl, rd, du, dw, b, m, batch, 1); },
        [&] { solve_kernel<4><<<blocks, kThreads, 0, st>>>(ds, dl, rd, du, dw, b, m, batch, 1); },
        [&] { solve_kernel<8><<<blocks, kThreads, 0, st>>>(ds, dl, rd, du, dw, b, m, batch, 1); });
    return check(cudaGetLastError(), "Launching the batched solve");
}

}  // extern "C"
