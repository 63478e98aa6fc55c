// Runs the reference's Cahn-Hilliard GPU program (cuPentSpeedUp/cuPentCahnADITiming/src/cuPentCahnADI.cu)
// on the GPU -- TEST INFRASTRUCTURE ONLY: the baseline "one simulation at a time" loop of the reference,
// rebuilt for sm_103a, and a GPU cross-check of the library's solver.
//
// The device code is the reference's own, compiled unchanged into oracle/_ref/custen_ref_ch_sm103a.cubin
// (oracle/ref_ch_kernels.cu). The host side restates the program's set-up and time loop:
//   * managed allocations, setMultiLHS + pentFactorBatch, inv1Multi / inv2Multi rows (:213-407);
//     omega, inv1Single and inv2Single (BatchHyper.cu:421-514, host code) are passed in, computed by the
//     serial oracle's restatement of the same functions;
//   * the linear and non-linear right-hand sides as cuStenCompute2DXYp / cuStenCompute2DXYpFun do them
//     for one tile (cuSten/src/kernels/2d_xy_p_kernel.cu:542-657, 2d_xy_p_fun_kernel.cu:549-665): prefetch
//     the weights, synchronise the copy stream, prefetch the tile and its halo rows, record an event, wait
//     for it on the host, launch on the compute stream, rotate the three streams and the two events;
//   * one step of the time loop (:528-596): findCBar, sync, the two stencils, sync, findRHS, sync,
//     cublasDgeam transpose, sync, cyclicInv (pentSolveBatch, sync, solveEnd, sync, solveFull, sync),
//     transpose, sync, cyclicInv, sync, findNew, sync.
// Parameters as the program sets them: D = 1, gamma = 0.01, dt = 0.1 dx, blocks 32 x 32 (stencil RHS and
// element-wise kernels), 8 x 8 (non-linear RHS), 64 threads (solves).
#include <cublas_v2.h>
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

namespace {

char g_err[512];
CUmodule g_mod = nullptr;
enum { K_CBAR, K_RHS, K_NEW, K_XYP, K_XYPFUN, K_SETLHS, K_FACTOR, K_SOLVE, K_END, K_FULL, K_COUNT };
const char* kNames[K_COUNT] = {"findCBar", "findRHS", "findNew", "kernel2DXYp", "kernel2DXYpFun",
                               "setMultiLHS", "pentFactorBatch", "pentSolveBatch", "solveEnd", "solveFull"};
CUfunction g_k[K_COUNT] = {};
double* g_devfunc = nullptr;   // the program's devFunc (nonLinRHS) as a device address
cublasHandle_t g_blas = nullptr;

int fail_cu(CUresult r, const char* what) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
    return 1;
}
int fail_rt(cudaError_t e, const char* what) {
    snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
    return 1;
}
#define RT(x, what) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return fail_rt(e_, what); } while (0)
#define CU(x, what) do { CUresult r_ = (x); if (r_ != CUDA_SUCCESS) return fail_cu(r_, what); } while (0)

std::string base_name(const char* m) {
    if (!m || m[0] != '_' || m[1] != 'Z') return m ? m : "";
    int i = 2, len = 0;
    if (m[i] == 'L') ++i;
    while (m[i] >= '0' && m[i] <= '9') len = len * 10 + (m[i++] - '0');
    return std::string(m + i, len);
}

// One cuSten XY handle (numTiles = 1, periodic) as the program creates it.
struct Sten {
    CUfunction k;
    bool fun;
    double *out, *in, *top, *bot, *w, *func;
    int numSten, H, L, R, V, T, B, nxLocal, nyLocal, BX, BY, nx, nyTile;
    unsigned smem;
    cudaStream_t streams[3];
    cudaEvent_t ev[2];
};

int sten_init(Sten& s, bool fun, double* out, double* in, double* w, double* func, int n, int H, int L, int R, int V,
              int T, int B, int BX, int BY) {
    s.k = fun ? g_k[K_XYPFUN] : g_k[K_XYP];
    s.fun = fun;
    s.out = out; s.in = in; s.w = w; s.func = func;
    s.numSten = H * V; s.H = H; s.L = L; s.R = R; s.V = V; s.T = T; s.B = B;
    s.BX = BX; s.BY = BY; s.nx = n; s.nyTile = n;
    s.nxLocal = BX + L + R;
    s.nyLocal = BY + T + B;
    s.smem = (unsigned)(((size_t)s.nxLocal * s.nyLocal + s.numSten) * sizeof(double));
    // one tile: top halo = last T rows, bottom halo = first rows (custenCreateDestroy2DXYp.cu:196-200)
    s.top = in + (size_t)(n - T) * n;
    s.bot = in;
    for (int i = 0; i < 3; ++i) RT(cudaStreamCreate(&s.streams[i]), "cudaStreamCreate");
    for (int i = 0; i < 2; ++i) RT(cudaEventCreate(&s.ev[i]), "cudaEventCreate");
    if (s.smem > 48 * 1024) CU(cuFuncSetAttribute(s.k, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)s.smem),
                               "cuFuncSetAttribute");
    return 0;
}

void sten_free(Sten& s) {
    for (int i = 0; i < 3; ++i) cudaStreamDestroy(s.streams[i]);
    for (int i = 0; i < 2; ++i) cudaEventDestroy(s.ev[i]);
}

cudaError_t prefetch_dev(const void* p, size_t bytes, cudaStream_t st) {
    cudaMemLocation loc;
    loc.type = cudaMemLocationTypeDevice;
    loc.id = 0;
    return cudaMemPrefetchAsync(p, bytes, loc, 0, st);
}

int sten_compute(Sten& s) {
    const size_t tile = (size_t)s.nx * s.nyTile * sizeof(double);
    const size_t halo = (size_t)s.T * s.nx * sizeof(double);   // numBoundaryTop, used for both halos
    RT(prefetch_dev(s.w, s.numSten * sizeof(double), s.streams[1]), "prefetch weights");
    RT(cudaStreamSynchronize(s.streams[1]), "cudaStreamSynchronize");
    RT(prefetch_dev(s.in, tile, s.streams[1]), "prefetch input");
    RT(prefetch_dev(s.out, tile, s.streams[1]), "prefetch output");
    RT(prefetch_dev(s.top, halo, s.streams[1]), "prefetch top");
    RT(prefetch_dev(s.bot, halo, s.streams[1]), "prefetch bottom");
    RT(cudaEventRecord(s.ev[0], s.streams[1]), "cudaEventRecord");
    RT(cudaEventSynchronize(s.ev[0]), "cudaEventSynchronize");
    void* args[20];
    int n = 0;
    args[n++] = &s.out; args[n++] = &s.in; args[n++] = &s.top; args[n++] = &s.bot; args[n++] = &s.w;
    if (s.fun) args[n++] = &s.func;
    args[n++] = &s.numSten; args[n++] = &s.H; args[n++] = &s.L; args[n++] = &s.R; args[n++] = &s.V;
    args[n++] = &s.T; args[n++] = &s.B; args[n++] = &s.nxLocal; args[n++] = &s.nyLocal; args[n++] = &s.BX;
    args[n++] = &s.BY; args[n++] = &s.nx; args[n++] = &s.nyTile;
    CU(cuLaunchKernel(s.k, s.nx / s.BX, s.nyTile / s.BY, 1, s.BX, s.BY, 1, s.smem, (CUstream)s.streams[0], args,
                      nullptr),
       "cuLaunchKernel stencil");
    cudaStream_t ts = s.streams[0];
    s.streams[0] = s.streams[1]; s.streams[1] = s.streams[2]; s.streams[2] = ts;
    cudaEvent_t te = s.ev[0]; s.ev[0] = s.ev[1]; s.ev[1] = te;
    return 0;
}

struct State {
    int n, size;
    double a, b, c, d, e;
    double omega[4];
    double *cOld, *cCurr, *cNonLinRHS, *cBar, *cHalf;
    double *ds, *dl, *diag, *du, *dw, *inv1Multi, *inv2Multi, *wLin, *coe;
    Sten lin, nonlin;
};

int launch(int k, unsigned gx, unsigned gy, unsigned bx, unsigned by, void** args) {
    CU(cuLaunchKernel(g_k[k], gx, gy, 1, bx, by, 1, 0, nullptr, args, nullptr), kNames[k]);
    return 0;
}

int sync(const char* what) {
    RT(cudaDeviceSynchronize(), what);
    return 0;
}

// cyclicInv (BatchHyper.cu:520-590)
int cyclic_inv(State& s, double* data) {
    const int n = s.n;
    const unsigned ginv = (unsigned)((n + 63) / 64), g32 = (unsigned)((n + 31) / 32);
    int size = s.size, nn = n;
    void* a1[] = {&s.ds, &s.dl, &s.diag, &s.du, &s.dw, &data, &size, &nn};
    if (launch(K_SOLVE, ginv, 1, 64, 1, a1)) return 1;
    if (sync("pentSolveBatch")) return 1;
    void* a2[] = {&data, &s.a, &s.b, &s.d, &s.e, &s.omega[0], &s.omega[1], &s.omega[2], &s.omega[3], &nn, &nn};
    if (launch(K_END, ginv, 1, 64, 1, a2)) return 1;
    if (sync("solveEnd")) return 1;
    void* a3[] = {&data, &s.inv1Multi, &s.inv2Multi, &nn, &nn};
    if (launch(K_FULL, g32, g32, 32, 32, a3)) return 1;
    return sync("solveFull");
}

int transpose(State& s, const double* src, double* dst) {
    const double alpha = 1.0, beta = 0.0;
    cublasStatus_t st = cublasDgeam(g_blas, CUBLAS_OP_T, CUBLAS_OP_T, s.n, s.n, &alpha, src, s.n, &beta, nullptr, s.n,
                                    dst, s.n);
    if (st != CUBLAS_STATUS_SUCCESS) {
        snprintf(g_err, sizeof(g_err), "cublasDgeam failed (%d)", (int)st);
        return 1;
    }
    return sync("transpose");
}

}  // namespace

extern "C" {

const char* refch_error(void) { return g_err; }

int refch_load(const char* cubin) {
    if (g_mod) return 0;
    RT(cudaSetDevice(0), "cudaSetDevice");
    RT(cudaFree(nullptr), "runtime init");
    CUcontext ctx;
    CU(cuCtxGetCurrent(&ctx), "cuCtxGetCurrent");
    CU(cuModuleLoad(&g_mod, cubin), "cuModuleLoad");
    unsigned int cnt = 0;
    CU(cuModuleGetFunctionCount(&cnt, g_mod), "cuModuleGetFunctionCount");
    CUfunction fs[512];
    if (cnt > 512) cnt = 512;
    CU(cuModuleEnumerateFunctions(fs, cnt, g_mod), "cuModuleEnumerateFunctions");
    for (unsigned i = 0; i < cnt; ++i) {
        const char* nm = nullptr;
        if (cuFuncGetName(&nm, fs[i]) != CUDA_SUCCESS) continue;
        const std::string b = base_name(nm);
        for (int k = 0; k < K_COUNT; ++k)
            if (b == kNames[k]) g_k[k] = fs[i];
    }
    for (int k = 0; k < K_COUNT; ++k)
        if (!g_k[k]) {
            snprintf(g_err, sizeof(g_err), "kernel %s not found in the reference cubin", kNames[k]);
            return 1;
        }
    CUdeviceptr p;
    size_t bytes;
    CU(cuModuleGetGlobal(&p, &bytes, g_mod, "devFunc"), "cuModuleGetGlobal devFunc");
    CU(cuMemcpyDtoH(&g_devfunc, p, sizeof(g_devfunc)), "reading devFunc");
    if (cublasCreate(&g_blas) != CUBLAS_STATUS_SUCCESS) {
        snprintf(g_err, sizeof(g_err), "cublasCreate failed");
        return 1;
    }
    return 0;
}

// n: grid size (multiple of 64), lx: domain length, c0: n x n initial field (cOld = cCurr = c0),
// omega4 / inv1 / inv2: findOmega's outputs for this n (length 4, n-2, n-2).
int refch_create(void** out, int n, double lx, const double* c0, const double* omega4, const double* inv1,
                 const double* inv2) {
    if (!g_mod) {
        snprintf(g_err, sizeof(g_err), "reference CH cubin not loaded");
        return 1;
    }
    if (n < 64 || n % 64 != 0) {
        snprintf(g_err, sizeof(g_err), "n must be a multiple of 64 (the program's 64-thread solves)");
        return 1;
    }
    State* s = new State();
    s->n = n;
    s->size = n - 2;
    const double D = 1.0, gamma = 0.01, dx = lx / n, dt = 0.1 * dx;
    const double sigmaLin = 2.0 * dt * D * gamma / (3.0 * (std::pow(dx, 4.0)));   // :373
    s->a = sigmaLin; s->b = -4 * sigmaLin; s->c = 1 + 6 * sigmaLin; s->d = -4 * sigmaLin; s->e = sigmaLin;
    memcpy(s->omega, omega4, sizeof(s->omega));
    const size_t nn = (size_t)n * n;
    double** fields[] = {&s->cOld, &s->cCurr, &s->cNonLinRHS, &s->cBar, &s->cHalf};
    for (double** f : fields) RT(cudaMallocManaged(f, nn * sizeof(double)), "cudaMallocManaged field");
    for (size_t i = 0; i < nn; ++i) {
        s->cOld[i] = c0[i];
        s->cCurr[i] = c0[i];
    }
    double** diags[] = {&s->ds, &s->dl, &s->diag, &s->du, &s->dw};
    for (double** f : diags) RT(cudaMallocManaged(f, (size_t)s->size * n * sizeof(double)), "cudaMallocManaged diag");
    const unsigned g32 = (unsigned)(n / 32), ginv = (unsigned)(n / 64);
    int size = s->size, nx = n;
    void* al[] = {&s->ds, &s->dl, &s->diag, &s->du, &s->dw, &s->a, &s->b, &s->c, &s->d, &s->e, &size, &nx};
    if (launch(K_SETLHS, g32, g32, 32, 32, al) || sync("setMultiLHS")) return 1;
    void* af[] = {&s->ds, &s->dl, &s->diag, &s->du, &s->dw, &size, &nx};
    if (launch(K_FACTOR, ginv, 1, 64, 1, af) || sync("pentFactorBatch")) return 1;
    RT(cudaMallocManaged(&s->inv1Multi, (size_t)n * s->size * sizeof(double)), "cudaMallocManaged inv1");
    RT(cudaMallocManaged(&s->inv2Multi, (size_t)n * s->size * sizeof(double)), "cudaMallocManaged inv2");
    for (int j = 0; j < s->size; ++j)
        for (int i = 0; i < n; ++i) {
            s->inv1Multi[(size_t)j * n + i] = inv1[j];
            s->inv2Multi[(size_t)j * n + i] = inv2[j];
        }
    // weightsLinRHS (:463-467) and the non-linear coefficients (:509-513)
    RT(cudaMallocManaged(&s->wLin, 25 * sizeof(double)), "cudaMallocManaged weights");
    static const double pat[25] = {0, 0, -1, 0, 0, 0, -2, 8, -2, 0, -1, 8, -20, 8, -1, 0, -2, 8, -2, 0, 0, 0, -1, 0, 0};
    for (int k = 0; k < 25; ++k) s->wLin[k] = pat[k] == 0 ? 0.0 : pat[k] * sigmaLin;
    RT(cudaMallocManaged(&s->coe, 9 * sizeof(double)), "cudaMallocManaged coe");
    const double sigmaNonLin = (dt / 3.0) * D * (2.0 / std::pow(dx, 2.0));   // :496
    static const double npat[9] = {0, 1, 0, 1, -4, 1, 0, 1, 0};
    for (int k = 0; k < 9; ++k) s->coe[k] = npat[k] == 0 ? 0.0 : npat[k] * sigmaNonLin;
    if (sten_init(s->lin, false, s->cHalf, s->cBar, s->wLin, nullptr, n, 5, 2, 2, 5, 2, 2, 32, 32)) return 1;
    if (sten_init(s->nonlin, true, s->cNonLinRHS, s->cCurr, s->coe, g_devfunc, n, 3, 1, 1, 3, 1, 1, 8, 8)) return 1;
    if (sync("create")) return 1;
    *out = s;
    return 0;
}

int refch_step(void* st, int steps) {
    State& s = *static_cast<State*>(st);
    const unsigned g32 = (unsigned)(s.n / 32);
    int nx = s.n;
    for (int it = 0; it < steps; ++it) {
        void* a0[] = {&s.cOld, &s.cCurr, &s.cBar, &nx};
        if (launch(K_CBAR, g32, g32, 32, 32, a0) || sync("findCBar")) return 1;
        if (sten_compute(s.nonlin) || sten_compute(s.lin) || sync("stencils")) return 1;
        void* a1[] = {&s.cOld, &s.cCurr, &s.cHalf, &s.cNonLinRHS, &nx};
        if (launch(K_RHS, g32, g32, 32, 32, a1) || sync("findRHS")) return 1;
        if (transpose(s, s.cHalf, s.cCurr)) return 1;
        if (cyclic_inv(s, s.cCurr)) return 1;
        if (transpose(s, s.cCurr, s.cHalf)) return 1;
        if (cyclic_inv(s, s.cHalf)) return 1;
        if (sync("solves")) return 1;
        void* a2[] = {&s.cCurr, &s.cBar, &s.cHalf, &nx};
        if (launch(K_NEW, g32, g32, 32, 32, a2) || sync("findNew")) return 1;
    }
    return 0;
}

int refch_get(void* st, double* c_curr, double* c_old) {
    State& s = *static_cast<State*>(st);
    if (sync("get")) return 1;
    const size_t bytes = (size_t)s.n * s.n * sizeof(double);
    if (c_curr) memcpy(c_curr, s.cCurr, bytes);
    if (c_old) memcpy(c_old, s.cOld, bytes);
    return 0;
}

// The reference's batched pentadiagonal kernels on caller buffers (device pointers), launched as the
// program launches them: 64-thread blocks over the systems (cuPentCahnADI.cu:357, BatchHyper.cu:565).
int refch_pent_factor(double* ds, double* dl, double* d, double* du, double* dw, int m, int batch) {
    if (!g_mod) {
        snprintf(g_err, sizeof(g_err), "reference CH cubin not loaded");
        return 1;
    }
    void* a[] = {&ds, &dl, &d, &du, &dw, &m, &batch};
    if (launch(K_FACTOR, (unsigned)((batch + 63) / 64), 1, 64, 1, a)) return 1;
    return sync("pentFactorBatch");
}

int refch_pent_solve(double* ds, double* dl, double* d, double* du, double* dw, double* b, int m, int batch) {
    if (!g_mod) {
        snprintf(g_err, sizeof(g_err), "reference CH cubin not loaded");
        return 1;
    }
    void* a[] = {&ds, &dl, &d, &du, &dw, &b, &m, &batch};
    if (launch(K_SOLVE, (unsigned)((batch + 63) / 64), 1, 64, 1, a)) return 1;
    return sync("pentSolveBatch");
}

int refch_destroy(void* st) {
    State* s = static_cast<State*>(st);
    if (!s) return 0;
    sten_free(s->lin);
    sten_free(s->nonlin);
    double* ptrs[] = {s->cOld, s->cCurr, s->cNonLinRHS, s->cBar, s->cHalf, s->ds, s->dl, s->diag, s->du, s->dw,
                      s->inv1Multi, s->inv2Multi, s->wLin, s->coe};
    for (double* p : ptrs) cudaFree(p);
    delete s;
    return 0;
}

}  // extern "C"
