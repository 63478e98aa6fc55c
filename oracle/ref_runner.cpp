// Runs the reference cuSten kernels (compiled unchanged from the reference sources into
// oracle/_ref/custen_ref_sm103a.cubin) on the GPU -- TEST INFRASTRUCTURE ONLY.
//
// The host side restates the reference's cuStenCompute2D* tile loops (cuSten/src/kernels/
// 2d_*_kernel.cu, e.g. 2d_x_p_kernel.cu:193-273): one launch per tile, grid (nx/BLOCK_X,
// nyTile/BLOCK_Y), block (BLOCK_X, BLOCK_Y), dynamic shared memory = the handle's mem_shared as the
// reference's Create computes it, the per-tile halo pointers of Create (periodic formulas,
// custenCreateDestroy2DYp.cu:182-216) and the tileTop/tileBottom flags of the np Computes. One
// deliberate difference: cuStenCreate2DXpFun sizes its shared tile from uninitialised fields
// (custenCreateDestroy2DXpFun.cu:153-154); here it gets the layout its kernel indexes,
// nxLocal = BLOCK_X + L + R, nyLocal = BLOCK_Y.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <string>

namespace {

CUmodule g_mod = nullptr;
CUfunction g_kern[12] = {};
CUfunction g_weno = nullptr;   // kernel2DXYWENOADVp
const char* kNames[12] = {"kernel2DXp", "kernel2DXnp", "kernel2DXpFun", "kernel2DXnpFun",
                          "kernel2DYp", "kernel2DYnp", "kernel2DYpFun", "kernel2DYnpFun",
                          "kernel2DXYp", "kernel2DXYnp", "kernel2DXYpFun", "kernel2DXYnpFun"};
char g_err[512];

int fail(CUresult r, const char* what) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
    return 1;
}

// Unmangled name of an Itanium-mangled free function: _Z<len><name>...
std::string base_name(const char* m) {
    if (!m || m[0] != '_' || m[1] != 'Z') return m ? m : "";
    int i = 2, len = 0;
    while (m[i] >= '0' && m[i] <= '9') len = len * 10 + (m[i++] - '0');
    return std::string(m + i, len);
}

}  // namespace

extern "C" {

const char* refrun_error(void) { return g_err; }

int refrun_load(const char* cubin) {
    CUresult r = cuInit(0);
    if (r != CUDA_SUCCESS) return fail(r, "cuInit");
    CUdevice dev;
    if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return fail(r, "cuDeviceGet");
    CUcontext ctx;
    if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return fail(r, "cuDevicePrimaryCtxRetain");
    if ((r = cuCtxSetCurrent(ctx)) != CUDA_SUCCESS) return fail(r, "cuCtxSetCurrent");
    if (g_mod) return 0;
    if ((r = cuModuleLoad(&g_mod, cubin)) != CUDA_SUCCESS) return fail(r, "cuModuleLoad");
    unsigned int n = 0;
    if ((r = cuModuleGetFunctionCount(&n, g_mod)) != CUDA_SUCCESS) return fail(r, "cuModuleGetFunctionCount");
    CUfunction fs[256];
    if (n > 256) n = 256;
    if ((r = cuModuleEnumerateFunctions(fs, n, g_mod)) != CUDA_SUCCESS) return fail(r, "cuModuleEnumerateFunctions");
    for (unsigned i = 0; i < n; ++i) {
        const char* nm = nullptr;
        if (cuFuncGetName(&nm, fs[i]) != CUDA_SUCCESS) continue;
        std::string b = base_name(nm);
        for (int k = 0; k < 12; ++k)
            if (b == kNames[k]) g_kern[k] = fs[i];
        if (b == "kernel2DXYWENOADVp") g_weno = fs[i];
    }
    for (int k = 0; k < 12; ++k)
        if (!g_kern[k]) {
            snprintf(g_err, sizeof(g_err), "kernel %s not found in the reference cubin", kNames[k]);
            return 1;
        }
    return 0;
}

int refrun_fun_ptr(int id, unsigned long long* out) {
    char name[64];
    snprintf(name, sizeof(name), "custen_ref_fun%d", id);
    CUdeviceptr p;
    size_t bytes;
    CUresult r = cuModuleGetGlobal(&p, &bytes, g_mod, name);
    if (r != CUDA_SUCCESS) return fail(r, "cuModuleGetGlobal");
    if ((r = cuMemcpyDtoH(out, p, sizeof(*out))) != CUDA_SUCCESS) return fail(r, "cuMemcpyDtoH");
    return 0;
}

// One reference Compute of `variant` (device-resident data, offload DEVICE).
int refrun_compute(int variant, int nx, int ny, int numTiles, int BX, int BY, double* out, double* in,
                   double* halo_src, double* coef, int numSten, int H, int L, int R, int V, int T, int B, int numCoe,
                   unsigned long long func) {
    if (!g_mod) {
        snprintf(g_err, sizeof(g_err), "reference cubin not loaded");
        return 1;
    }
    const int nyTile = ny / numTiles;
    const int dir = variant < 4 ? 0 : (variant < 8 ? 1 : 2);
    int nxLocal, nyLocal;
    size_t smem;
    if (dir == 0) {
        nxLocal = BX + L + R;
        nyLocal = BY;
        int nc = (variant == 0 || variant == 1) ? numSten : numCoe;
        smem = ((size_t)nxLocal * nyLocal + nc) * sizeof(double);
    } else if (dir == 1) {
        nxLocal = BX;
        nyLocal = BY + T + B;
        int nc = (variant == 6) ? numCoe : numSten;
        smem = ((size_t)nxLocal * nyLocal + nc) * sizeof(double);
    } else {
        nxLocal = BX + L + R;
        nyLocal = BY + T + B;
        smem = ((size_t)nxLocal * nyLocal + (size_t)H * V) * sizeof(double);
    }
    CUfunction k = g_kern[variant];
    if (smem > 48 * 1024) {
        CUresult r = cuFuncSetAttribute(k, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
        if (r != CUDA_SUCCESS) return fail(r, "cuFuncSetAttribute");
    }
    const int numStenXY = H * V;
    for (int t = 0; t < numTiles; ++t) {
        double* o = out + (size_t)t * nyTile * nx;
        double* i = in + (size_t)t * nyTile * nx;
        double* btop = halo_src + (size_t)((t == 0) ? (ny - T) : (t * nyTile - T)) * nx;
        double* bbot = halo_src + (size_t)((t == numTiles - 1) ? 0 : (t + 1) * nyTile) * nx;
        int tileTop, tileBottom;
        if (numTiles == 1) { tileTop = 1; tileBottom = 1; }
        else if (t == 0) { tileTop = 1; tileBottom = 0; }
        else if (t == numTiles - 1) { tileTop = 0; tileBottom = 1; }
        else { tileTop = 0; tileBottom = 0; }
        void* fptr = reinterpret_cast<void*>(func);
        void* args[24];
        int n = 0;
        switch (variant) {
        case 0: case 1:   // (out, in, w, numSten, L, R, nxLocal, nyLocal, BX, nx)
            args[n++] = &o; args[n++] = &i; args[n++] = &coef; args[n++] = &numSten; args[n++] = &L;
            args[n++] = &R; args[n++] = &nxLocal; args[n++] = &nyLocal; args[n++] = &BX; args[n++] = &nx;
            break;
        case 2: case 3:   // (out, in, coe, func, L, R, numCoe, nxLocal, nyLocal, BX, nx)
            args[n++] = &o; args[n++] = &i; args[n++] = &coef; args[n++] = &fptr; args[n++] = &L; args[n++] = &R;
            args[n++] = &numCoe; args[n++] = &nxLocal; args[n++] = &nyLocal; args[n++] = &BX; args[n++] = &nx;
            break;
        case 4: case 5:   // (out, in, top, bot, w, numSten, T, B, nxLocal, nyLocal, BY, nx, nyTile[, tT, tB])
            args[n++] = &o; args[n++] = &i; args[n++] = &btop; args[n++] = &bbot; args[n++] = &coef;
            args[n++] = &numSten; args[n++] = &T; args[n++] = &B; args[n++] = &nxLocal; args[n++] = &nyLocal;
            args[n++] = &BY; args[n++] = &nx; args[n++] = (void*)&nyTile;
            if (variant == 5) { args[n++] = &tileTop; args[n++] = &tileBottom; }
            break;
        case 6:           // (out, in, top, bot, func, coe, numCoe, T, B, nxLocal, nyLocal, BY, nx, nyTile)
            args[n++] = &o; args[n++] = &i; args[n++] = &btop; args[n++] = &bbot; args[n++] = &fptr;
            args[n++] = &coef; args[n++] = &numCoe; args[n++] = &T; args[n++] = &B; args[n++] = &nxLocal;
            args[n++] = &nyLocal; args[n++] = &BY; args[n++] = &nx; args[n++] = (void*)&nyTile;
            break;
        case 7:           // (out, in, top, bot, coe, func, numSten, T, B, nxLocal, nyLocal, BY, nx, nyTile, tT, tB)
            args[n++] = &o; args[n++] = &i; args[n++] = &btop; args[n++] = &bbot; args[n++] = &coef;
            args[n++] = &fptr; args[n++] = &numSten; args[n++] = &T; args[n++] = &B; args[n++] = &nxLocal;
            args[n++] = &nyLocal; args[n++] = &BY; args[n++] = &nx; args[n++] = (void*)&nyTile;
            args[n++] = &tileTop; args[n++] = &tileBottom;
            break;
        default:          // XY: (out, in, top, bot, w|coe, [func,] numSten, H, L, R, V, T, B, nxLocal, nyLocal,
                          //      BX, BY, nx, nyTile[, tT, tB])
            args[n++] = &o; args[n++] = &i; args[n++] = &btop; args[n++] = &bbot; args[n++] = &coef;
            if (variant == 10 || variant == 11) args[n++] = &fptr;
            args[n++] = (void*)&numStenXY; args[n++] = &H; args[n++] = &L; args[n++] = &R; args[n++] = &V;
            args[n++] = &T; args[n++] = &B; args[n++] = &nxLocal; args[n++] = &nyLocal; args[n++] = &BX;
            args[n++] = &BY; args[n++] = &nx; args[n++] = (void*)&nyTile;
            if (variant == 9 || variant == 11) { args[n++] = &tileTop; args[n++] = &tileBottom; }
            break;
        }
        CUresult r = cuLaunchKernel(k, nx / BX, nyTile / BY, 1, BX, BY, 1, (unsigned)smem, nullptr, args, nullptr);
        if (r != CUDA_SUCCESS) return fail(r, "cuLaunchKernel");
    }
    CUresult r = cuCtxSynchronize();
    if (r != CUDA_SUCCESS) return fail(r, "cuCtxSynchronize");
    return 0;
}

// One reference Compute of the WENO advection operator (cuStenCompute2DXYWENOADVp,
// 2d_xyADVWENO_p_kernel.cu:440-548): per tile, grid (nx/BLOCK_X, nyTile/BLOCK_Y), shared memory
// (nxLocal*nyLocal + 49) doubles with nxLocal = BLOCK_X + 6, nyLocal = BLOCK_Y + 6
// (custenCreateDestroy2DXYADVWENOp.cu:149-156), the periodic halo pointers of its Create (:206-243).
int refrun_weno(int nx, int ny, int numTiles, int BX, int BY, double* out, double* in, double* u, double* v,
                double cdx, double cdy) {
    if (!g_mod || !g_weno) {
        snprintf(g_err, sizeof(g_err), "reference WENO kernel not loaded");
        return 1;
    }
    const int nyTile = ny / numTiles;
    int numSten = 49, H = 7, L = 3, R = 3, V = 7, T = 3, B = 3;
    int nxLocal = BX + 6, nyLocal = BY + 6;
    const size_t smem = ((size_t)nxLocal * nyLocal + 49) * sizeof(double);
    if (smem > 48 * 1024) {
        CUresult r = cuFuncSetAttribute(g_weno, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
        if (r != CUDA_SUCCESS) return fail(r, "cuFuncSetAttribute");
    }
    for (int t = 0; t < numTiles; ++t) {
        const size_t off = (size_t)t * nyTile * nx;
        double* o = out + off;
        double* i = in + off;
        double* uu = u + off;
        double* vv = v + off;
        double* btop = in + (size_t)((t == 0) ? (ny - T) : (t * nyTile - T)) * nx;
        double* bbot = in + (size_t)((t == numTiles - 1) ? 0 : (t + 1) * nyTile) * nx;
        void* args[] = {&o, &i, &uu, &vv, &btop, &bbot, &cdx, &cdy, &numSten, &H, &L, &R, &V, &T, &B,
                        &nxLocal, &nyLocal, &BX, &BY, &nx, (void*)&nyTile};
        CUresult r = cuLaunchKernel(g_weno, nx / BX, nyTile / BY, 1, BX, BY, 1, (unsigned)smem, nullptr, args, nullptr);
        if (r != CUDA_SUCCESS) return fail(r, "cuLaunchKernel");
    }
    CUresult r = cuCtxSynchronize();
    if (r != CUDA_SUCCESS) return fail(r, "cuCtxSynchronize");
    return 0;
}

}  // extern "C"
