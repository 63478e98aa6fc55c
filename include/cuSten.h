/*
 * cuSten.h -- drop-in public header of the GB300 (sm_103a) rebuild of the cuSten 2D stencil library.
 *
 * This header keeps the reference library's C++ API exactly: the same `cuSten_t` handle layout
 * (200 bytes on LP64, field order unchanged), the same function names and argument lists, C++
 * linkage (no extern "C"), so that code written against the reference `cuSten.h` and linked
 * against the reference `libcuSten.a` compiles and links unchanged against this library.
 *
 * Reference interfaces replaced (paths inside the cuSten project):
 *   cuSten/cuSten.h:27-43                                  umbrella header, DEVICE/HOST macros
 *   cuSten/src/struct/cuSten_struct_type.h:84-122           cuSten_t
 *   cuSten/src/struct/cuSten_struct_functions.h:67-838      cuStenCreate* / cuStenSwap* / cuStenDestroy*
 *   cuSten/src/kernels/stencil_kernels.h:52-189             cuStenCompute*
 *   cuSten/src/util/util.h:43                               checkError
 *
 * Semantics kept from the reference:
 *   - Create stores the caller's pointers (data, weights/coefficients, function pointer); it never
 *     copies or owns user data. Weights are re-read from memory on every Compute.
 *   - Compute is asynchronous at return; callers synchronise (cudaDeviceSynchronize) before reading.
 *   - Swap exchanges per-tile input/output pointers; the Y and XY variants recompute the per-tile
 *     halo pointers from the pointer passed to Swap.
 *   - Errors print "Error while '<action>': <cuda error string>" and exit(EXIT_FAILURE).
 * Extensions (documented, do not change existing behaviour):
 *   - data may be managed memory (prefetched per tile as in the reference) or plain device memory
 *     (the reference exits on the failing prefetch; this library skips the prefetch).
 *   - cuStenCompute2DXpFun is defined as well as the reference's misspelt cuSenCompute2DXpFun.
 */
#ifndef CUSTEN_H
#define CUSTEN_H

#include <cuda_runtime.h>

#define DEVICE 0
#define HOST 1

/* Handle. Field order and types are those of cuSten/src/struct/cuSten_struct_type.h:84-122. The
 * rebuild keeps its private state behind the `streams` allocation, so the struct never grows. */
typedef struct
{
    int deviceNum;
    int numStreams;
    int numTiles;
    int nx;
    int ny;
    int nyTile;
    int numSten;
    int numStenLeft;
    int numStenRight;
    int numStenTop;
    int numStenBottom;
    int numStenHoriz;
    int numStenVert;
    int BLOCK_X;
    int BLOCK_Y;
    int xGrid;
    int yGrid;
    int mem_shared;
    double** dataInput;
    double** dataOutput;
    double** uVel;
    double** vVel;
    double* weights;
    double* coe;
    double coeDx;
    double coeDy;
    int numCoe;
    int nxLocal;
    int nyLocal;
    double** boundaryTop;
    double** boundaryBottom;
    int numBoundaryTop;
    int numBoundaryBottom;
    cudaStream_t* streams;
    cudaEvent_t* events;
    double* devFunc;
} cuSten_t;

/* ---- error utility (cuSten/src/util/util.h:43, error.cu:43-53) ---- */
void checkError(const char* action);

/* ---- 2D x direction, non periodic (cuSten_struct_functions.h:67-118) ---- */
void cuStenCreate2DXnp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                       double* dataOutput, double* dataInput, double* weights, int numSten, int numStenLeft,
                       int numStenRight);
void cuStenSwap2DXnp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXnp(cuSten_t* pt_cuSten);

/* ---- 2D x direction, non periodic, user function (:125-176) ---- */
void cuStenCreate2DXnpFun(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                          double* dateOutput, double* dateInput, double* coe, int numSten, int numStenLeft,
                          int numStenRight, int numCoe, double* func);
void cuStenSwap2DXnpFun(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXnpFun(cuSten_t* pt_cuSten);

/* ---- 2D x direction, periodic (:184-235) ---- */
void cuStenCreate2DXp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                      double* dataNew, double* dataOld, double* weights, int numSten, int numStenLeft,
                      int numStenRight);
void cuStenSwap2DXp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXp(cuSten_t* pt_cuSten);

/* ---- 2D x direction, periodic, user function (:242-293) ---- */
void cuStenCreate2DXpFun(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                         double* dataNew, double* dataOld, double* coe, int numSten, int numStenLeft,
                         int numStenRight, int numCoe, double* func);
void cuStenSwap2DXpFun(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXpFun(cuSten_t* pt_cuSten);

/* ---- 2D xy direction, non periodic (:371-422) ---- */
void cuStenCreate2DXYnp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                        double* dataOutput, double* dataInput, double* weights, int numStenHoriz, int numStenLeft,
                        int numStenRight, int numStenVert, int numStenTop, int numStenBottom);
void cuStenSwap2DXYnp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXYnp(cuSten_t* pt_cuSten);

/* ---- 2D xy direction, non periodic, user function (:435-486) ---- */
void cuStenCreate2DXYnpFun(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X,
                           int BLOCK_Y, double* dataNew, double* dataOld, double* coe, int numStenHoriz,
                           int numStenLeft, int numStenRight, int numStenVert, int numStenTop, int numStenBottom,
                           double* func);
void cuStenSwap2DXYnpFun(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXYnpFun(cuSten_t* pt_cuSten);

/* ---- 2D xy direction, periodic (:500-551) ---- */
void cuStenCreate2DXYp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                       double* dataNew, double* dataOld, double* weights, int numStenHoriz, int numStenLeft,
                       int numStenRight, int numStenVert, int numStenTop, int numStenBottom);
void cuStenSwap2DXYp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXYp(cuSten_t* pt_cuSten);

/* ---- 2D xy direction, periodic, user function (:564-615) ---- */
void cuStenCreate2DXYpFun(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X,
                          int BLOCK_Y, double* dataNew, double* dataOld, double* coe, int numStenHoriz,
                          int numStenLeft, int numStenRight, int numStenVert, int numStenTop, int numStenBottom,
                          double* func);
void cuStenSwap2DXYpFun(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXYpFun(cuSten_t* pt_cuSten);

/* ---- 2D y direction, non periodic (:626-677) ---- */
void cuStenCreate2DYnp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                       double* dataOutput, double* dataInput, double* weights, int numSten, int numStenTop,
                       int numStenBottom);
void cuStenSwap2DYnp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DYnp(cuSten_t* pt_cuSten);

/* ---- 2D y direction, non periodic, user function; no numCoe argument (:684-734) ---- */
void cuStenCreate2DYnpFun(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                          double* dataOutput, double* dataInput, double* coe, int numSten, int numStenTop,
                          int numStenBottom, double* func);
void cuStenSwap2DYnpFun(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DYnpFun(cuSten_t* pt_cuSten);

/* ---- 2D y direction, periodic (:742-793) ---- */
void cuStenCreate2DYp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                      double* dataOutput, double* dataInput, double* weights, int numSten, int numStenTop,
                      int numStenBottom);
void cuStenSwap2DYp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DYp(cuSten_t* pt_cuSten);

/* ---- 2D y direction, periodic, user function (:801-853) ---- */
void cuStenCreate2DYpFun(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X, int BLOCK_Y,
                         double* dataOutput, double* dataInput, double* coe, int numSten, int numStenTop,
                         int numStenBottom, int numCoe, double* func);
void cuStenSwap2DYpFun(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DYpFun(cuSten_t* pt_cuSten);

/* ---- 2D xy direction, periodic WENO advection (:290-347) ----
 * out = u * WENO5_x(in) + v * WENO5_y(in), upwinded on the signs of u and v; coeDx = 1/dx and
 * coeDy = 1/dy are stored in the handle. */
void cuStenCreate2DXYWENOADVp(cuSten_t* pt_cuSten, int deviceNum, int numTiles, int nx, int ny, int BLOCK_X,
                              int BLOCK_Y, double dx, double dy, double* u, double* v, double* dataOutput,
                              double* dataInput);
void cuStenSwap2DXYWENOADVp(cuSten_t* pt_cuSten, double* dataInput);
void cuStenDestroy2DXYWENOADVp(cuSten_t* pt_cuSten);

/* ---- Compute (cuSten/src/kernels/stencil_kernels.h:52-189) ---- */
void cuStenCompute2DXnp(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXnpFun(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXp(cuSten_t* pt_cuSten, bool offload);
/* The reference header declares cuStenCompute2DXpFun (stencil_kernels.h:85-90) but the reference
 * library defines cuSenCompute2DXpFun (kernels/2d_x_p_fun_kernel.cu:172). Both are defined here. */
void cuStenCompute2DXpFun(cuSten_t* pt_cuSten, bool offload);
void cuSenCompute2DXpFun(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DYp(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DYpFun(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DYnp(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DYnpFun(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXYp(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXYpFun(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXYnp(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXYnpFun(cuSten_t* pt_cuSten, bool offload);
void cuStenCompute2DXYWENOADVp(cuSten_t* pt_cuSten, bool offload);

#endif /* CUSTEN_H */
