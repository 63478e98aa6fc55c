// Compiles the reference cuSten kernels (the twelve stencils and the WENO advection), unchanged, from the reference sources into one sm_103a
// cubin (oracle/_ref/custen_ref_sm103a.cubin) -- TEST INFRASTRUCTURE ONLY. Built by
// oracle/ref_build.py where the reference sources exist (REF_ROOT); driven by oracle/ref_runner.cpp.
// The user functions are the library's shipped Fun functions (custen_gb300/csrc/builtin_funs.cuh),
// so the reference Fun kernels and the library's call identical device code.
#include "custen_gb300/csrc/builtin_funs.cuh"

#define CUSTEN_REF_KERNEL(f) <REF_ROOT/cuSten/src/kernels/f>
#include CUSTEN_REF_KERNEL(2d_x_p_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_x_np_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_x_p_fun_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_x_np_fun_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_y_p_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_y_np_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_y_p_fun_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_y_np_fun_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_xy_p_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_xy_np_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_xy_p_fun_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_xy_np_fun_kernel.cu)
#include CUSTEN_REF_KERNEL(2d_xyADVWENO_p_kernel.cu)

typedef double (*RefFx)(double*, double*, int);
typedef double (*RefFy)(double*, double*, int, int);
typedef double (*RefFxy)(double*, double*, int, int, int, int);
extern "C" {
__device__ RefFx custen_ref_fun0 = custen_funs::x_second_diff<double>;
__device__ RefFx custen_ref_fun1 = custen_funs::x_cube_lap5<double>;
__device__ RefFy custen_ref_fun2 = custen_funs::y_central9<double>;
__device__ RefFy custen_ref_fun3 = custen_funs::y_cube_lap5<double>;
__device__ RefFxy custen_ref_fun4 = custen_funs::xy_weighted<double>;
__device__ RefFxy custen_ref_fun5 = custen_funs::xy_cube<double>;
}
