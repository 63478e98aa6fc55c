// Compiles the device code of the reference's Cahn-Hilliard GPU timing program, unchanged, from the
// reference sources into one sm_103a cubin (oracle/_ref/custen_ref_ch_sm103a.cubin) -- TEST
// INFRASTRUCTURE ONLY. Built by oracle/ref_build.py where the reference sources exist (REF_ROOT);
// driven by oracle/ref_ch_runner.cpp.
//
// One translation unit, so that the XYpFun kernel and the nonLinRHS function that the program hands it
// through `devFunc` live in the same module. The program's macros (BLOCK_X, ...) come last because the
// cuSten kernel files use those names as parameters. Host code in these files is parsed, not built.
#define CUSTEN_REF_FILE(f) <REF_ROOT/f>
#include CUSTEN_REF_FILE(cuSten/src/kernels/2d_xy_p_kernel.cu)
#include CUSTEN_REF_FILE(cuSten/src/kernels/2d_xy_p_fun_kernel.cu)
#include CUSTEN_REF_FILE(cuPentSpeedUp/cuPentCahnADITiming/src/cuPentBatch.cu)
#include CUSTEN_REF_FILE(cuPentSpeedUp/cuPentCahnADITiming/src/BatchHyper.cu)
#include CUSTEN_REF_FILE(cuPentSpeedUp/cuPentCahnADITiming/src/cuPentCahnADI.cu)
