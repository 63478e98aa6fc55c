// Checked builds: index checks that report instead of trapping.
//
// Compiled with -DCUSTEN_CHECKED=1 (custen_gb300.build(checked=True), a separate library), the kernels
// re-check the indexes of their global stores and of their shared-window reads against the extents the
// accesses must stay in. A violation raises kErrBounds in the device error flags (custen_device_error)
// and the access is skipped, so a stray index shows up as a flag on the host, never as a fault. It is
// the stand-in for a memory checker on GPUs where none may run. In normal builds every check compiles
// to nothing.
#pragma once

#ifndef CUSTEN_CHECKED
#define CUSTEN_CHECKED 0
#endif

namespace custen {

extern __device__ unsigned int g_custen_device_error;
constexpr unsigned int kErrBounds = 2u;

// True when lo <= idx < hi; in checked builds a violation also raises kErrBounds.
__device__ __forceinline__ bool in_bounds(long long idx, long long lo, long long hi) {
#if CUSTEN_CHECKED
    if (idx < lo || idx >= hi) {
        atomicOr(&g_custen_device_error, kErrBounds);
        return false;
    }
#else
    (void)idx; (void)lo; (void)hi;
#endif
    return true;
}

// A span [first, first + count) inside [0, extent).
__device__ __forceinline__ bool span_ok(long long first, long long count, long long extent) {
    return in_bounds(first, 0, extent) && in_bounds(first + count - 1, 0, extent);
}

}  // namespace custen
