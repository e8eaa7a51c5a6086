// bounds.cuh -- device-side index checks of the debug build.
//
// Built with SGDG_DEBUG (the build's SGDG_DEBUG=1), every gather and scatter
// index of the matrix-free stage kernel, the CSR kernels and the device
// assembly is checked against the length of the vector it addresses; a
// failed check adds one to this translation unit's violation counter and the
// access is skipped -- no trap, no fault, the context stays usable -- and the
// host reads the counters with sgdg_debug_bounds.  In the normal build the
// checks compile to nothing.
#pragma once
#include <cuda_runtime.h>

#ifdef SGDG_DEBUG
static __device__ unsigned int g_bounds_violations;
// true when 0 <= i < n; otherwise counts a violation and is false
#define SGDG_IN(i, n) \
    (((unsigned long long)(long long)(i) < (unsigned long long)(long long)(n)) || (atomicAdd(&g_bounds_violations, 1u), false))
// host side: this translation unit's counter (read, and optionally reset)
#define SGDG_BOUNDS_READER(name)                                                   \
    cudaError_t name(unsigned int* out, bool reset) {                              \
        cudaError_t e = cudaMemcpyFromSymbol(out, g_bounds_violations, sizeof(unsigned int)); \
        if (e == cudaSuccess && reset) {                                           \
            const unsigned int z = 0;                                              \
            e = cudaMemcpyToSymbol(g_bounds_violations, &z, sizeof(unsigned int)); \
        }                                                                          \
        return e;                                                                  \
    }
#else
#define SGDG_IN(i, n) true
#define SGDG_BOUNDS_READER(name)                        \
    cudaError_t name(unsigned int* out, bool) {         \
        *out = 0;                                       \
        return cudaSuccess;                             \
    }
#endif
