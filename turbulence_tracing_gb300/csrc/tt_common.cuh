// Shared helpers for the libturbotrace CUDA sources (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/turbotrace.h"

#define TT_C_LIGHT 299792458.0

namespace tt {

// Per-host-thread detail message for the last failure (tt_last_error_detail).
void set_detail(const char* fmt, ...);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int cuda_status(cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return TT_OK;
    set_detail("%s: %s", where, cudaGetErrorString(e));
    return TT_ERR_CUDA;
}

// Launch-error check after a kernel launch.
inline int launch_status(const char* where) { return cuda_status(cudaGetLastError(), where); }

inline int invalid(const char* fmt_what)
{
    set_detail("%s", fmt_what);
    return TT_ERR_INVALID_ARGUMENT;
}

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// SM count of the current device, cached per device.
int sm_count();

}  // namespace tt

#define TT_TRY(expr)                     \
    do {                                 \
        int tt_rc__ = (expr);            \
        if (tt_rc__ != TT_OK) return tt_rc__; \
    } while (0)
