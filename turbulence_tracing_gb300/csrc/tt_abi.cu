// Status strings, error detail and device queries shared by every entry point.
#include <stdarg.h>

#include <atomic>
#include <string.h>

#include "tt_common.cuh"

namespace tt {

static thread_local char g_detail[512];

void set_detail(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_detail, sizeof(g_detail), fmt, ap);
    va_end(ap);
}

int sm_count()
{
    // per-device cache; threads may race to fill an entry, all with the same value
    static std::atomic<int> cached[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < 64) {
        const int c = cached[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int n = 1;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    if (dev >= 0 && dev < 64) cached[dev].store(n, std::memory_order_relaxed);
    return n;
}

}  // namespace tt

extern "C" int tt_abi_version(void) { return TT_ABI_VERSION; }

extern "C" const char* tt_strerror(int status)
{
    switch (status) {
        case TT_OK: return "ok";
        case TT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case TT_ERR_WORKSPACE_TOO_SMALL: return "workspace too small";
        case TT_ERR_CUDA: return "CUDA error";
        case TT_ERR_CUFFT: return "cuFFT error";
        case TT_ERR_UNSUPPORTED: return "unsupported input";
        case TT_ERR_TOO_LARGE: return "size above the supported maximum";
        default: return "unknown status";
    }
}

extern "C" const char* tt_last_error_detail(void) { return tt::g_detail; }
