// Status codes and per-thread error messages of the C ABI.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace s2c {

static thread_local char g_msg[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

s2c_status cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return S2C_OK;
    set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return S2C_ERR_CUDA;
}

}  // namespace s2c

extern "C" int s2c_version(void) { return 1; }
extern "C" const char* s2c_last_error(void) { return s2c::g_msg; }
