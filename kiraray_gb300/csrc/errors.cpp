// Status codes and the per-thread last-error text of the C ABI.
#include <cstdarg>
#include <cstdio>
#include <string>

#include "internal.h"

namespace krr {

static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }

int fail(int status, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

}  // namespace krr

extern "C" const char *krr_last_error(void) { return krr::g_last_error.c_str(); }

extern "C" const char *krr_status_string(int status) {
    switch (status) {
        case KRR_OK: return "ok";
        case KRR_ERR_INVALID_ARGUMENT: return "invalid argument";
        case KRR_ERR_CUDA: return "CUDA error";
        case KRR_ERR_OVERFLOW: return "capacity overflow";
        case KRR_ERR_TIMEOUT: return "device wait timed out";
        case KRR_ERR_NOT_READY: return "not ready";
        case KRR_ERR_OUT_OF_MEMORY: return "out of memory";
        default: return "unknown status";
    }
}

extern "C" int krr_version(void) { return 1; }
