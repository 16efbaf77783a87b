// Host-side plumbing shared by the translation units of libkrr_gb300.so:
// status codes, the per-thread last-error text and CUDA error mapping.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>

#include "../../include/krr_gb300.h"

namespace krr {

void set_last_error(const std::string &msg);
int fail(int status, const char *fmt, ...);

inline int cuda_status(cudaError_t e, const char *what, const char *file, int line) {
    if (e == cudaSuccess) return KRR_OK;
    return fail(e == cudaErrorMemoryAllocation ? KRR_ERR_OUT_OF_MEMORY : KRR_ERR_CUDA,
                "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Device-side error flags (set by kernels instead of trapping).
enum DeviceError : uint32_t {
    kErrStackOverflow = 1u << 0,
    kErrQueueOverflow = 1u << 1,
    kErrLoopLimit = 1u << 2,
    kErrBadInput = 1u << 3,
};

}  // namespace krr

#define KRR_CUDA(call)                                                              \
    do {                                                                            \
        cudaError_t _e = (call);                                                    \
        if (_e != cudaSuccess) return ::krr::cuda_status(_e, #call, __FILE__, __LINE__); \
    } while (0)

#define KRR_TRY(call)                  \
    do {                               \
        int _s = (call);               \
        if (_s != KRR_OK) return _s;   \
    } while (0)

#define KRR_CHECK_ARG(cond, msg)                                                   \
    do {                                                                           \
        if (!(cond)) return ::krr::fail(KRR_ERR_INVALID_ARGUMENT, "%s", msg);      \
    } while (0)
