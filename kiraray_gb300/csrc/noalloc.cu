// krr_accel_trace_stats_noalloc: the counter-instrumented trace replay
// (krr_accel_trace_stats) for callers that cannot allocate device memory.
//
// Who cannot allocate: render loops that have a fixed per-frame memory budget
// and must not call cudaMalloc/cudaFree mid-frame (both can synchronise the
// whole device and stall the frame), and hosts that hand all device memory to
// their own pool allocator up front.  krr_accel_trace_stats allocates its
// scratch (per-ray hit records, node/triangle counters, the ray work counter)
// on every call; this variant keeps that scratch in a file-scope device array
// instead and calls no allocating routine.
//
// Limits and sharing: the array holds the scratch of at most
// KRR_NOALLOC_MAX_RAYS rays (1 MiB of hit records plus 256 bytes of
// counters) and stays resident on every GPU that loads the library until
// the process exits.  All calls share it and it keeps the last call's
// contents; the counters are cleared at the start of every call.  Calls
// whose work overlaps on the GPU (on different streams, or from different
// host threads without ordering) race on the array and give wrong counts.
//
// Set-up: host code cannot use the array's name as a device address (on the
// host it names a stand-in object, not device memory), so the first call on
// each device looks the address up with cudaGetSymbolAddress, with that
// device current, and caches it for the life of the process: make that first
// call before any stream capture begins on the device, and do not reset the
// device (cudaDeviceReset) after it.
//
// The call is synchronous: it waits for the stream and copies the counts to
// the caller's host array before it returns.  A traversal cut off by the stack limit
// (krr_accel_set_stack_limit) makes it return KRR_ERR_OVERFLOW, as the
// allocating entry point does.
#include <mutex>

#include "accel.h"
#include "internal.h"

namespace krr {
int launch_trace_stats(const krr_accel *a, const TraceLaunch &l, bool any,
                       unsigned long long *d_stats, cudaStream_t s);
}

using namespace krr;

namespace {

// [0, 64): counters (2 x node/triangle totals, ray work counter, error flags)
// [64, 64 + 16 * max): closest-hit records, or one byte per ray for any-hit
constexpr size_t kCounterWords = 32;   // 256 bytes of 8-byte words
constexpr size_t kScratchWords = kCounterWords + 2 * (size_t)KRR_NOALLOC_MAX_RAYS;

static __device__ __align__(256) unsigned long long g_stats_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned long long *g_scratch_addr[kMaxDevices] = {};

int scratch_address(unsigned long long **out) {
    int dev = 0;
    KRR_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(KRR_ERR_INVALID_ARGUMENT, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_stats_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
        g_scratch_addr[dev] = static_cast<unsigned long long *>(p);
    }
    *out = g_scratch_addr[dev];
    return KRR_OK;
}

}  // namespace

extern "C" int krr_accel_trace_stats_noalloc(const krr_accel *a, const krr_ray *d_rays, int64_t n,
                                             int32_t any_hit, unsigned long long *h_counts,
                                             void *stream) {
    KRR_CHECK_ARG(a && d_rays && h_counts, "NULL argument");
    if (n <= 0 || n > (int64_t)KRR_NOALLOC_MAX_RAYS)
        return fail(KRR_ERR_INVALID_ARGUMENT,
                    "krr_accel_trace_stats_noalloc: %lld rays; the static scratch holds 1 to %d",
                    (long long)n, (int)KRR_NOALLOC_MAX_RAYS);
    if (a->n_tris == 0) return fail(KRR_ERR_NOT_READY, "empty acceleration structure");
    cudaStream_t s = as_stream(stream);
    unsigned long long *base = nullptr;
    KRR_TRY(scratch_address(&base));
    unsigned long long *counts = base;            // [0], [1]
    int *ray_counter = reinterpret_cast<int *>(base + 2);
    int *err = reinterpret_cast<int *>(base + 4);
    KRR_CUDA(cudaMemsetAsync(base, 0, kCounterWords * sizeof(unsigned long long), s));

    TraceLaunch l{};
    l.ray_o = reinterpret_cast<const float4 *>(d_rays);
    l.ray_d = reinterpret_cast<const float4 *>(d_rays) + 1;
    l.ray_stride = 2;
    l.n = n;
    l.d_count = nullptr;
    l.counter = ray_counter;
    l.err = err;
    l.hits = reinterpret_cast<float4 *>(base + kCounterWords);
    l.occluded = reinterpret_cast<uint8_t *>(base + kCounterWords);
    KRR_TRY(launch_trace_stats(a, l, any_hit != 0, counts, s));
    KRR_CUDA(cudaMemcpyAsync(h_counts, counts, 2 * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, s));
    return take_trace_errors(err, s, nullptr);
}
