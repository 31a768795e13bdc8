// trace.cu -- launch counter and per-kernel-class CUDA-event timing behind
// MLU_LAUNCH (trace.cuh).  No counterpart in the reference, whose testers
// time whole calls on the host (testing/testing_zgesv_batched.cpp:158-166);
// a benchmark uses this to attribute device time to one kernel of a
// multi-kernel routine without a profiler.  Meant for one host thread.
#include "common.cuh"
#include "trace.cuh"

#include <atomic>
#include <mutex>
#include <vector>

namespace {
std::atomic<unsigned long long> g_launches{0};
std::atomic<int> g_class{-1};
std::mutex g_mu;
std::vector<cudaEvent_t> g_events;   // a start/end pair per timed launch
int g_capacity = 0, g_used = 0, g_dropped = 0;
bool g_open = false;

void release_events() {
    for (cudaEvent_t e : g_events) cudaEventDestroy(e);
    g_events.clear();
    g_capacity = g_used = g_dropped = 0;
    g_open = false;
}
}  // namespace

void mlu::trace_before(int cls, cudaStream_t s) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (g_class.load(std::memory_order_relaxed) != cls) return;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    if (st != cudaStreamCaptureStatusNone) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_used >= g_capacity) {
        g_dropped++;
        return;
    }
    g_open = cudaEventRecord(g_events[2 * g_used], s) == cudaSuccess;
}

void mlu::trace_after(int cls, cudaStream_t s) {
    if (g_class.load(std::memory_order_relaxed) != cls) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_open) return;
    g_open = false;
    if (cudaEventRecord(g_events[2 * g_used + 1], s) == cudaSuccess) g_used++;
}

extern "C" long long magma_lu_launch_count(void) {
    return (long long)g_launches.load(std::memory_order_relaxed);
}

extern "C" magma_int_t magma_lu_timing_start(magma_int_t kernel_class, magma_int_t capacity) {
    if (kernel_class < 0 || kernel_class >= mlu::KC_COUNT) return -1;
    if (capacity <= 0 || capacity > (1 << 20)) return -2;
    std::lock_guard<std::mutex> lk(g_mu);
    g_class.store(-1);
    release_events();
    g_events.resize(2 * (size_t)capacity);
    for (size_t i = 0; i < g_events.size(); i++) {
        if (cudaEventCreate(&g_events[i]) != cudaSuccess) {
            g_events.resize(i);
            release_events();
            cudaGetLastError();
            return MAGMA_ERR_UNKNOWN;
        }
    }
    g_capacity = capacity;
    g_class.store(kernel_class);
    return MAGMA_SUCCESS;
}

extern "C" magma_int_t magma_lu_timing_stop(magma_int_t *launches, magma_int_t *dropped,
                                            double *total_ms) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_class.store(-1);
    double ms = 0.0;
    magma_int_t rc = MAGMA_SUCCESS;
    for (int i = 0; i < g_used; i++) {
        float t = 0.f;
        if (cudaEventSynchronize(g_events[2 * i + 1]) != cudaSuccess ||
            cudaEventElapsedTime(&t, g_events[2 * i], g_events[2 * i + 1]) != cudaSuccess) {
            cudaGetLastError();
            rc = MAGMA_ERR_UNKNOWN;
            break;
        }
        ms += t;
    }
    if (launches) *launches = g_used;
    if (dropped) *dropped = g_dropped;
    if (total_ms) *total_ms = ms;
    release_events();
    return rc;
}
