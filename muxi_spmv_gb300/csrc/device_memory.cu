// Every device allocation of the library goes through these wrappers, which
// (a) count the live allocations and bytes, so a test can show that a call
// that failed half-way released everything it had taken, and (b) can be told
// to fail the n-th allocation from now with cudaErrorMemoryAllocation,
// without asking the CUDA driver, so the library's out-of-memory paths run on any
// machine.  Neither changes what a successful call does.
#include <atomic>
#include <mutex>
#include <unordered_map>

#include "internal.h"

namespace mxs {
namespace {

std::mutex g_mu;
std::unordered_map<void*, size_t> g_live;  // device pointer -> bytes
long long g_liveBytes = 0;
std::atomic<long long> g_failCountdown{0};  // > 0: allocations left until the injected failure

// True when this allocation is the one to fail.
bool injected_failure() {
    long long c = g_failCountdown.load();
    while (c > 0) {
        if (g_failCountdown.compare_exchange_weak(c, c - 1)) return c == 1;
    }
    return false;
}

void track(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_mu);
    g_live[p] = bytes;
    g_liveBytes += (long long)bytes;
}

void untrack(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_live.find(p);
    if (it == g_live.end()) return;
    g_liveBytes -= (long long)it->second;
    g_live.erase(it);
}

}  // namespace

cudaError_t dev_malloc(void** p, size_t bytes) {
    *p = nullptr;
    if (injected_failure()) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) track(*p, bytes);
    return e;
}

cudaError_t dev_free(void* p) {
    untrack(p);
    return cudaFree(p);
}

cudaError_t dev_malloc_async(void** p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    if (injected_failure()) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaMallocAsync(p, bytes, s);
    if (e == cudaSuccess) track(*p, bytes);
    return e;
}

cudaError_t dev_malloc_pool_async(void** p, size_t bytes, cudaMemPool_t pool, cudaStream_t s) {
    *p = nullptr;
    if (injected_failure()) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, s);
    if (e == cudaSuccess) track(*p, bytes);
    return e;
}

cudaError_t dev_free_async(void* p, cudaStream_t s) {
    untrack(p);
    return cudaFreeAsync(p, s);
}

}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_debug_fail_allocation(long long n) {
    clear_error();
    if (n < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "allocation index must be >= 0 (0 turns injection off)");
    g_failCountdown.store(n);
    return SPMV_SUCCESS;
}

spmv_status_t spmv_debug_device_memory(long long* liveBytes, long long* liveAllocations) {
    clear_error();
    if (!liveBytes || !liveAllocations) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL argument");
    std::lock_guard<std::mutex> lk(g_mu);
    *liveBytes = g_liveBytes;
    *liveAllocations = (long long)g_live.size();
    return SPMV_SUCCESS;
}

}  // extern "C"
