// Host-side internals shared by the translation units of libmuxispmv.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "muxi_spmv.h"

namespace mxs {

// Records a message for spmv_last_error() on the calling host thread.
void set_error(const char* file, int line, const char* fmt, ...);
void clear_error();

// Maps a CUDA error to SPMV_ERROR_DEVICE and records its text.
spmv_status_t cuda_fail(cudaError_t e, const char* what, const char* file, int line);

inline cudaStream_t opts_stream(const spmv_opts_t* o) {
    return (o && o->stream) ? reinterpret_cast<cudaStream_t>(o->stream) : (cudaStream_t)0;
}

// 16-byte loads of colIdx / values need both arrays 16-byte aligned.
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// Launch shape helpers.
inline unsigned grid_for(long long work, int per_block) {
    long long g = (work + per_block - 1) / per_block;
    return (unsigned)(g < 1 ? 1 : g);
}

// Internal state hanging off spmv_handle_t::internal.
struct HandleState {
    int device = 0;
    spmv_mlp_t selector = nullptr;  // borrowed; AUTO plans consult it when set
    spmv_select_mode_t selectorMode = SPMV_SELECT_LEARNED;  // or SPMV_SELECT_LEARNED_FALLBACK
};

// Device allocations of the library (device_memory.cu): counted while live,
// and failable on demand for tests (spmv_debug_fail_allocation).
cudaError_t dev_malloc(void** p, size_t bytes);
template <typename T>
inline cudaError_t dev_malloc(T** p, size_t bytes) {
    return dev_malloc(reinterpret_cast<void**>(p), bytes);
}
cudaError_t dev_free(void* p);
cudaError_t dev_malloc_async(void** p, size_t bytes, cudaStream_t s);
template <typename T>
inline cudaError_t dev_malloc_async(T** p, size_t bytes, cudaStream_t s) {
    return dev_malloc_async(reinterpret_cast<void**>(p), bytes, s);
}
cudaError_t dev_malloc_pool_async(void** p, size_t bytes, cudaMemPool_t pool, cudaStream_t s);
cudaError_t dev_free_async(void* p, cudaStream_t s);

// Per-device properties cached on first use (SM count, L2 size, smem).
struct DeviceProps {
    int sm_count = 0;
    size_t l2_bytes = 0;
    size_t smem_optin = 0;
    size_t smem_per_sm = 0;
    int cc_major = 0, cc_minor = 0;
};
const DeviceProps& device_props(int dev);

// Returns the current device's SM count (cached).
int current_sm_count();

}  // namespace mxs

#define MXS_CUDA(expr)                                                        \
    do {                                                                      \
        cudaError_t e_ = (expr);                                              \
        if (e_ != cudaSuccess) return mxs::cuda_fail(e_, #expr, __FILE__, __LINE__); \
    } while (0)

#define MXS_LAUNCH_CHECK()                                                    \
    do {                                                                      \
        cudaError_t e_ = cudaGetLastError();                                  \
        if (e_ != cudaSuccess) return mxs::cuda_fail(e_, "kernel launch", __FILE__, __LINE__); \
    } while (0)

#define MXS_FAIL(status, ...)                                                 \
    do {                                                                      \
        mxs::set_error(__FILE__, __LINE__, __VA_ARGS__);                      \
        return (status);                                                      \
    } while (0)

#define MXS_TRY(expr)                                                         \
    do {                                                                      \
        spmv_status_t s_ = (expr);                                            \
        if (s_ != SPMV_SUCCESS) return s_;                                    \
    } while (0)
