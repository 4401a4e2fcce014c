// Exhaustive autotuner: times every variant of the search space on one
// matrix and reports the per-variant times and the fastest.  Its timings are
// the labels the learned selector is trained on, and its result is the
// selector's fallback when the network is not confident.  The reference has
// no autotuner; its closest pieces are the fixed dispatch rules
// (src/spmv/csr/spmv_csr.cu:115-153) and the manual sweeps of
// tests/test_block_optimization.cu:147-290.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "kernels.h"
#include "plan.h"

namespace mxs {

// The search space: kernel family x block size x threads per row x items per
// thread x load width.  Order is part of the ABI (selector outputs index it).
static const spmv_variant_t kSpace[] = {
    {SPMV_KERNEL_SCALAR, 128, 1, 0, 1},
    {SPMV_KERNEL_SCALAR, 256, 1, 0, 1},
    {SPMV_KERNEL_VECTOR, 256, 2, 0, 4},
    {SPMV_KERNEL_VECTOR, 256, 4, 0, 4},
    {SPMV_KERNEL_VECTOR, 256, 8, 0, 4},
    {SPMV_KERNEL_VECTOR, 256, 16, 0, 4},
    {SPMV_KERNEL_VECTOR, 256, 32, 0, 4},
    {SPMV_KERNEL_VECTOR, 128, 4, 0, 4},
    {SPMV_KERNEL_VECTOR, 512, 4, 0, 4},
    {SPMV_KERNEL_VECTOR, 128, 16, 0, 4},
    {SPMV_KERNEL_VECTOR, 512, 16, 0, 4},
    {SPMV_KERNEL_MERGE, 256, 0, 4, 4},
    {SPMV_KERNEL_MERGE, 256, 0, 8, 4},
    {SPMV_KERNEL_MERGE, 256, 0, 12, 4},
    {SPMV_KERNEL_MERGE, 128, 0, 8, 4},
    {SPMV_KERNEL_CSR5, 256, 0, 8, 1},
    {SPMV_KERNEL_CSR5, 128, 0, 8, 32},
    {SPMV_KERNEL_CSR5, 128, 0, 4, 32},
    {SPMV_KERNEL_CSR5, 256, 0, 8, 32},
    {SPMV_KERNEL_CSR5, 128, 0, 16, 32},
    {SPMV_KERNEL_CSR5, 512, 0, 8, 32},
    {SPMV_KERNEL_BAND, 1024, 25, 8, 14},
    {SPMV_KERNEL_ELL, 256, 0, 0, 1},
    // block ranges, one per resident block (contiguous tiles per SM)
    {SPMV_KERNEL_CSR5, 1024, SPMV_RANGE_PER_RESIDENT_BLOCK, 16, SPMV_CSR5_ORDERED},
    {SPMV_KERNEL_CSR5, 640, SPMV_RANGE_PER_RESIDENT_BLOCK, 16, SPMV_CSR5_ORDERED},
    // the same with the next tile's loads in flight during the current tile
    {SPMV_KERNEL_CSR5, 1024, SPMV_RANGE_PER_RESIDENT_BLOCK, 8, SPMV_CSR5_ORDERED_PREFETCH},
    {SPMV_KERNEL_CSR5, 512, SPMV_RANGE_PER_RESIDENT_BLOCK, 16, SPMV_CSR5_ORDERED_PREFETCH},
    {SPMV_KERNEL_STREAM, 1024, 2, 8, 0},
};
constexpr int kSpaceSize = (int)(sizeof(kSpace) / sizeof(kSpace[0]));

int variant_space(spmv_variant_t* out, int cap) {
    if (out)
        for (int i = 0; i < kSpaceSize && i < cap; ++i) out[i] = kSpace[i];
    return kSpaceSize;
}

template <typename T>
__global__ void fill_kernel_t(long long n, T* __restrict__ v, T value) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[i] = value;
}

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

template <typename T>
static spmv_status_t tune(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                          const int* colIdx, const void* values, const spmv_variant_t* cand, int nc, int repeats,
                          float* msOut, int* best) {
    const cudaStream_t s = h->stream;
    T* x = nullptr;
    T* y = nullptr;
    MXS_CUDA(dev_malloc(&x, sizeof(T) * (size_t)(C > 0 ? C : 1)));
    cudaError_t e = dev_malloc(&y, sizeof(T) * (size_t)(R > 0 ? R : 1));
    if (e != cudaSuccess) {
        dev_free(x);
        return cuda_fail(e, "autotune buffers", __FILE__, __LINE__);
    }
    fill_kernel_t<T><<<256, 256, 0, s>>>(C, x, T(1));
    EventPair ev;
    cudaEventCreate(&ev.a);
    cudaEventCreate(&ev.b);
    float bestMs = 3.4e38f;
    int bestIdx = -1;
    spmv_status_t result = SPMV_SUCCESS;
    for (int i = 0; i < nc; ++i) {
        msOut[i] = -1.0f;
        spmv_plan_t p = nullptr;
        if (spmv_plan_create(h, type, R, C, N, rowPtr, colIdx, values, &cand[i], &p) != SPMV_SUCCESS) continue;
        auto exec = [&]() {
            return sizeof(T) == 4 ? spmv_plan_exec_f32(h, p, 1.0f, reinterpret_cast<const float*>(x), 0.0f,
                                                       reinterpret_cast<float*>(y))
                                  : spmv_plan_exec_f64(h, p, 1.0, reinterpret_cast<const double*>(x), 0.0,
                                                       reinterpret_cast<double*>(y));
        };
        // One timed warm-up decides how many repeats this variant deserves:
        // variants 20x slower than the best so far are not repeated.
        spmv_status_t st = exec();
        cudaEventRecord(ev.a, s);
        if (st == SPMV_SUCCESS) st = exec();
        cudaEventRecord(ev.b, s);
        float warm = 0.f;
        if (cudaEventSynchronize(ev.b) != cudaSuccess || cudaEventElapsedTime(&warm, ev.a, ev.b) != cudaSuccess)
            st = SPMV_ERROR_DEVICE;
        if (st == SPMV_SUCCESS) {
            float ms = warm;
            if (warm < 20.0f * bestMs) {
                // repeats <= 0: loop for about 2 ms (3..500 executions).
                int reps = repeats;
                if (reps <= 0) {
                    const float want = 2.0f / (warm > 1e-4f ? warm : 1e-4f);
                    reps = want < 3.f ? 3 : (want > 500.f ? 500 : (int)want);
                }
                cudaEventRecord(ev.a, s);
                for (int r = 0; r < reps && st == SPMV_SUCCESS; ++r) st = exec();
                cudaEventRecord(ev.b, s);
                if (cudaEventSynchronize(ev.b) == cudaSuccess && cudaEventElapsedTime(&ms, ev.a, ev.b) == cudaSuccess)
                    ms /= (float)reps;
                else
                    st = SPMV_ERROR_DEVICE;
            }
            int devErr = 0;
            if (st == SPMV_SUCCESS && spmv_plan_device_error(p, &devErr) != SPMV_SUCCESS) st = SPMV_ERROR_DEVICE;
            if (st == SPMV_SUCCESS) {
                msOut[i] = ms;
                if (ms < bestMs) {
                    bestMs = ms;
                    bestIdx = i;
                }
            }
        }
        spmv_plan_destroy(p);
        if (st == SPMV_ERROR_DEVICE) {
            result = st;
            break;
        }
    }
    dev_free(x);
    dev_free(y);
    if (best) *best = bestIdx;
    if (result != SPMV_SUCCESS) MXS_FAIL(result, "autotune aborted on a device error");
    if (bestIdx < 0) MXS_FAIL(SPMV_ERROR_INTERNAL, "no variant could run on this matrix");
    return SPMV_SUCCESS;
}

}  // namespace mxs

using namespace mxs;

extern "C" {

int spmv_variant_space(spmv_variant_t* out, int capacity) { return variant_space(out, capacity); }

spmv_status_t spmv_autotune(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                            const int* colIdx, const void* values, const spmv_variant_t* candidates,
                            int numCandidates, int repeats, float* msOut, int* bestIndex) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!msOut) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "msOut is NULL");
    std::vector<spmv_variant_t> space;
    if (!candidates) {
        space.resize(variant_space(nullptr, 0));
        variant_space(space.data(), (int)space.size());
        candidates = space.data();
        numCandidates = (int)space.size();
    }
    if (numCandidates <= 0) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "no candidates");
    if (type == SPMV_TYPE_FLOAT)
        return tune<float>(h, type, R, C, N, rowPtr, colIdx, values, candidates, numCandidates, repeats, msOut,
                           bestIndex);
    if (type == SPMV_TYPE_DOUBLE)
        return tune<double>(h, type, R, C, N, rowPtr, colIdx, values, candidates, numCandidates, repeats, msOut,
                            bestIndex);
    MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "float or double");
}

}  // extern "C"
