// Host-to-host SpMV pipeline: x arrives in pinned host memory, y leaves to
// pinned host memory, and the copies overlap the SpMV.
//
// The reference measures this path with one stream per row range and whole-
// vector copies around the kernels (tests/test_pinned_memory.cu:245-380,
// testPinnedMultiStream): its copies never overlap its kernels.  Here the
// matrix is cut into row slices of equal merge-path length (rows + nonzeros),
// each slice is an ordinary plan over a rebased rowPtr, and
//   * the copy of slice s of y to the host starts as soon as slice s is done,
//     while later slices compute (consecutive slices alternate between two
//     compute streams, so one slice's tail overlaps the next slice's start);
//   * up to `depth` requests are in flight, each with its own device x / y
//     buffers, so request i+1's x copy runs under request i's SpMV.
// Request order on each stream and one event per (slot, slice) carry every
// dependency; the host never waits inside submit.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "plan.h"

namespace mxs {

// Slice boundaries: boundary s sits on merge-path diagonal d = s*(R+N)/S, at
// the largest row r with r + rowPtr[r] <= d (rows [rowStart[s], rowStart[s+1])
// form slice s).  rowPtr is monotone, so r + rowPtr[r] is strictly increasing.
// The boundary then moves back (at most 256 rows) to a row whose first nonzero
// sits at a multiple of 4, so every slice's colIdx / values start 16-byte
// aligned and the kernels that read 16-byte quads keep them; with no such row
// nearby it falls to row 0 and the host drops it.
__global__ void slice_bounds_kernel(const int* __restrict__ rowPtr, int R, int N, int S, int* __restrict__ rowStart,
                                    int* __restrict__ nnzStart) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > S) return;
    const long long L = (long long)R + N;
    const long long d = L * s / S;
    int lo = 0, hi = R;  // answer in [lo, hi]
    while (lo < hi) {
        const int mid = lo + (hi - lo + 1) / 2;
        if ((long long)mid + rowPtr[mid] <= d)
            lo = mid;
        else
            hi = mid - 1;
    }
    if (s == S) {
        lo = R;
    } else if (s > 0) {
        int r = lo;
        while (r > 0 && lo - r < 256 && (rowPtr[r] & 3)) --r;
        lo = (rowPtr[r] & 3) ? 0 : r;
    }
    rowStart[s] = lo;
    nnzStart[s] = rowPtr[lo];
}

// out[i] = rowPtr[r0 + i] - rowPtr[r0] for i in [0, rows].
__global__ void rebase_rows_kernel(const int* __restrict__ rowPtr, int r0, int rows, int* __restrict__ out) {
    const int base = rowPtr[r0];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i <= rows; i += (long long)gridDim.x * blockDim.x)
        out[i] = rowPtr[r0 + i] - base;
}

}  // namespace mxs

using namespace mxs;

struct spmv_pipeline_s {
    spmv_type_t type = SPMV_TYPE_FLOAT;
    int numRows = 0, numCols = 0, nnz = 0;
    int depth = 0;
    spmv_variant_t variant{};
    std::vector<int> rowStart;       // slice s = rows [rowStart[s], rowStart[s+1])
    std::vector<spmv_plan_t> plans;  // one per slice
    int* rebased = nullptr;          // all slices' rebased rowPtr arrays
    char* xbuf = nullptr;            // depth device copies of x
    char* ybuf = nullptr;            // depth device copies of y
    size_t deviceBytes = 0;
    cudaStream_t sIn = nullptr, sOut = nullptr, sComp[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> evIn, evOut;  // per slot
    std::vector<cudaEvent_t> evSlice;      // per slot x slice
    cudaEvent_t evOrder = nullptr;         // spmv_pipeline_order_after
    cudaEvent_t evJoin[4] = {nullptr, nullptr, nullptr, nullptr};
    long long submitted = 0;
};

static void pipeline_free(spmv_pipeline_t p) {
    if (!p) return;
    for (cudaStream_t s : {p->sIn, p->sOut, p->sComp[0], p->sComp[1]})
        if (s) cudaStreamSynchronize(s);
    for (spmv_plan_t q : p->plans)
        if (q) spmv_plan_destroy(q);
    for (auto v : {&p->evIn, &p->evOut, &p->evSlice})
        for (cudaEvent_t e : *v)
            if (e) cudaEventDestroy(e);
    if (p->evOrder) cudaEventDestroy(p->evOrder);
    for (cudaEvent_t e : p->evJoin)
        if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {p->sIn, p->sOut, p->sComp[0], p->sComp[1]})
        if (s) cudaStreamDestroy(s);
    if (p->rebased) dev_free(p->rebased);
    if (p->xbuf) dev_free(p->xbuf);
    if (p->ybuf) dev_free(p->ybuf);
    delete p;
}

static spmv_status_t pipeline_build(spmv_handle_t* h, spmv_pipeline_t p, const int* rowPtr, const int* colIdx,
                                    const void* values, const spmv_variant_t* variant, int S) {
    const int R = p->numRows, C = p->numCols, N = p->nnz;
    const size_t vs = p->type == SPMV_TYPE_FLOAT ? 4 : 8;
    const cudaStream_t hs = h->stream;
    // One variant for every slice, chosen on the whole matrix.
    MXS_TRY(plan_variant(h, p->type, R, C, N, rowPtr, colIdx, values, variant, &p->variant));
    for (cudaStream_t* s : {&p->sIn, &p->sOut, &p->sComp[0], &p->sComp[1]})
        MXS_CUDA(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));

    // Slice boundaries (empty slices, e.g. inside one long row, are dropped).
    std::vector<int> rows(S + 1), nz(S + 1);
    if (R > 0) {
        int* d = nullptr;
        MXS_CUDA(dev_malloc_async(&d, 2 * sizeof(int) * (S + 1), hs));
        slice_bounds_kernel<<<grid_for(S + 1, 128), 128, 0, hs>>>(rowPtr, R, N, S, d, d + S + 1);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(rows.data(), d, sizeof(int) * (S + 1), cudaMemcpyDeviceToHost, hs);
        if (e == cudaSuccess) e = cudaMemcpyAsync(nz.data(), d + S + 1, sizeof(int) * (S + 1), cudaMemcpyDeviceToHost, hs);
        dev_free_async(d, hs);
        if (e == cudaSuccess) e = cudaStreamSynchronize(hs);
        if (e != cudaSuccess) return cuda_fail(e, "pipeline slice bounds", __FILE__, __LINE__);
    }
    // Keep strictly increasing boundaries: nnzAt[s] = rowPtr[rowStart[s]].
    std::vector<int> nnzAt;
    p->rowStart.push_back(0);
    nnzAt.push_back(0);
    for (int s = 1; s <= S && R > 0; ++s)
        if (rows[s] > p->rowStart.back()) {
            p->rowStart.push_back(rows[s]);
            nnzAt.push_back(nz[s]);
        }
    const int slices = (int)p->rowStart.size() - 1;

    // Rebased rowPtr of every slice, then one plan per slice.
    if (slices > 0) {
        const size_t total = (size_t)R + slices;
        MXS_CUDA(dev_malloc(&p->rebased, sizeof(int) * total));
        p->deviceBytes += sizeof(int) * total;
        size_t off = 0;
        for (int s = 0; s < slices; ++s) {
            const int r0 = p->rowStart[s], nr = p->rowStart[s + 1] - r0;
            rebase_rows_kernel<<<grid_for(nr + 1, 256) > 4096 ? 4096 : grid_for(nr + 1, 256), 256, 0, hs>>>(
                rowPtr, r0, nr, p->rebased + off);
            MXS_LAUNCH_CHECK();
            MXS_CUDA(cudaStreamSynchronize(hs));
            spmv_plan_t q = nullptr;
            const int n0 = nnzAt[s], ns = nnzAt[s + 1] - n0;
            MXS_TRY(spmv_plan_create(h, p->type, nr, C, ns, p->rebased + off, colIdx + n0,
                                     static_cast<const char*>(values) + vs * (size_t)n0, &p->variant, &q));
            p->plans.push_back(q);
            size_t ws = 0;
            spmv_plan_get_workspace_bytes(q, &ws);
            p->deviceBytes += ws;
            off += (size_t)nr + 1;
        }
    }

    // Device x / y per slot and the events that order the slots.
    const size_t xb = ((vs * (size_t)C) + 255) & ~size_t(255), yb = ((vs * (size_t)R) + 255) & ~size_t(255);
    if (xb) MXS_CUDA(dev_malloc(&p->xbuf, xb * p->depth));
    if (yb) MXS_CUDA(dev_malloc(&p->ybuf, yb * p->depth));
    p->deviceBytes += (xb + yb) * p->depth;
    auto mk = [](cudaEvent_t* e) { return cudaEventCreateWithFlags(e, cudaEventDisableTiming); };
    p->evIn.assign(p->depth, nullptr);
    p->evOut.assign(p->depth, nullptr);
    p->evSlice.assign((size_t)p->depth * (slices > 0 ? slices : 1), nullptr);
    for (auto v : {&p->evIn, &p->evOut, &p->evSlice})
        for (cudaEvent_t& e : *v) MXS_CUDA(mk(&e));
    MXS_CUDA(mk(&p->evOrder));
    for (cudaEvent_t& e : p->evJoin) MXS_CUDA(mk(&e));
    return SPMV_SUCCESS;
}

template <typename T>
static spmv_status_t pipeline_submit(spmv_pipeline_t p, T alpha, const T* hx, T beta, T* hy) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline is NULL");
    const spmv_type_t want = sizeof(T) == 4 ? SPMV_TYPE_FLOAT : SPMV_TYPE_DOUBLE;
    if (p->type != want) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "pipeline value type does not match the call");
    if (p->numRows > 0 && !hy) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y is NULL");
    if (p->numCols > 0 && p->nnz > 0 && !hx) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x is NULL");
    const int R = p->numRows, C = p->numCols;
    if (R == 0) return SPMV_SUCCESS;
    const int slices = (int)p->plans.size();
    const int b = (int)(p->submitted % p->depth);
    const size_t xb = ((sizeof(T) * (size_t)C) + 255) & ~size_t(255), yb = ((sizeof(T) * (size_t)R) + 255) & ~size_t(255);
    T* dx = reinterpret_cast<T*>(p->xbuf + xb * b);
    T* dy = reinterpret_cast<T*>(p->ybuf + yb * b);
    cudaEvent_t* evS = &p->evSlice[(size_t)b * slices];
    const bool readY = beta != T(0);

    // x slot b is free once the request that used it last has finished its
    // slices (the last slice on each compute stream); y slot b once its copy
    // out has finished.
    if (p->submitted >= p->depth) {
        for (int s = std::max(0, slices - 2); s < slices; ++s) MXS_CUDA(cudaStreamWaitEvent(p->sIn, evS[s], 0));
        if (readY) MXS_CUDA(cudaStreamWaitEvent(p->sIn, p->evOut[b], 0));
    }
    if (C > 0 && p->nnz > 0) MXS_CUDA(cudaMemcpyAsync(dx, hx, sizeof(T) * (size_t)C, cudaMemcpyHostToDevice, p->sIn));
    if (readY) MXS_CUDA(cudaMemcpyAsync(dy, hy, sizeof(T) * (size_t)R, cudaMemcpyHostToDevice, p->sIn));
    MXS_CUDA(cudaEventRecord(p->evIn[b], p->sIn));
    for (int c = 0; c < 2; ++c) {
        MXS_CUDA(cudaStreamWaitEvent(p->sComp[c], p->evIn[b], 0));
        if (p->submitted >= p->depth) MXS_CUDA(cudaStreamWaitEvent(p->sComp[c], p->evOut[b], 0));
    }
    for (int s = 0; s < slices; ++s) {
        const int r0 = p->rowStart[s], r1 = p->rowStart[s + 1];
        const cudaStream_t cs = p->sComp[s & 1];
        MXS_TRY(plan_exec_stream<T>(p->plans[s], alpha, dx, beta, dy + r0, cs));
        MXS_CUDA(cudaEventRecord(evS[s], cs));
        MXS_CUDA(cudaStreamWaitEvent(p->sOut, evS[s], 0));
        MXS_CUDA(cudaMemcpyAsync(hy + r0, dy + r0, sizeof(T) * (size_t)(r1 - r0), cudaMemcpyDeviceToHost, p->sOut));
    }
    MXS_CUDA(cudaEventRecord(p->evOut[b], p->sOut));
    ++p->submitted;
    return SPMV_SUCCESS;
}

extern "C" {

spmv_status_t spmv_pipeline_create(spmv_handle_t* h, spmv_type_t type, int numRows, int numCols, int nnz,
                                   const int* rowPtr, const int* colIdx, const void* values,
                                   const spmv_variant_t* variant, int slices, int depth, spmv_pipeline_t* out) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline pointer is NULL");
    *out = nullptr;
    if (type != SPMV_TYPE_FLOAT && type != SPMV_TYPE_DOUBLE)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "only SPMV_TYPE_FLOAT and SPMV_TYPE_DOUBLE are supported");
    if (numRows < 0 || numCols < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (numRows > 0 && !rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (nnz > 0 && (!colIdx || !values)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx/values is NULL");
    if (slices <= 0) slices = 1;
    if (depth <= 0) depth = 2;
    if (slices > 256) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "slices must be in [1, 256] (got %d)", slices);
    if (depth > 8) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "depth must be in [1, 8] (got %d)", depth);
    spmv_pipeline_s* p = new (std::nothrow) spmv_pipeline_s();
    if (!p) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    p->type = type;
    p->numRows = numRows;
    p->numCols = numCols;
    p->nnz = nnz;
    p->depth = depth;
    const spmv_status_t st = pipeline_build(h, p, rowPtr, colIdx, values, variant, slices);
    if (st != SPMV_SUCCESS) {
        pipeline_free(p);
        return st;
    }
    *out = p;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_pipeline_destroy(spmv_pipeline_t p) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline is NULL");
    pipeline_free(p);
    return SPMV_SUCCESS;
}

spmv_status_t spmv_pipeline_submit_f32(spmv_pipeline_t p, float alpha, const float* hx, float beta, float* hy) {
    return pipeline_submit<float>(p, alpha, hx, beta, hy);
}
spmv_status_t spmv_pipeline_submit_f64(spmv_pipeline_t p, double alpha, const double* hx, double beta, double* hy) {
    return pipeline_submit<double>(p, alpha, hx, beta, hy);
}

spmv_status_t spmv_pipeline_wait(spmv_pipeline_t p) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline is NULL");
    for (cudaStream_t s : {p->sIn, p->sComp[0], p->sComp[1], p->sOut}) MXS_CUDA(cudaStreamSynchronize(s));
    for (spmv_plan_t q : p->plans) {
        int code = 0;
        MXS_TRY(spmv_plan_device_error(q, &code));
    }
    return SPMV_SUCCESS;
}

spmv_status_t spmv_pipeline_order_after(spmv_pipeline_t p, cudaStream_t s) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline is NULL");
    MXS_CUDA(cudaEventRecord(p->evOrder, s));
    for (cudaStream_t q : {p->sIn, p->sComp[0], p->sComp[1], p->sOut}) MXS_CUDA(cudaStreamWaitEvent(q, p->evOrder, 0));
    return SPMV_SUCCESS;
}

spmv_status_t spmv_pipeline_join(spmv_pipeline_t p, cudaStream_t s) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline is NULL");
    int i = 0;
    for (cudaStream_t q : {p->sIn, p->sComp[0], p->sComp[1], p->sOut}) {
        MXS_CUDA(cudaEventRecord(p->evJoin[i], q));
        MXS_CUDA(cudaStreamWaitEvent(s, p->evJoin[i], 0));
        ++i;
    }
    return SPMV_SUCCESS;
}

spmv_status_t spmv_pipeline_info(spmv_pipeline_t p, int* slices, int* depth, spmv_variant_t* variant,
                                 size_t* deviceBytes, int* launchesPerRequest) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "pipeline is NULL");
    if (slices) *slices = (int)p->plans.size();
    if (depth) *depth = p->depth;
    if (variant) *variant = p->variant;
    if (deviceBytes) *deviceBytes = p->deviceBytes;
    if (launchesPerRequest) {
        int n = 0;
        for (spmv_plan_t q : p->plans) {
            spmv_variant_t v{};
            spmv_plan_get_variant(q, &v);
            n += (v.kernel == SPMV_KERNEL_MERGE || v.kernel == SPMV_KERNEL_CSR5 || v.kernel == SPMV_KERNEL_BAND ||
                  v.kernel == SPMV_KERNEL_STREAM) ? 2 : 1;
        }
        *launchesPerRequest = n;
    }
    return SPMV_SUCCESS;
}

}  // extern "C"
