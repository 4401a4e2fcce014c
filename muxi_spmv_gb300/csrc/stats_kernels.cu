// Matrix statistics on the device: distinct columns (for the x-gather term of
// the algorithmic byte count) and CSR validation (rowPtr monotone, bounds).
#include "internal.h"
#include "device.cuh"
#include "kernels.h"

namespace mxs {

__global__ void mark_columns_kernel(long long nnz, const int* __restrict__ colIdx, unsigned* __restrict__ bits,
                                    int numCols) {
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nnz;
         j += (long long)gridDim.x * blockDim.x) {
        const int c = colIdx[j];
        if (c >= 0 && c < numCols) atomicOr(bits + (c >> 5), 1u << (c & 31));
    }
}

__global__ void popcount_kernel(long long words, const unsigned* __restrict__ bits,
                                unsigned long long* __restrict__ total) {
    unsigned long long local = 0;
    for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
         w += (long long)gridDim.x * blockDim.x)
        local += __popc(bits[w]);
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(kFull, local, off);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(total, local);
}

spmv_status_t count_distinct_columns(int numCols, int nnz, const int* colIdx, long long* out,
                                     cudaStream_t s) {
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    *out = 0;
    if (numCols <= 0 || nnz <= 0) return SPMV_SUCCESS;
    if (!colIdx) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx is NULL");
    const long long words = ((long long)numCols + 31) / 32;
    const long long padded = words + (words & 1);  // keeps the 8-byte counter aligned
    const size_t bytes = sizeof(unsigned) * padded + sizeof(unsigned long long);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, bytes, s));
    unsigned* bits = static_cast<unsigned*>(buf);
    unsigned long long* total = reinterpret_cast<unsigned long long*>(bits + padded);
    cudaError_t e = cudaMemsetAsync(buf, 0, bytes, s);
    if (e != cudaSuccess) {
        scratch_free(buf, s);
        return cuda_fail(e, "memset", __FILE__, __LINE__);
    }
    const unsigned g = grid_for(nnz, 256);
    mark_columns_kernel<<<g < 4096u ? g : 4096u, 256, 0, s>>>(nnz, colIdx, bits, numCols);
    const unsigned g2 = grid_for(words, 256);
    popcount_kernel<<<g2 < 1024u ? g2 : 1024u, 256, 0, s>>>(words, bits, total);
    unsigned long long h = 0;
    e = cudaMemcpyAsync(&h, total, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "distinct columns", __FILE__, __LINE__);
    *out = (long long)h;
    return SPMV_SUCCESS;
}

__global__ void validate_kernel(int numRows, int numCols, long long nnz, const int* __restrict__ rowPtr,
                                const int* __restrict__ colIdx, unsigned long long* __restrict__ bad) {
    unsigned long long local = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long r = t0; r <= numRows; r += stride) {
        const int v = rowPtr[r];
        if (r == 0 && v != 0) ++local;
        if (r == numRows && v != nnz) ++local;
        if (r < numRows && rowPtr[r + 1] < v) ++local;
    }
    // Column checks only make sense when rowPtr bounds are sane; they read
    // colIdx[0..nnz) which the caller declared as the array length.
    for (long long j = t0; j < nnz; j += stride) {
        const int c = colIdx[j];
        if (c < 0 || c >= numCols) ++local;
    }
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(kFull, local, off);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(bad, local);
}

spmv_status_t validate_csr(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                           long long* bad, cudaStream_t s) {
    if (!bad) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "bad is NULL");
    *bad = 0;
    if (numRows < 0 || numCols < 0 || nnz < 0) {
        *bad = 1;
        return SPMV_SUCCESS;
    }
    if (!rowPtr || (nnz > 0 && !colIdx)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR array");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned long long), s));
    unsigned long long* d = static_cast<unsigned long long*>(buf);
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(*d), s);
    if (e == cudaSuccess) {
        const long long work = (long long)numRows + 1 > nnz ? (long long)numRows + 1 : nnz;
        const unsigned g = grid_for(work, 256);
        validate_kernel<<<g < 4096u ? g : 4096u, 256, 0, s>>>(numRows, numCols, nnz, rowPtr, colIdx, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "validate", __FILE__, __LINE__);
    *bad = (long long)h;
    return SPMV_SUCCESS;
}

}  // namespace mxs
