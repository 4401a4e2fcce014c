// BSR (block sparse row) format: conversion from CSR on the device and SpMV.
//
// The reference declares BSRMatrix<T, BlockSize> (src/formats/sparse_formats.h:
// 207-269) -- block row pointers, block column indices and dense BxB blocks --
// without a conversion or a kernel.  Here:
//   * conversion: a thread per block row merges its B rows' (sorted) column
//     lists into the distinct block columns (counted, scanned, then written),
//     and a thread per row adds its nonzeros into the blocks (row r writes only
//     row r % B of each block, so no two threads touch one value; duplicate
//     (row, column) entries of a row add in row order);
//   * SpMV: a warp per block row, lanes over the elements of one or more
//     blocks (coalesced block values, the B x values of a block column in one
//     sector), per-lane sums over the row's blocks, then fixed butterfly
//     reductions -- deterministic, no atomics.
// Blocks are row-major; block columns past numCols hold zeros and their x
// reads are skipped.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "sort.h"

namespace mxs {

// Distinct block columns of block row br (count when out == nullptr).
__device__ __forceinline__ int bsr_merge_row(const int* __restrict__ rowPtr, const int* __restrict__ colIdx, int R,
                                             int B, int br, int* __restrict__ out) {
    int pos[8], end[8];
    const int r0 = br * B;
    const int nr = min(B, R - r0);
    for (int i = 0; i < nr; ++i) {
        pos[i] = rowPtr[r0 + i];
        end[i] = rowPtr[r0 + i + 1];
    }
    int n = 0, last = -1;
    while (true) {
        int best = 0x7fffffff;
        for (int i = 0; i < nr; ++i)
            if (pos[i] < end[i]) best = min(best, colIdx[pos[i]] / B);
        if (best == 0x7fffffff) break;
        if (best != last) {
            if (out) out[n] = best;
            ++n;
            last = best;
        }
        for (int i = 0; i < nr; ++i)  // consume every entry of this block column
            while (pos[i] < end[i] && colIdx[pos[i]] / B == best) ++pos[i];
    }
    return n;
}

__global__ void bsr_count_kernel(const int* __restrict__ rowPtr, const int* __restrict__ colIdx, int R, int B,
                                 int nbr, unsigned* __restrict__ cnt) {
    const long long br = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (br < nbr) cnt[br] = (unsigned)bsr_merge_row(rowPtr, colIdx, R, B, (int)br, nullptr);
}

__global__ void bsr_cols_kernel(const int* __restrict__ rowPtr, const int* __restrict__ colIdx, int R, int B,
                                int nbr, const int* __restrict__ bRowPtr, int* __restrict__ bColIdx) {
    const long long br = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (br < nbr) bsr_merge_row(rowPtr, colIdx, R, B, (int)br, bColIdx + bRowPtr[br]);
}

template <typename T>
__global__ void bsr_fill_kernel(const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                                const T* __restrict__ values, int R, int B, const int* __restrict__ bRowPtr,
                                const int* __restrict__ bColIdx, T* __restrict__ bValues) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const int br = (int)(r / B), i = (int)(r % B);
    const int b0 = bRowPtr[br], b1 = bRowPtr[br + 1];
    int lo = b0;  // the row's columns are sorted: its blocks are found in order
    for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) {
        const int c = colIdx[j], bc = c / B;
        while (lo < b1 && bColIdx[lo] < bc) ++lo;
        bValues[((size_t)lo * B + i) * B + (c % B)] += values[j];
    }
}

__global__ void rows_sorted_kernel(const int* __restrict__ rowPtr, const int* __restrict__ colIdx, int R,
                                   unsigned* __restrict__ bad) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    for (int j = rowPtr[r] + 1; j < rowPtr[r + 1]; ++j)
        if (colIdx[j] < colIdx[j - 1]) {
            atomicAdd(bad, 1u);
            return;
        }
}

// y = alpha*A*x + beta*y.  EB = B*B elements per block; a warp step covers
// SLOTS = 32/EB blocks (EB <= 32) or one block in EB/32 steps (B = 8).
template <typename T, int B>
__global__ void __launch_bounds__(256)
bsr_kernel(int R, int C, int nbr, const int* __restrict__ bRowPtr, const int* __restrict__ bColIdx,
           const T* __restrict__ bValues, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta, int betaZero) {
    constexpr int EB = B * B;
    constexpr int SLOTS = EB <= 32 ? 32 / EB : 1;
    constexpr int PER = EB <= 32 ? 1 : EB / 32;  // elements per lane and block
    const long long br = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (br >= nbr) return;  // uniform per warp
    const int lane = threadIdx.x & 31;
    const int b0 = bRowPtr[br], b1 = bRowPtr[br + 1];
    T acc[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) acc[q] = T(0);
    static_assert(B == 2 || B == 4 || B == 8, "32 lanes cover whole blocks");
    const int slot = EB <= 32 ? lane / EB : 0;
    const int e0 = EB <= 32 ? lane % EB : lane;  // element of the block (row-major)
    // Four block steps at a time: their loads and gathers are in flight together.
    constexpr int U = 4;
    int b = b0 + slot;
    for (; b + (U - 1) * SLOTS < b1; b += U * SLOTS) {
        int bc[U];
        T v[U][PER], g[U][PER];
#pragma unroll
        for (int u = 0; u < U; ++u) bc[u] = __ldg(bColIdx + b + u * SLOTS);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < PER; ++q) v[u][q] = ld_stream(bValues + (size_t)(b + u * SLOTS) * EB + e0 + 32 * q);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int col = bc[u] * B + (e0 + 32 * q) % B;
                g[u][q] = ld_x(x + (col < C ? col : 0));  // padding columns past C hold zeros
            }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int col = bc[u] * B + (e0 + 32 * q) % B;
                acc[q] += col < C ? v[u][q] * g[u][q] : T(0);
            }
    }
    for (; b < b1; b += SLOTS) {
        const int bc = __ldg(bColIdx + b);
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int e = e0 + 32 * q;
            const int col = bc * B + e % B;
            const T v = ld_stream(bValues + (size_t)b * EB + e);
            const T g = ld_x(x + (col < C ? col : 0));
            acc[q] += col < C ? v * g : T(0);
        }
    }
    // Reduce the B columns of each block row, then the slots: fixed order.
#pragma unroll
    for (int q = 0; q < PER; ++q) {
#pragma unroll
        for (int off = 1; off < B; off <<= 1) acc[q] += __shfl_xor_sync(kFull, acc[q], off);
        if (EB <= 32) {
#pragma unroll
            for (int off = EB; off < 32; off <<= 1) acc[q] += __shfl_xor_sync(kFull, acc[q], off);
        }
    }
    // Lanes with column 0 of slot 0 hold the row sums.
    if ((EB <= 32 ? slot == 0 : true) && e0 % B == 0) {
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const long long r = br * B + (e0 + 32 * q) / B;
            if (r < R) y[r] = axpby(alpha, acc[q], beta, betaZero != 0, y + r);
        }
    }
}

template <typename T>
static spmv_status_t run_bsr(int R, int C, int B, int nbr, const int* bRowPtr, const int* bColIdx, const T* bValues,
                             const T* x, T* y, T alpha, T beta, cudaStream_t s) {
    const unsigned g = grid_for((long long)nbr * 32, 256);
    const int bz = beta == T(0) ? 1 : 0;
    switch (B) {
        case 2: bsr_kernel<T, 2><<<g, 256, 0, s>>>(R, C, nbr, bRowPtr, bColIdx, bValues, x, y, alpha, beta, bz); break;
        case 4: bsr_kernel<T, 4><<<g, 256, 0, s>>>(R, C, nbr, bRowPtr, bColIdx, bValues, x, y, alpha, beta, bz); break;
        case 8: bsr_kernel<T, 8><<<g, 256, 0, s>>>(R, C, nbr, bRowPtr, bColIdx, bValues, x, y, alpha, beta, bz); break;
        default: MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "BSR block size must be 2, 4 or 8 (got %d)", B);
    }
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

static spmv_status_t bsr_args(int R, int C, int N, const int* rowPtr, const int* colIdx, int B) {
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (B != 2 && B != 4 && B != 8) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "BSR block size must be 2, 4 or 8");
    if (R > 0 && !rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (N > 0 && !colIdx) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx is NULL");
    return SPMV_SUCCESS;
}

}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_csr_to_bsr_count(int R, int C, int N, const int* rowPtr, const int* colIdx, int B, int* bRowPtr,
                                    int* numBlocks, cudaStream_t s) {
    clear_error();
    MXS_TRY(bsr_args(R, C, N, rowPtr, colIdx, B));
    if (!bRowPtr || !numBlocks) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "bRowPtr / numBlocks is NULL");
    const int nbr = (R + B - 1) / B;
    *numBlocks = 0;
    if (nbr == 0) {
        MXS_CUDA(cudaMemsetAsync(bRowPtr, 0, sizeof(int), s));
        return SPMV_SUCCESS;
    }
    void* buf = nullptr;
    const size_t a = (sizeof(unsigned) * ((size_t)nbr + 1) + 255) & ~size_t(255);
    MXS_TRY(scratch_alloc(&buf, a + 256, s));
    unsigned* cnt = static_cast<unsigned*>(buf);
    unsigned* flags = reinterpret_cast<unsigned*>(static_cast<char*>(buf) + a);
    unsigned hbad = 0, total = 0;
    cudaError_t e = cudaMemsetAsync(flags, 0, 2 * sizeof(unsigned), s);
    if (e == cudaSuccess) {
        rows_sorted_kernel<<<grid_for(R, 256), 256, 0, s>>>(rowPtr, colIdx, R, flags);
        bsr_count_kernel<<<grid_for(nbr, 128), 128, 0, s>>>(rowPtr, colIdx, R, B, nbr, cnt);
        e = cudaGetLastError();
    }
    spmv_status_t st = e == cudaSuccess ? SPMV_SUCCESS : cuda_fail(e, "BSR count", __FILE__, __LINE__);
    if (st == SPMV_SUCCESS) {
        e = cudaMemsetAsync(cnt + nbr, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) st = cuda_fail(e, "BSR count", __FILE__, __LINE__);
    }
    if (st == SPMV_SUCCESS)
        st = scan_exclusive_u32(cnt, reinterpret_cast<unsigned*>(bRowPtr), (long long)nbr + 1, flags + 1, s);
    if (st == SPMV_SUCCESS) {
        e = cudaMemcpyAsync(&hbad, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&total, flags + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "BSR count", __FILE__, __LINE__);
    }
    scratch_free(buf, s);
    MXS_TRY(st);
    if (hbad) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%u rows have unsorted columns (spmv_sort_columns_within_rows)", hbad);
    *numBlocks = (int)total;
    return SPMV_SUCCESS;
}

}  // extern "C"

namespace mxs {
template <typename T>
static spmv_status_t csr_to_bsr(int R, int C, int N, const int* rowPtr, const int* colIdx, const T* values, int B,
                                const int* bRowPtr, int* bColIdx, T* bValues, cudaStream_t s) {
    clear_error();
    MXS_TRY(bsr_args(R, C, N, rowPtr, colIdx, B));
    const int nbr = (R + B - 1) / B;
    if (nbr == 0 || N == 0) return SPMV_SUCCESS;
    if (!bRowPtr || !bColIdx || !bValues || !values) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL BSR array");
    int nb = 0;
    MXS_CUDA(cudaMemcpyAsync(&nb, bRowPtr + nbr, sizeof(int), cudaMemcpyDeviceToHost, s));
    MXS_CUDA(cudaStreamSynchronize(s));
    MXS_CUDA(cudaMemsetAsync(bValues, 0, sizeof(T) * (size_t)nb * B * B, s));
    bsr_cols_kernel<<<grid_for(nbr, 128), 128, 0, s>>>(rowPtr, colIdx, R, B, nbr, bRowPtr, bColIdx);
    bsr_fill_kernel<T><<<grid_for(R, 256), 256, 0, s>>>(rowPtr, colIdx, values, R, B, bRowPtr, bColIdx, bValues);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

template <typename T>
static spmv_status_t bsr_exec(int R, int C, int B, int nbr, const int* bRowPtr, const int* bColIdx,
                              const T* bValues, const T* x, T* y, T alpha, T beta, cudaStream_t s) {
    clear_error();
    if (R < 0 || C < 0 || nbr < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (nbr != (R + B - 1) / (B > 0 ? B : 1)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "numBlockRows != ceil(R / B)");
    if (R > 0 && (!y || !bRowPtr)) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y / bRowPtr is NULL");
    if (R == 0) return SPMV_SUCCESS;
    return run_bsr<T>(R, C, B, nbr, bRowPtr, bColIdx, bValues, x, y, alpha, beta, s);
}
}  // namespace mxs

extern "C" {

spmv_status_t spmv_csr_to_bsr_f32(int R, int C, int N, const int* rowPtr, const int* colIdx, const float* values,
                                  int B, const int* bRowPtr, int* bColIdx, float* bValues, cudaStream_t stream) {
    return csr_to_bsr<float>(R, C, N, rowPtr, colIdx, values, B, bRowPtr, bColIdx, bValues, stream);
}
spmv_status_t spmv_csr_to_bsr_f64(int R, int C, int N, const int* rowPtr, const int* colIdx, const double* values,
                                  int B, const int* bRowPtr, int* bColIdx, double* bValues, cudaStream_t stream) {
    return csr_to_bsr<double>(R, C, N, rowPtr, colIdx, values, B, bRowPtr, bColIdx, bValues, stream);
}
spmv_status_t spmv_bsr_f32(int R, int C, int B, int numBlockRows, const int* bRowPtr, const int* bColIdx,
                           const float* bValues, const float* x, float* y, float alpha, float beta,
                           cudaStream_t stream) {
    return bsr_exec<float>(R, C, B, numBlockRows, bRowPtr, bColIdx, bValues, x, y, alpha, beta, stream);
}
spmv_status_t spmv_bsr_f64(int R, int C, int B, int numBlockRows, const int* bRowPtr, const int* bColIdx,
                           const double* bValues, const double* x, double* y, double alpha, double beta,
                           cudaStream_t stream) {
    return bsr_exec<double>(R, C, B, numBlockRows, bRowPtr, bColIdx, bValues, x, y, alpha, beta, stream);
}

}  // extern "C"
