// Format conversion and reordering on the GPU.  Each index output is
// bit-exact with the reference function named beside it (paths inside the
// muxi_spmv project); the reference runs all of these serially on the host.
//
//   csr5 tiles        csr5_compute_tile_boundaries_kernel, spmv_csr5.cu:36-58
//   ELL conversion    csr_to_ellpack, spmv_ellpack.cu:11-70
//   row reorder       reorderMatrixByRowLength, tests/test_row_reordering.cu:99-143
//   restore order     restoreOrder, tests/test_combined_optimizations.cu:176-181
//   column orders     reorderColumns (centre of mass), column_reorder.cuh:42-141;
//                     reorderColumnsRCM / ByFrequency, test_column_reordering.cu:116-199
//   x permutation     reorderXVector, column_reorder.cuh:150-161
//   in-row sort       sortColumnsWithinRows, column_reorder.cuh:175-201
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "preprocess.h"
#include "sort.h"

namespace mxs {

// ---------------------------------------------------------------------------
// CSR5 tile metadata
// ---------------------------------------------------------------------------
__global__ void csr5_tiles_kernel(const int* __restrict__ rowPtr, int numRows, int sigma, long long tiles,
                                  int* __restrict__ tileRow, int* __restrict__ tileOff) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    const long long start = t * sigma;
    const int r = row_of_nnz(rowPtr, numRows, start);
    tileRow[t] = r;
    if (tileOff) tileOff[t] = (int)(start - rowPtr[r]);
}

spmv_status_t csr5_tiles(const int* rowPtr, int numRows, int nnz, int sigma, int* tileRow, int* tileOff,
                         cudaStream_t s) {
    if (sigma <= 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "sigma must be positive");
    const long long tiles = ((long long)nnz + sigma - 1) / sigma;
    if (tiles == 0) return SPMV_SUCCESS;
    if (!rowPtr || numRows <= 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL or no rows");
    if (!tileRow) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "tile row array is NULL");  // tileOff may be NULL
    csr5_tiles_kernel<<<grid_for(tiles, 256), 256, 0, s>>>(rowPtr, numRows, sigma, tiles, tileRow, tileOff);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

// ---------------------------------------------------------------------------
// Row lengths, max row length
// ---------------------------------------------------------------------------
__global__ void row_lengths_kernel(const int* __restrict__ rowPtr, int numRows, unsigned* __restrict__ len,
                                   unsigned* __restrict__ ids, unsigned* __restrict__ maxLen) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned l = 0;
    if (r < numRows) {
        l = (unsigned)(rowPtr[r + 1] - rowPtr[r]);
        if (len) len[r] = l;
        if (ids) ids[r] = (unsigned)r;
    }
    for (int off = 16; off > 0; off >>= 1) l = max(l, __shfl_xor_sync(kFull, l, off));
    if ((threadIdx.x & 31) == 0 && maxLen) atomicMax(maxLen, l);
}

__global__ void empty_rows_kernel(const int* __restrict__ rowPtr, int numRows, unsigned long long* __restrict__ out) {
    unsigned long long n = 0;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < numRows;
         r += (long long)gridDim.x * blockDim.x)
        n += rowPtr[r] == rowPtr[r + 1];
    for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(kFull, n, off);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(out, n);
}

spmv_status_t count_empty_rows(const int* rowPtr, int numRows, long long* out, cudaStream_t s) {
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    *out = 0;
    if (numRows <= 0) return SPMV_SUCCESS;
    if (!rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned long long), s));
    unsigned long long* d = static_cast<unsigned long long*>(buf);
    unsigned long long h = 0;
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(*d), s);
    if (e == cudaSuccess) {
        const unsigned g = grid_for(numRows, 256);
        empty_rows_kernel<<<g < 4096u ? g : 4096u, 256, 0, s>>>(rowPtr, numRows, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "empty rows", __FILE__, __LINE__);
    *out = (long long)h;
    return SPMV_SUCCESS;
}

spmv_status_t max_row_length(const int* rowPtr, int numRows, int* out, cudaStream_t s) {
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    *out = 0;
    if (numRows <= 0) return SPMV_SUCCESS;
    if (!rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned), s));
    unsigned* d = static_cast<unsigned*>(buf);
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        row_lengths_kernel<<<grid_for(numRows, 256), 256, 0, s>>>(rowPtr, numRows, nullptr, nullptr, d);
        e = cudaGetLastError();
    }
    unsigned h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "max row length", __FILE__, __LINE__);
    *out = (int)h;
    return SPMV_SUCCESS;
}

// ---------------------------------------------------------------------------
// ELL conversion: slot (row r, element i) at r + i*numRows; padding -1 / 0.
// Rows longer than the width keep their first `width` entries, as the
// reference does; *truncated counts them.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void csr_to_ell_kernel(const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                                  const T* __restrict__ values, int numRows, int width, int* __restrict__ ellCol,
                                  T* __restrict__ ellVal, unsigned long long* __restrict__ truncated) {
    const long long total = (long long)numRows * width;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long i = idx / numRows;
        const int r = (int)(idx - i * numRows);
        const int s = rowPtr[r], len = rowPtr[r + 1] - s;
        if (i < len) {
            ellCol[idx] = colIdx[s + i];
            ellVal[idx] = values[s + i];
        } else {
            ellCol[idx] = -1;
            ellVal[idx] = T(0);
        }
        if (i == 0 && len > width && truncated) atomicAdd(truncated, 1ull);
    }
}

template <typename T>
spmv_status_t csr_to_ell(int numRows, const int* rowPtr, const int* colIdx, const T* values, int width,
                         int* ellCol, T* ellVal, long long* truncated, cudaStream_t s) {
    if (truncated) *truncated = 0;
    if (numRows < 0 || width < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative size");
    if (numRows == 0 || width == 0) return SPMV_SUCCESS;
    if (!rowPtr || !colIdx || !values) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR array");
    if (!ellCol || !ellVal) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL ELL array");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned long long), s));
    auto* d = static_cast<unsigned long long*>(buf);
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(*d), s);
    if (e == cudaSuccess) {
        const long long total = (long long)numRows * width;
        const unsigned g = grid_for(total, 256);
        csr_to_ell_kernel<T><<<g < 65535u * 16 ? g : 65535u * 16, 256, 0, s>>>(rowPtr, colIdx, values, numRows,
                                                                            width, ellCol, ellVal, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "csr_to_ell", __FILE__, __LINE__);
    if (truncated) *truncated = (long long)h;
    return SPMV_SUCCESS;
}
template spmv_status_t csr_to_ell<float>(int, const int*, const int*, const float*, int, int*, float*, long long*,
                                         cudaStream_t);
template spmv_status_t csr_to_ell<double>(int, const int*, const int*, const double*, int, int*, double*,
                                          long long*, cudaStream_t);

// ---------------------------------------------------------------------------
// Row reorder by length (stable) and its inverse scatter
// ---------------------------------------------------------------------------
template <typename T>
__global__ void copy_rows_kernel(int numRows, const int* __restrict__ rowMap, const int* __restrict__ rowPtr,
                                 const int* __restrict__ colIdx, const T* __restrict__ values,
                                 const int* __restrict__ newRowPtr, int* __restrict__ newCol, T* __restrict__ newVal) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= numRows) return;
    const int o = rowMap[w];
    const int s = rowPtr[o], len = rowPtr[o + 1] - s, d = newRowPtr[w];
    for (int k = lane; k < len; k += 32) {
        newCol[d + k] = colIdx[s + k];
        newVal[d + k] = values[s + k];
    }
}

template <typename T>
spmv_status_t reorder_rows_by_length(int numRows, int nnz, const int* rowPtr, const int* colIdx, const T* values,
                                     int* rowMap, int* newRowPtr, int* newCol, T* newVal, cudaStream_t s) {
    if (numRows < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative size");
    if (numRows == 0) {
        if (newRowPtr) MXS_CUDA(cudaMemsetAsync(newRowPtr, 0, sizeof(int), s));
        return SPMV_SUCCESS;
    }
    if (!rowPtr || (nnz > 0 && (!colIdx || !values))) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR array");
    if (!rowMap || !newRowPtr || (nnz > 0 && (!newCol || !newVal))) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL output");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned) * ((size_t)numRows + 1), s));
    unsigned* keys = static_cast<unsigned*>(buf);
    unsigned* maxLen = keys + numRows;
    spmv_status_t st = SPMV_SUCCESS;
    cudaError_t e = cudaMemsetAsync(maxLen, 0, sizeof(unsigned), s);
    unsigned hmax = 0;
    if (e == cudaSuccess) {
        row_lengths_kernel<<<grid_for(numRows, 256), 256, 0, s>>>(rowPtr, numRows, keys,
                                                                  reinterpret_cast<unsigned*>(rowMap), maxLen);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hmax, maxLen, sizeof(hmax), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_fail(e, "row lengths", __FILE__, __LINE__);
    if (st == SPMV_SUCCESS)
        st = radix_sort_pairs(keys, reinterpret_cast<unsigned*>(rowMap), numRows, bits_for(hmax), s);
    if (st == SPMV_SUCCESS)
        st = scan_exclusive_u32(keys, reinterpret_cast<unsigned*>(newRowPtr), numRows,
                                reinterpret_cast<unsigned*>(newRowPtr) + numRows, s);
    if (st == SPMV_SUCCESS && nnz > 0) {
        copy_rows_kernel<T><<<grid_for((long long)numRows * 32, 256), 256, 0, s>>>(numRows, rowMap, rowPtr, colIdx,
                                                                                 values, newRowPtr, newCol, newVal);
        if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
    }
    scratch_free(buf, s);
    return st;
}
template spmv_status_t reorder_rows_by_length<float>(int, int, const int*, const int*, const float*, int*, int*,
                                                     int*, float*, cudaStream_t);
template spmv_status_t reorder_rows_by_length<double>(int, int, const int*, const int*, const double*, int*, int*,
                                                      int*, double*, cudaStream_t);

template <typename T>
__global__ void restore_order_kernel(int numRows, const T* __restrict__ yPerm, const int* __restrict__ rowMap,
                                     T* __restrict__ y) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < numRows) y[rowMap[i]] = yPerm[i];
}

template <typename T>
spmv_status_t restore_order(int numRows, const T* yPerm, const int* rowMap, T* y, cudaStream_t s) {
    if (numRows <= 0) return SPMV_SUCCESS;
    if (!yPerm || !rowMap || !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    restore_order_kernel<T><<<grid_for(numRows, 256), 256, 0, s>>>(numRows, yPerm, rowMap, y);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
template spmv_status_t restore_order<float>(int, const float*, const int*, float*, cudaStream_t);
template spmv_status_t restore_order<double>(int, const double*, const int*, double*, cudaStream_t);

// ---------------------------------------------------------------------------
// Column permutations
// ---------------------------------------------------------------------------
__global__ void iota_kernel(unsigned* __restrict__ v, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (unsigned)i;
}

__global__ void fill_kernel(unsigned* __restrict__ v, long long n, unsigned value) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = value;
}

// Row id of every nonzero (warp per row).
__global__ void expand_rows_kernel(const int* __restrict__ rowPtr, int numRows, unsigned* __restrict__ rowOf) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= numRows) return;
    const int s = rowPtr[w], e = rowPtr[w + 1];
    for (int j = s + lane; j < e; j += 32) rowOf[j] = (unsigned)w;
}

__global__ void min_row_kernel(const int* __restrict__ rowPtr, int numRows, const int* __restrict__ colIdx,
                               unsigned* __restrict__ key) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= numRows) return;
    const int s = rowPtr[w], e = rowPtr[w + 1];
    for (int j = s + lane; j < e; j += 32) atomicMin(key + colIdx[j], (unsigned)w);
}

__global__ void count_cols_kernel(long long nnz, const int* __restrict__ colIdx, unsigned* __restrict__ cnt) {
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + colIdx[j], 1u);
}

__global__ void descending_key_kernel(int numCols, unsigned nnz, const unsigned* __restrict__ cnt,
                                      unsigned* __restrict__ key, int* __restrict__ keyOut) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCols) return;
    if (keyOut) keyOut[c] = (int)cnt[c];
    key[c] = nnz - cnt[c];
}

// Centre of mass of column c: float sum of the rows touching c, added in
// ascending row order (the order of the reference's row loop), divided by
// the count; 0 for untouched columns.
__global__ void center_of_mass_kernel(int numCols, const unsigned* __restrict__ colStart,
                                      const unsigned* __restrict__ rowsByCol, unsigned* __restrict__ keyBits,
                                      float* __restrict__ keyOut) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= numCols) return;
    const unsigned b = colStart[c], e = colStart[c + 1];
    float sum = 0.0f;
    for (unsigned k = b; k < e; ++k) sum = __fadd_rn(sum, __uint2float_rn(rowsByCol[k]));
    const float key = e > b ? __fdiv_rn(sum, __uint2float_rn(e - b)) : sum;
    keyBits[c] = __float_as_uint(key);  // keys are >= +0, so bit order is numeric order
    if (keyOut) keyOut[c] = key;
}

spmv_status_t column_perm(int kind, int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                          int* perm, void* keysOut, cudaStream_t s) {
    if (numRows < 0 || numCols < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative size");
    if (numCols == 0) return SPMV_SUCCESS;
    if (!perm) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "perm is NULL");
    if ((numRows > 0 && !rowPtr) || (nnz > 0 && !colIdx)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR array");
    unsigned* up = reinterpret_cast<unsigned*>(perm);
    const long long C = numCols;
    spmv_status_t st = SPMV_SUCCESS;
    if (kind == SPMV_COLPERM_MIN_ROW || kind == SPMV_COLPERM_FREQUENCY) {
        void* buf = nullptr;
        MXS_TRY(scratch_alloc(&buf, sizeof(unsigned) * C, s));
        unsigned* key = static_cast<unsigned*>(buf);
        iota_kernel<<<grid_for(C, 256), 256, 0, s>>>(up, C);
        int bits = 1;
        if (kind == SPMV_COLPERM_MIN_ROW) {
            fill_kernel<<<grid_for(C, 256), 256, 0, s>>>(key, C, (unsigned)numRows);
            if (numRows > 0)
                min_row_kernel<<<grid_for((long long)numRows * 32, 256), 256, 0, s>>>(rowPtr, numRows, colIdx, key);
            if (keysOut && cudaMemcpyAsync(keysOut, key, sizeof(unsigned) * C, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                st = SPMV_ERROR_DEVICE;
            bits = bits_for((unsigned)numRows);
        } else {
            fill_kernel<<<grid_for(C, 256), 256, 0, s>>>(key, C, 0u);
            if (nnz > 0) {
                const unsigned g = grid_for(nnz, 256);
                count_cols_kernel<<<g < 8192u ? g : 8192u, 256, 0, s>>>(nnz, colIdx, key);
            }
            descending_key_kernel<<<grid_for(C, 256), 256, 0, s>>>(numCols, (unsigned)nnz, key, key,
                                                                    static_cast<int*>(keysOut));
            bits = bits_for((unsigned)nnz);
        }
        if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
        if (st == SPMV_SUCCESS) st = radix_sort_pairs(key, up, C, bits, s);
        scratch_free(buf, s);
        return st;
    }
    if (kind != SPMV_COLPERM_CENTER_OF_MASS) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "unknown column order %d", kind);
    // Stable transpose: (col, row) pairs in row-major order sorted by col keep
    // each column's rows ascending.
    const long long N = nnz;
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned) * (2 * N + 3 * C + 2), s));
    unsigned* ck = static_cast<unsigned*>(buf);
    unsigned* rv = ck + N;
    unsigned* cnt = rv + N;
    unsigned* colStart = cnt + C;  // C + 1 entries
    unsigned* keyBits = colStart + C + 1;
    cudaError_t e = cudaSuccess;
    if (N > 0) e = cudaMemcpyAsync(ck, colIdx, sizeof(unsigned) * N, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && N > 0) {
        expand_rows_kernel<<<grid_for((long long)numRows * 32, 256), 256, 0, s>>>(rowPtr, numRows, rv);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) st = cuda_fail(e, "centre of mass setup", __FILE__, __LINE__);
    if (st == SPMV_SUCCESS && N > 0) st = radix_sort_pairs(ck, rv, N, bits_for((unsigned)(numCols - 1)), s);
    if (st == SPMV_SUCCESS) {
        fill_kernel<<<grid_for(C, 256), 256, 0, s>>>(cnt, C, 0u);
        if (N > 0) {
            const unsigned g = grid_for(N, 256);
            count_cols_kernel<<<g < 8192u ? g : 8192u, 256, 0, s>>>(N, colIdx, cnt);
        }
        if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
    }
    if (st == SPMV_SUCCESS) st = scan_exclusive_u32(cnt, colStart, C, colStart + C, s);
    if (st == SPMV_SUCCESS) {
        center_of_mass_kernel<<<grid_for(C, 256), 256, 0, s>>>(numCols, colStart, rv, keyBits,
                                                               static_cast<float*>(keysOut));
        iota_kernel<<<grid_for(C, 256), 256, 0, s>>>(up, C);
        if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
    }
    if (st == SPMV_SUCCESS) st = radix_sort_pairs(keyBits, up, C, 32, s);
    scratch_free(buf, s);
    return st;
}

__global__ void invert_kernel(int n, const int* __restrict__ perm, int* __restrict__ inv) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) inv[perm[i]] = (int)i;
}

__global__ void remap_kernel(long long nnz, const int* __restrict__ inv, const int* __restrict__ colIdx,
                             int* __restrict__ out) {
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (long long)gridDim.x * blockDim.x)
        out[j] = inv[colIdx[j]];
}

spmv_status_t apply_column_perm(int numCols, int nnz, const int* perm, const int* colIdx, int* out, cudaStream_t s) {
    if (numCols < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative size");
    if (nnz == 0) return SPMV_SUCCESS;
    if (!perm || !colIdx || !out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(int) * (size_t)numCols, s));
    int* inv = static_cast<int*>(buf);
    invert_kernel<<<grid_for(numCols, 256), 256, 0, s>>>(numCols, perm, inv);
    const unsigned g = grid_for(nnz, 256);
    remap_kernel<<<g < 16384u ? g : 16384u, 256, 0, s>>>(nnz, inv, colIdx, out);
    const cudaError_t e = cudaGetLastError();
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "apply column permutation", __FILE__, __LINE__);
    return SPMV_SUCCESS;
}

template <typename T>
__global__ void gather_kernel(int n, const int* __restrict__ perm, const T* __restrict__ x, T* __restrict__ xr) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xr[i] = x[perm[i]];
}

template <typename T>
spmv_status_t permute_x(int numCols, const int* perm, const T* x, T* xr, cudaStream_t s) {
    if (numCols <= 0) return SPMV_SUCCESS;
    if (!perm || !x || !xr) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    gather_kernel<T><<<grid_for(numCols, 256), 256, 0, s>>>(numCols, perm, x, xr);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
template spmv_status_t permute_x<float>(int, const int*, const float*, float*, cudaStream_t);
template spmv_status_t permute_x<double>(int, const int*, const double*, double*, cudaStream_t);

// ---------------------------------------------------------------------------
// In-row sort by (column, value): three stable LSD sorts of a permutation --
// by value, then column, then row -- order every row by column with ties
// broken by value, like std::sort on pair<int, T>.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned sortable(unsigned u) { return (u & 0x80000000u) ? ~u : (u | 0x80000000u); }

template <typename T>
__global__ void value_key_kernel(long long n, const unsigned* __restrict__ idx, const T* __restrict__ values,
                                 unsigned* __restrict__ key, int word) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const T v = values[idx[k]];
    if (sizeof(T) == 4) {
        key[k] = sortable(__float_as_uint((float)v));
    } else {
        const unsigned long long b = (unsigned long long)__double_as_longlong((double)v);
        const unsigned long long sb = (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
        key[k] = word == 0 ? (unsigned)sb : (unsigned)(sb >> 32);
    }
}

__global__ void gather_u32_kernel(long long n, const unsigned* __restrict__ idx, const unsigned* __restrict__ src,
                                  unsigned* __restrict__ dst) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[idx[k]];
}

template <typename T>
__global__ void apply_order_kernel(long long n, const unsigned* __restrict__ idx, const int* __restrict__ colIn,
                                   const T* __restrict__ valIn, int* __restrict__ colOut, T* __restrict__ valOut) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        colOut[k] = colIn[idx[k]];
        valOut[k] = valIn[idx[k]];
    }
}

template <typename T>
spmv_status_t sort_within_rows(int numRows, int numCols, int nnz, const int* rowPtr, int* colIdx, T* values,
                               cudaStream_t s) {
    if (numRows < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative size");
    if (nnz <= 1) return SPMV_SUCCESS;
    if (!rowPtr || !colIdx || !values) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR array");
    const long long N = nnz;
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned) * 4 * N + sizeof(T) * N, s));
    unsigned* idx = static_cast<unsigned*>(buf);
    unsigned* key = idx + N;
    unsigned* rowOf = key + N;
    int* colTmp = reinterpret_cast<int*>(rowOf + N);
    T* valTmp = reinterpret_cast<T*>(colTmp + N);
    const unsigned g = grid_for(N, 256);
    spmv_status_t st = SPMV_SUCCESS;
    iota_kernel<<<g, 256, 0, s>>>(idx, N);
    expand_rows_kernel<<<grid_for((long long)numRows * 32, 256), 256, 0, s>>>(rowPtr, numRows, rowOf);
    if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
    for (int word = 0; word < (int)(sizeof(T) / 4) && st == SPMV_SUCCESS; ++word) {
        value_key_kernel<T><<<g, 256, 0, s>>>(N, idx, values, key, word);
        st = radix_sort_pairs(key, idx, N, 32, s);
    }
    if (st == SPMV_SUCCESS) {
        gather_u32_kernel<<<g, 256, 0, s>>>(N, idx, reinterpret_cast<const unsigned*>(colIdx), key);
        st = radix_sort_pairs(key, idx, N, bits_for((unsigned)(numCols > 0 ? numCols - 1 : 0)), s);
    }
    if (st == SPMV_SUCCESS) {
        gather_u32_kernel<<<g, 256, 0, s>>>(N, idx, rowOf, key);
        st = radix_sort_pairs(key, idx, N, bits_for((unsigned)(numRows > 0 ? numRows - 1 : 0)), s);
    }
    if (st == SPMV_SUCCESS) {
        apply_order_kernel<T><<<g, 256, 0, s>>>(N, idx, colIdx, values, colTmp, valTmp);
        cudaError_t e = cudaMemcpyAsync(colIdx, colTmp, sizeof(int) * N, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(values, valTmp, sizeof(T) * N, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) st = cuda_fail(e, "in-row sort", __FILE__, __LINE__);
    }
    scratch_free(buf, s);
    return st;
}
template spmv_status_t sort_within_rows<float>(int, int, int, const int*, int*, float*, cudaStream_t);
template spmv_status_t sort_within_rows<double>(int, int, int, const int*, int*, double*, cudaStream_t);

}  // namespace mxs

namespace mxs {

// ---------------------------------------------------------------------------
// Transpose: stable radix sort of the nonzeros by column (ties keep row
// order), counts of each column scanned into the new row pointers, and a
// gather of rows and values in sorted order.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void transpose_gather_kernel(long long n, const unsigned* __restrict__ pos,
                                        const unsigned* __restrict__ rowOf, const T* __restrict__ values,
                                        int* __restrict__ tCol, T* __restrict__ tVal) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned p = pos[k];
    tCol[k] = (int)rowOf[p];
    tVal[k] = values[p];
}

template <typename T>
spmv_status_t csr_transpose(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx, const T* values,
                            int* tRowPtr, int* tColIdx, T* tValues, cudaStream_t s) {
    if (numRows < 0 || numCols < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (!tRowPtr) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "tRowPtr is NULL");
    if (nnz == 0) {
        MXS_CUDA(cudaMemsetAsync(tRowPtr, 0, sizeof(int) * ((size_t)numCols + 1), s));
        return SPMV_SUCCESS;
    }
    if (!rowPtr || !colIdx || !values || !tColIdx || !tValues) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL array");
    const size_t n = (size_t)nnz;
    const size_t a = (sizeof(unsigned) * n + 255) & ~size_t(255);
    const size_t ac = (sizeof(unsigned) * ((size_t)numCols + 1) + 255) & ~size_t(255);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, 3 * a + ac, s));
    char* b = static_cast<char*>(buf);
    unsigned* keys = reinterpret_cast<unsigned*>(b);
    unsigned* pos = reinterpret_cast<unsigned*>(b + a);
    unsigned* rowOf = reinterpret_cast<unsigned*>(b + 2 * a);
    unsigned* cnt = reinterpret_cast<unsigned*>(b + 3 * a);
    const unsigned g = grid_for(nnz, 256);
    cudaError_t e = cudaMemcpyAsync(keys, colIdx, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(unsigned) * ((size_t)numCols + 1), s);
    spmv_status_t st = e == cudaSuccess ? SPMV_SUCCESS : cuda_fail(e, "transpose", __FILE__, __LINE__);
    if (st == SPMV_SUCCESS) {
        iota_kernel<<<g, 256, 0, s>>>(pos, nnz);
        count_cols_kernel<<<g < 4096u ? g : 4096u, 256, 0, s>>>(nnz, colIdx, cnt);
        expand_rows_kernel<<<grid_for((long long)numRows * 32, 256), 256, 0, s>>>(rowPtr, numRows, rowOf);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(e, "transpose", __FILE__, __LINE__);
    }
    if (st == SPMV_SUCCESS) st = radix_sort_pairs(keys, pos, nnz, bits_for(numCols > 0 ? numCols - 1 : 0), s);
    if (st == SPMV_SUCCESS)
        st = scan_exclusive_u32(cnt, reinterpret_cast<unsigned*>(tRowPtr), numCols + 1, nullptr, s);
    if (st == SPMV_SUCCESS) {
        transpose_gather_kernel<T><<<g, 256, 0, s>>>(nnz, pos, rowOf, values, tColIdx, tValues);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(e, "transpose", __FILE__, __LINE__);
    }
    scratch_free(buf, s);
    return st;
}
template spmv_status_t csr_transpose<float>(int, int, int, const int*, const int*, const float*, int*, int*, float*,
                                            cudaStream_t);
template spmv_status_t csr_transpose<double>(int, int, int, const int*, const int*, const double*, int*, int*,
                                             double*, cudaStream_t);

// ---------------------------------------------------------------------------
// COO -> CSR: entries ordered by (row, column) with two stable radix sorts
// (column, then row; equal (row, column) pairs keep their input order), row
// counts scanned into rowPtr, and a gather of columns and values.
// ---------------------------------------------------------------------------
__global__ void count_keys_kernel(long long n, const int* __restrict__ key, unsigned* __restrict__ cnt) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + key[k], 1u);
}
__global__ void gather_keys_kernel(long long n, const unsigned* __restrict__ pos, const int* __restrict__ src,
                                   unsigned* __restrict__ dst) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (unsigned)src[pos[k]];
}
__global__ void coo_bad_kernel(long long n, const int* __restrict__ row, const int* __restrict__ col, int R, int C,
                               unsigned* __restrict__ bad) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && ((unsigned)row[k] >= (unsigned)R || (unsigned)col[k] >= (unsigned)C)) atomicAdd(bad, 1u);
}
template <typename T>
__global__ void coo_gather_kernel(long long n, const unsigned* __restrict__ pos, const int* __restrict__ col,
                                  const T* __restrict__ val, int* __restrict__ outCol, T* __restrict__ outVal) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned p = pos[k];
    outCol[k] = col[p];
    outVal[k] = val[p];
}

template <typename T>
spmv_status_t coo_to_csr(int numRows, int numCols, int nnz, const int* rowIdx, const int* colIdx, const T* values,
                         int* rowPtr, int* outCol, T* outVal, cudaStream_t s) {
    if (numRows < 0 || numCols < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (!rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "rowPtr is NULL");
    if (nnz == 0) {
        MXS_CUDA(cudaMemsetAsync(rowPtr, 0, sizeof(int) * ((size_t)numRows + 1), s));
        return SPMV_SUCCESS;
    }
    if (!rowIdx || !colIdx || !values || !outCol || !outVal) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL array");
    const size_t n = (size_t)nnz;
    const size_t a = (sizeof(unsigned) * n + 255) & ~size_t(255);
    const size_t ar = (sizeof(unsigned) * ((size_t)numRows + 1) + 255) & ~size_t(255);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, 2 * a + ar + 256, s));
    char* b = static_cast<char*>(buf);
    unsigned* keys = reinterpret_cast<unsigned*>(b);
    unsigned* pos = reinterpret_cast<unsigned*>(b + a);
    unsigned* cnt = reinterpret_cast<unsigned*>(b + 2 * a);
    unsigned* bad = reinterpret_cast<unsigned*>(b + 2 * a + ar);
    const unsigned g = grid_for(nnz, 256);
    unsigned hbad = 0;
    cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        coo_bad_kernel<<<g, 256, 0, s>>>(nnz, rowIdx, colIdx, numRows, numCols, bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    spmv_status_t st = e == cudaSuccess ? SPMV_SUCCESS : cuda_fail(e, "COO to CSR", __FILE__, __LINE__);
    if (st == SPMV_SUCCESS && hbad) {
        set_error(__FILE__, __LINE__, "%u COO entries lie outside the %d x %d matrix", hbad, numRows, numCols);
        st = SPMV_ERROR_INVALID_MATRIX;
    }
    if (st == SPMV_SUCCESS) {
        e = cudaMemcpyAsync(keys, colIdx, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(unsigned) * ((size_t)numRows + 1), s);
        if (e == cudaSuccess) {
            iota_kernel<<<g, 256, 0, s>>>(pos, nnz);
            count_keys_kernel<<<g < 4096u ? g : 4096u, 256, 0, s>>>(nnz, rowIdx, cnt);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) st = cuda_fail(e, "COO to CSR", __FILE__, __LINE__);
    }
    if (st == SPMV_SUCCESS) st = radix_sort_pairs(keys, pos, nnz, bits_for(numCols > 0 ? numCols - 1 : 0), s);
    if (st == SPMV_SUCCESS) {
        gather_keys_kernel<<<g, 256, 0, s>>>(nnz, pos, rowIdx, keys);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(e, "COO to CSR", __FILE__, __LINE__);
    }
    if (st == SPMV_SUCCESS) st = radix_sort_pairs(keys, pos, nnz, bits_for(numRows > 0 ? numRows - 1 : 0), s);
    if (st == SPMV_SUCCESS) st = scan_exclusive_u32(cnt, reinterpret_cast<unsigned*>(rowPtr), numRows + 1, nullptr, s);
    if (st == SPMV_SUCCESS) {
        coo_gather_kernel<T><<<g, 256, 0, s>>>(nnz, pos, colIdx, values, outCol, outVal);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_fail(e, "COO to CSR", __FILE__, __LINE__);
    }
    scratch_free(buf, s);
    return st;
}
template spmv_status_t coo_to_csr<float>(int, int, int, const int*, const int*, const float*, int*, int*, float*,
                                         cudaStream_t);
template spmv_status_t coo_to_csr<double>(int, int, int, const int*, const int*, const double*, int*, int*, double*,
                                          cudaStream_t);

}  // namespace mxs

