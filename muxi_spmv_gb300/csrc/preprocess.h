// Format conversion / reordering kernels (preprocess_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include "muxi_spmv.h"

namespace mxs {

spmv_status_t csr5_tiles(const int* rowPtr, int numRows, int nnz, int sigma, int* tileRow, int* tileOff,
                         cudaStream_t s);
// Host result: the longest row.
spmv_status_t max_row_length(const int* rowPtr, int numRows, int* out, cudaStream_t s);
// Number of rows without nonzeros (synchronises the stream).
spmv_status_t count_empty_rows(const int* rowPtr, int numRows, long long* out, cudaStream_t s);
template <typename T>
spmv_status_t csr_to_ell(int numRows, const int* rowPtr, const int* colIdx, const T* values, int width,
                         int* ellCol, T* ellVal, long long* truncated, cudaStream_t s);
template <typename T>
spmv_status_t reorder_rows_by_length(int numRows, int nnz, const int* rowPtr, const int* colIdx, const T* values,
                                     int* rowMap, int* newRowPtr, int* newCol, T* newVal, cudaStream_t s);
template <typename T>
spmv_status_t restore_order(int numRows, const T* yPerm, const int* rowMap, T* y, cudaStream_t s);
// kind: spmv_colperm_t.  keysOut (optional, device): float per column for
// the centre of mass, int per column otherwise.
spmv_status_t column_perm(int kind, int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                          int* perm, void* keysOut, cudaStream_t s);
spmv_status_t apply_column_perm(int numCols, int nnz, const int* perm, const int* colIdx, int* out, cudaStream_t s);
template <typename T>
spmv_status_t permute_x(int numCols, const int* perm, const T* x, T* xr, cudaStream_t s);
template <typename T>
spmv_status_t sort_within_rows(int numRows, int numCols, int nnz, const int* rowPtr, int* colIdx, T* values,
                               cudaStream_t s);
// CSR of the transpose: tRowPtr[numCols+1], tColIdx/tValues[nnz].  Rows of the
// transpose list the original rows in ascending order (stable by position).
template <typename T>
spmv_status_t csr_transpose(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx, const T* values,
                            int* tRowPtr, int* tColIdx, T* tValues, cudaStream_t s);
// CSR of a COO matrix: entries ordered by (row, column), equal pairs in input
// order (they stay separate entries, which add); entries outside the matrix
// are refused (synchronises the stream to check).
template <typename T>
spmv_status_t coo_to_csr(int numRows, int numCols, int nnz, const int* rowIdx, const int* colIdx, const T* values,
                         int* rowPtr, int* outCol, T* outVal, cudaStream_t s);

}  // namespace mxs
