/*
 * oracle.h -- CPU restatement of the muxi_spmv hot path.  TEST
 * INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline call it as the checker or as the timed CPU path.  The library never
 * links or calls it.
 *
 * Each function names the reference file:line it restates (paths inside the
 * muxi_spmv project).  oracle/ref/ builds the reference's own functions from
 * their sources, and tests/test_oracle_pins.py checks this restatement against
 * them.
 */
#ifndef MUXI_SPMV_ORACLE_H_
#define MUXI_SPMV_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y_ref[r] = sum_j values[j]*x[col[j]] for each row, in FP64 with
 * compensated (Neumaier) summation of exact products (FP32 inputs: the
 * product of two floats is exact in double).  absum[r] = sum_j |a_rj x_j|,
 * the scale of the per-row error bound.  threads <= 0: all cores. */
void oracle_spmv_f32(int rows, const int* rowPtr, const int* colIdx, const float* values,
                     const float* x, double* y_ref, double* absum, int threads);
/* FP64 inputs: products and sums in double-double (TwoProduct via fma and
 * TwoSum); y_ref is the rounded double-double result. */
void oracle_spmv_f64(int rows, const int* rowPtr, const int* colIdx, const double* values,
                     const double* x, double* y_ref, double* absum, int threads);

/* The reference's CPU CSR loop (tests/deep_analysis.cu:189-195,
 * tests/deep_analysis_runner.cpp:184-190): float sum += values*x in row
 * order.  threads == 1 is the reference's serial loop; threads > 1 splits
 * rows into contiguous blocks across threads (its OpenMP-style
 * row-parallel form).  Returns nothing; y is FP32. */
void oracle_cpu_spmv_f32(int rows, const int* rowPtr, const int* colIdx, const float* values,
                         const float* x, float* y, int threads);
void oracle_cpu_spmv_f64(int rows, const int* rowPtr, const int* colIdx, const double* values,
                         const double* x, double* y, int threads);

/* csr5_compute_tile_boundaries_kernel (src/spmv/csr5/spmv_csr5.cu:36-58)
 * with csr5_binary_search_row (src/spmv/csr5/spmv_csr5.cuh:44-61):
 * for tile t, start = t*sigma, row = last r in [0,rows) with rowPtr[r] <=
 * start, offset = start - rowPtr[row]. numTiles = ceil(nnz/sigma). */
void oracle_csr5_tiles(int rows, int nnz, const int* rowPtr, int sigma, int* tile_row_ptr,
                       int* tile_nnz_offset);

/* compute_merge_partitions_kernel (spmv_csr5.cu:912-925):
 * pos[t] = min(t*ceil(L/P), L), t = 0..P, L = rows+nnz. */
void oracle_merge_partitions(int rows, int nnz, int P, int* pos);
/* merge_path_search (spmv_csr5.cu:497-533), the three-way binary search. */
void oracle_merge_search(const int* rowPtr, int rows, int nnz, const int* diag, int count, int* rowIdx,
                         int* nnzIdx);
/* Partition count of spmv_merge_based for warp 32 (spmv_csr5.cu:941-972). */
int oracle_merge_default_partitions(int rows, int nnz);

/* csr_to_ellpack (src/spmv/ellpack/spmv_ellpack.cu:11-70): width W (0 =
 * max row length), column-major slot row + i*rows, padding col -1 / val 0.
 * Rows longer than W are truncated as the reference does; the return value
 * is the number of truncated rows.  *width_out = W. */
long long oracle_csr_to_ell_f32(int rows, const int* rowPtr, const int* colIdx, const float* values,
                                int width, int* width_out, int* ellCol, float* ellVal);
long long oracle_csr_to_ell_f64(int rows, const int* rowPtr, const int* colIdx, const double* values,
                                int width, int* width_out, int* ellCol, double* ellVal);
/* Max row length (the width csr_to_ellpack auto-detects, spmv_ellpack.cu:17-24). */
int oracle_max_row_length(int rows, const int* rowPtr);

/* reorderMatrixByRowLength (tests/test_row_reordering.cu:99-143):
 * std::stable_sort of row ids by length ascending; rowMap[new] = old;
 * rows copied in that order. */
void oracle_row_reorder_f32(int rows, const int* rowPtr, const int* colIdx, const float* values,
                            int* rowMap, int* newRowPtr, int* newColIdx, float* newValues);
/* restoreOrder (tests/test_combined_optimizations.cu:176-181):
 * y[rowMap[i]] = y_perm[i]. */
void oracle_restore_order_f32(int rows, const float* y_perm, const int* rowMap, float* y);

/* reorderColumns (src/preprocessing/column_reorder.cuh:42-141), steps 1-3:
 * key[c] = float sum of the rows touching c (in row order) / count
 * (0 for untouched columns); forwardMap = column ids sorted by (key, id).
 * key_out may be NULL. */
void oracle_colperm_center_of_mass(int rows, int cols, const int* rowPtr, const int* colIdx,
                                   int* forwardMap, float* key_out);
/* reorderColumnsRCM (tests/test_column_reordering.cu:156-199): key[c] =
 * min row touching c (rows if none); columns sorted by key ascending.  The
 * reference uses std::sort (tie order unspecified); ties here are broken by
 * ascending column id. */
void oracle_colperm_min_row(int rows, int cols, const int* rowPtr, const int* colIdx, int* perm,
                            int* key_out);
/* reorderColumnsByFrequency (test_column_reordering.cu:116-154): count of
 * nonzeros per column, sorted descending; ties by ascending column id. */
void oracle_colperm_frequency(int cols, int nnz, const int* colIdx, int* perm, int* key_out);
/* newCol[j] = inv[colIdx[j]] where inv[perm[i]] = i (column_reorder.cuh:
 * 95-118, test_column_reordering.cu:144-153). */
void oracle_apply_colperm(int cols, int nnz, const int* perm, const int* colIdx, int* newColIdx);
/* reorderXVector (column_reorder.cuh:150-161): xr[i] = x[forwardMap[i]]. */
void oracle_permute_x_f32(int cols, const int* forwardMap, const float* x, float* xr);
/* sortColumnsWithinRows (column_reorder.cuh:175-201): each row's
 * (col, value) pairs sorted by col, then value (pair ordering). In place. */
void oracle_sort_within_rows_f32(int rows, const int* rowPtr, int* colIdx, float* values);

/* Number of distinct columns in colIdx. */
long long oracle_distinct_columns(int cols, long long nnz, const int* colIdx);

#ifdef __cplusplus
}
#endif
#endif
