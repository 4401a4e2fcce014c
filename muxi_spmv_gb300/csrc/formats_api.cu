// C ABI of the CSR5 / ELL formats and of the reorders.
#include "internal.h"
#include "formats.h"
#include "kernels.h"
#include "preprocess.h"

namespace mxs {

template <typename T>
static spmv_status_t csr5_exec(int R, int C, int N, const int* rowPtr, const int* colIdx, const T* values, int sigma,
                               const int* tileRow, const int* tileOff, const T* x, T* y, T alpha, T beta,
                               const spmv_opts_t* opts) {
    clear_error();
    (void)tileOff;  // the kernel needs only the tile start rows
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (sigma != 128 && sigma != 256 && sigma != 512)
        MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "sigma must be 128, 256 or 512 (got %d)", sigma);
    if (R > 0 && !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y is NULL");
    const cudaStream_t s = opts_stream(opts);
    if (R == 0) return SPMV_SUCCESS;
    if (N == 0) {
        MXS_TRY(run_scale<T>(R, y, beta, s));
    } else {
        if (!rowPtr || !colIdx || !values || !tileRow) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR5 array");
        if (!x) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x is NULL");
        if (N > 0x7fffffff - 32768)
            MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "CSR5 tiles need nnz <= 2^31 - 32769 (got %d)", N);
        const long long tiles = ((long long)N + sigma - 1) / sigma;
        void* buf = nullptr;
        MXS_TRY(scratch_alloc(&buf, (sizeof(int) + sizeof(T)) * tiles + 256, s));
        int* cr = static_cast<int*>(buf);
        T* cv = reinterpret_cast<T*>(static_cast<char*>(buf) + ((sizeof(int) * tiles + 255) & ~size_t(255)));
        RowsArgs<T> a{R, N, rowPtr, colIdx, values, x, y, alpha, beta, beta == T(0)};
        // Gathers in nonzero order (the ordered tile kernel, 128-thread blocks).
        spmv_status_t st = run_csr5<T>(sigma, tileRow, tiles, cr, cv, a, s, nullptr, true, 128);
        scratch_free(buf, s);
        MXS_TRY(st);
    }
    if (opts && opts->sync) MXS_CUDA(cudaStreamSynchronize(s));
    return SPMV_SUCCESS;
}

template <typename T>
static spmv_status_t ell_exec(int R, int W, const int* ellCol, const T* ellVal, const T* x, T* y, T alpha, T beta,
                              cudaStream_t s) {
    clear_error();
    if (R < 0 || W < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (R > 0 && !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y is NULL");
    if (R > 0 && W > 0 && (!ellCol || !ellVal)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL ELL array");
    if (R > 0 && W > 0 && !x) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x is NULL");
    return run_ell<T>(R, W, ellCol, ellVal, x, y, alpha, beta, s);
}

}  // namespace mxs

using namespace mxs;

extern "C" {

int spmv_csr5_default_sigma(void) { return 128; }

int spmv_csr5_num_tiles(int nnz, int sigma) {
    if (nnz <= 0 || sigma <= 0) return 0;
    return (int)(((long long)nnz + sigma - 1) / sigma);
}

spmv_status_t spmv_csr5_preprocess(const int* rowPtr, int numRows, int nnz, int sigma, int* tile_row_ptr,
                                   int* tile_nnz_offset, cudaStream_t stream) {
    clear_error();
    if (numRows < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    return csr5_tiles(rowPtr, numRows, nnz, sigma, tile_row_ptr, tile_nnz_offset, stream);
}

spmv_status_t spmv_csr5_f32(int R, int C, int N, const int* rowPtr, const int* colIdx, const float* values, int sigma,
                            const int* tileRow, const int* tileOff, const float* x, float* y, float alpha, float beta,
                            const spmv_opts_t* opts) {
    return csr5_exec<float>(R, C, N, rowPtr, colIdx, values, sigma, tileRow, tileOff, x, y, alpha, beta, opts);
}
spmv_status_t spmv_csr5_f64(int R, int C, int N, const int* rowPtr, const int* colIdx, const double* values,
                            int sigma, const int* tileRow, const int* tileOff, const double* x, double* y,
                            double alpha, double beta, const spmv_opts_t* opts) {
    return csr5_exec<double>(R, C, N, rowPtr, colIdx, values, sigma, tileRow, tileOff, x, y, alpha, beta, opts);
}

spmv_status_t spmv_max_row_length(const int* rowPtr, int numRows, int* maxLen, cudaStream_t stream) {
    clear_error();
    return max_row_length(rowPtr, numRows, maxLen, stream);
}

spmv_status_t spmv_csr_to_ell_f32(int R, int N, const int* rowPtr, const int* colIdx, const float* values, int width,
                                  int* ellCol, float* ellVal, long long* truncated, cudaStream_t stream) {
    clear_error();
    (void)N;
    return csr_to_ell<float>(R, rowPtr, colIdx, values, width, ellCol, ellVal, truncated, stream);
}
spmv_status_t spmv_csr_to_ell_f64(int R, int N, const int* rowPtr, const int* colIdx, const double* values,
                                  int width, int* ellCol, double* ellVal, long long* truncated, cudaStream_t stream) {
    clear_error();
    (void)N;
    return csr_to_ell<double>(R, rowPtr, colIdx, values, width, ellCol, ellVal, truncated, stream);
}

spmv_status_t spmv_ellpack_f32(int R, int W, const int* ellCol, const float* ellVal, const float* x, float* y,
                               float alpha, float beta, cudaStream_t stream) {
    return ell_exec<float>(R, W, ellCol, ellVal, x, y, alpha, beta, stream);
}
spmv_status_t spmv_ellpack_f64(int R, int W, const int* ellCol, const double* ellVal, const double* x, double* y,
                               double alpha, double beta, cudaStream_t stream) {
    return ell_exec<double>(R, W, ellCol, ellVal, x, y, alpha, beta, stream);
}

spmv_status_t spmv_reorder_rows_by_length_f32(int R, int N, const int* rowPtr, const int* colIdx, const float* values,
                                              int* rowMap, int* newRowPtr, int* newColIdx, float* newValues,
                                              cudaStream_t stream) {
    clear_error();
    return reorder_rows_by_length<float>(R, N, rowPtr, colIdx, values, rowMap, newRowPtr, newColIdx, newValues,
                                         stream);
}
spmv_status_t spmv_reorder_rows_by_length_f64(int R, int N, const int* rowPtr, const int* colIdx,
                                              const double* values, int* rowMap, int* newRowPtr, int* newColIdx,
                                              double* newValues, cudaStream_t stream) {
    clear_error();
    return reorder_rows_by_length<double>(R, N, rowPtr, colIdx, values, rowMap, newRowPtr, newColIdx, newValues,
                                          stream);
}

spmv_status_t spmv_restore_order_f32(int R, const float* yPerm, const int* rowMap, float* y, cudaStream_t stream) {
    clear_error();
    return restore_order<float>(R, yPerm, rowMap, y, stream);
}
spmv_status_t spmv_restore_order_f64(int R, const double* yPerm, const int* rowMap, double* y, cudaStream_t stream) {
    clear_error();
    return restore_order<double>(R, yPerm, rowMap, y, stream);
}

spmv_status_t spmv_column_perm(spmv_colperm_t kind, int R, int C, int N, const int* rowPtr, const int* colIdx,
                               int* perm, void* keys, cudaStream_t stream) {
    clear_error();
    return column_perm((int)kind, R, C, N, rowPtr, colIdx, perm, keys, stream);
}

spmv_status_t spmv_apply_column_perm(int C, int N, const int* perm, const int* colIdx, int* newColIdx,
                                     cudaStream_t stream) {
    clear_error();
    return apply_column_perm(C, N, perm, colIdx, newColIdx, stream);
}

spmv_status_t spmv_permute_x_f32(int C, const int* perm, const float* x, float* xr, cudaStream_t stream) {
    clear_error();
    return permute_x<float>(C, perm, x, xr, stream);
}
spmv_status_t spmv_permute_x_f64(int C, const int* perm, const double* x, double* xr, cudaStream_t stream) {
    clear_error();
    return permute_x<double>(C, perm, x, xr, stream);
}

spmv_status_t spmv_sort_columns_within_rows_f32(int R, int C, int N, const int* rowPtr, int* colIdx, float* values,
                                                cudaStream_t stream) {
    clear_error();
    return sort_within_rows<float>(R, C, N, rowPtr, colIdx, values, stream);
}
spmv_status_t spmv_sort_columns_within_rows_f64(int R, int C, int N, const int* rowPtr, int* colIdx, double* values,
                                                cudaStream_t stream) {
    clear_error();
    return sort_within_rows<double>(R, C, N, rowPtr, colIdx, values, stream);
}

spmv_status_t spmv_csr_transpose_f32(int R, int C, int N, const int* rowPtr, const int* colIdx, const float* values,
                                     int* tRowPtr, int* tColIdx, float* tValues, cudaStream_t stream) {
    clear_error();
    return csr_transpose<float>(R, C, N, rowPtr, colIdx, values, tRowPtr, tColIdx, tValues, stream);
}

spmv_status_t spmv_csr_transpose_f64(int R, int C, int N, const int* rowPtr, const int* colIdx, const double* values,
                                     int* tRowPtr, int* tColIdx, double* tValues, cudaStream_t stream) {
    clear_error();
    return csr_transpose<double>(R, C, N, rowPtr, colIdx, values, tRowPtr, tColIdx, tValues, stream);
}

spmv_status_t spmv_coo_to_csr_f32(int R, int C, int N, const int* rowIdx, const int* colIdx, const float* values,
                                  int* rowPtr, int* outColIdx, float* outValues, cudaStream_t stream) {
    clear_error();
    return coo_to_csr<float>(R, C, N, rowIdx, colIdx, values, rowPtr, outColIdx, outValues, stream);
}
spmv_status_t spmv_coo_to_csr_f64(int R, int C, int N, const int* rowIdx, const int* colIdx, const double* values,
                                  int* rowPtr, int* outColIdx, double* outValues, cudaStream_t stream) {
    clear_error();
    return coo_to_csr<double>(R, C, N, rowIdx, colIdx, values, rowPtr, outColIdx, outValues, stream);
}

}  // extern "C"
