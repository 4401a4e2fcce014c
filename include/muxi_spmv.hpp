// muxi_spmv.hpp -- the reference's C++ interface over the C ABI.
//
// A caller of the muxi_spmv library (src/api/spmv_api.h and the headers it
// pulls in) recompiles against this header unchanged: the same namespace,
// struct names and fields, template functions and default arguments, now
// running this library's sm_103a kernels.  Differences a caller can observe
// are fixes of reference defects: alpha/beta are applied, spmv_set_stream
// stores the stream itself, rows beyond 65535 blocks are computed, merge-path
// results are correct on split rows, csr_to_ellpack reports truncated rows.
//
// Reference interfaces mirrored (paths inside the muxi_spmv project):
//   src/formats/sparse_formats.h:24-103   CSRMatrix<T>
//   src/formats/sparse_formats.h:284-386  CSR5Matrix<T>
//   src/spmv/ellpack/spmv_ellpack.cuh:26-39  ELLPACKMatrix<T>
//   src/api/spmv_api.h:33-92              handle functions, spmv_exec,
//                                          spmv_exec_transpose, spmv_csr_exec
//   src/spmv/csr/spmv_csr.cuh:1100-1106    spmv_csr<T>
//   src/spmv/csr5/spmv_csr5.cuh:250-330    spmv_csr5, spmv_merge_based,
//                                          csr5_preprocess
//   src/spmv/ellpack/spmv_ellpack.cuh:49-70  csr_to_ellpack, spmv_ellpack
//   src/preprocessing/column_reorder.cuh:42-201  reorderColumns,
//                                          reorderXVector, sortColumnsWithinRows
#ifndef MUXI_SPMV_HPP_
#define MUXI_SPMV_HPP_

#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "muxi_spmv.h"

namespace muxi_spmv {

using ::spmv_handle_t;
using ::spmv_create_handle;
using ::spmv_destroy_handle;
using ::spmv_set_stream;

namespace detail {
template <typename T> struct is_supported : std::integral_constant<bool, std::is_same<T, float>::value ||
                                                                         std::is_same<T, double>::value> {};
inline cudaStream_t stream_of(const spmv_opts_t& o) { return reinterpret_cast<cudaStream_t>(o.stream); }
template <typename T> constexpr spmv_type_t type_of() {
    return std::is_same<T, float>::value ? SPMV_TYPE_FLOAT : SPMV_TYPE_DOUBLE;
}
}  // namespace detail

// ---------------------------------------------------------------------------
// Formats
// ---------------------------------------------------------------------------
template <typename FloatType>
struct CSRMatrix {
    int numRows = 0, numCols = 0, nnz = 0;
    int* rowPtr = nullptr;
    int* colIdx = nullptr;
    FloatType* values = nullptr;
    int* d_rowPtr = nullptr;
    int* d_colIdx = nullptr;
    FloatType* d_values = nullptr;
    bool ownsHostMemory = false;
    bool ownsDeviceMemory = false;

    CSRMatrix() = default;
    CSRMatrix(const CSRMatrix&) = delete;
    CSRMatrix& operator=(const CSRMatrix&) = delete;
    ~CSRMatrix() {
        if (ownsHostMemory) {
            std::free(rowPtr);
            std::free(colIdx);
            std::free(values);
        }
        if (ownsDeviceMemory) {
            cudaFree(d_rowPtr);
            cudaFree(d_colIdx);
            cudaFree(d_values);
        }
    }
    void allocateHost(int rows, int cols, int nonzeros) {
        numRows = rows;
        numCols = cols;
        nnz = nonzeros;
        rowPtr = static_cast<int*>(std::malloc(sizeof(int) * (size_t)(rows + 1)));
        colIdx = static_cast<int*>(std::malloc(sizeof(int) * (size_t)(nonzeros > 0 ? nonzeros : 1)));
        values = static_cast<FloatType*>(std::malloc(sizeof(FloatType) * (size_t)(nonzeros > 0 ? nonzeros : 1)));
        ownsHostMemory = true;
    }
    void allocateDevice() {
        cudaMalloc(&d_rowPtr, sizeof(int) * (size_t)(numRows + 1));
        cudaMalloc(&d_colIdx, sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
        cudaMalloc(&d_values, sizeof(FloatType) * (size_t)(nnz > 0 ? nnz : 1));
        ownsDeviceMemory = true;
    }
    void copyToDevice(cudaStream_t stream = 0) {
        cudaMemcpyAsync(d_rowPtr, rowPtr, sizeof(int) * (size_t)(numRows + 1), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_colIdx, colIdx, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_values, values, sizeof(FloatType) * (size_t)nnz, cudaMemcpyHostToDevice, stream);
    }
    void copyFromDevice(cudaStream_t stream = 0) {
        cudaMemcpyAsync(rowPtr, d_rowPtr, sizeof(int) * (size_t)(numRows + 1), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(colIdx, d_colIdx, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(values, d_values, sizeof(FloatType) * (size_t)nnz, cudaMemcpyDeviceToHost, stream);
    }
};

template <typename FloatType>
struct CSR5Matrix {
    int numRows = 0, numCols = 0, nnz = 0;
    int* rowPtr = nullptr;
    int* colIdx = nullptr;
    FloatType* values = nullptr;
    int sigma = 256;
    int numTiles = 0;
    int* tile_row_ptr = nullptr;     // host copy, filled by copyTileMetadataToHost()
    int* tile_nnz_offset = nullptr;
    int* d_rowPtr = nullptr;
    int* d_colIdx = nullptr;
    FloatType* d_values = nullptr;
    int* d_tile_row_ptr = nullptr;
    int* d_tile_nnz_offset = nullptr;
    bool ownsCsrData = false;
    bool ownsTileData = false;
    bool ownsDeviceMemory = false;
    double conversionTimeMs = 0.0;

    CSR5Matrix() = default;
    CSR5Matrix(const CSR5Matrix&) = delete;
    CSR5Matrix& operator=(const CSR5Matrix&) = delete;
    ~CSR5Matrix() {
        if (ownsTileData) {
            std::free(tile_row_ptr);
            std::free(tile_nnz_offset);
        }
        if (ownsDeviceMemory) {
            cudaFree(d_tile_row_ptr);
            cudaFree(d_tile_nnz_offset);
        }
    }
    void referenceFromCSR(const CSRMatrix<FloatType>& csr) {
        numRows = csr.numRows;
        numCols = csr.numCols;
        nnz = csr.nnz;
        rowPtr = csr.rowPtr;
        colIdx = csr.colIdx;
        values = csr.values;
        d_rowPtr = csr.d_rowPtr;
        d_colIdx = csr.d_colIdx;
        d_values = csr.d_values;
        ownsCsrData = false;
    }
    void allocateTileMetadata(int tileCount) {
        numTiles = tileCount;
        tile_row_ptr = static_cast<int*>(std::malloc(sizeof(int) * (size_t)(tileCount > 0 ? tileCount : 1)));
        tile_nnz_offset = static_cast<int*>(std::malloc(sizeof(int) * (size_t)(tileCount > 0 ? tileCount : 1)));
        ownsTileData = true;
    }
    void allocateDeviceTileMetadata() {
        cudaMalloc(&d_tile_row_ptr, sizeof(int) * (size_t)(numTiles > 0 ? numTiles : 1));
        cudaMalloc(&d_tile_nnz_offset, sizeof(int) * (size_t)(numTiles > 0 ? numTiles : 1));
        ownsDeviceMemory = true;
    }
    void copyTileMetadataToHost(cudaStream_t stream = 0) {
        cudaMemcpyAsync(tile_row_ptr, d_tile_row_ptr, sizeof(int) * (size_t)numTiles, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(tile_nnz_offset, d_tile_nnz_offset, sizeof(int) * (size_t)numTiles, cudaMemcpyDeviceToHost,
                        stream);
    }
};

// COOMatrix<T> (sparse_formats.h:113-162): the reference declares the type
// without a kernel; here spmv_exec(SPMV_FORMAT_COO, ...) converts it to CSR
// on the device and runs the stateless CSR SpMV.
template <typename FloatType>
struct COOMatrix {
    int numRows = 0, numCols = 0, nnz = 0;
    int* rowIdx = nullptr;
    int* colIdx = nullptr;
    FloatType* values = nullptr;
    int* d_rowIdx = nullptr;
    int* d_colIdx = nullptr;
    FloatType* d_values = nullptr;
    bool ownsHostMemory = false;
    bool ownsDeviceMemory = false;

    COOMatrix() = default;
    COOMatrix(const COOMatrix&) = delete;
    COOMatrix& operator=(const COOMatrix&) = delete;
    ~COOMatrix() {
        if (ownsHostMemory) {
            std::free(rowIdx);
            std::free(colIdx);
            std::free(values);
        }
        if (ownsDeviceMemory) {
            cudaFree(d_rowIdx);
            cudaFree(d_colIdx);
            cudaFree(d_values);
        }
    }
    void allocateHost(int rows, int cols, int nonzeros) {
        numRows = rows;
        numCols = cols;
        nnz = nonzeros;
        const size_t n = (size_t)(nonzeros > 0 ? nonzeros : 1);
        rowIdx = static_cast<int*>(std::malloc(sizeof(int) * n));
        colIdx = static_cast<int*>(std::malloc(sizeof(int) * n));
        values = static_cast<FloatType*>(std::malloc(sizeof(FloatType) * n));
        ownsHostMemory = true;
    }
    void allocateDevice() {
        const size_t n = (size_t)(nnz > 0 ? nnz : 1);
        cudaMalloc(&d_rowIdx, sizeof(int) * n);
        cudaMalloc(&d_colIdx, sizeof(int) * n);
        cudaMalloc(&d_values, sizeof(FloatType) * n);
        ownsDeviceMemory = true;
    }
    void copyToDevice(cudaStream_t stream = 0) {
        if (nnz <= 0) return;
        cudaMemcpyAsync(d_rowIdx, rowIdx, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_colIdx, colIdx, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_values, values, sizeof(FloatType) * (size_t)nnz, cudaMemcpyHostToDevice, stream);
    }
};

// CSR2Matrix<T> (sparse_formats.h:164-205): declared by the reference without
// a kernel or conversion; the same members here, so code naming it compiles;
// spmv_exec refuses it (SPMV_ERROR_UNSUPPORTED_FORMAT).  BSRMatrix<T, B>
// (sparse_formats.h:207-269): the same members, filled on the device by
// csr_to_bsr<T, B> (B = 2, 4 or 8) and run by spmv_bsr<T, B> / spmv_exec.
template <typename FloatType>
struct CSR2Matrix {
    int numRows = 0, numCols = 0, nnz = 0;
    int* rowPtr = nullptr;
    FloatType* values = nullptr;
    uint8_t* metadata = nullptr;
    int* d_rowPtr = nullptr;
    FloatType* d_values = nullptr;
    uint8_t* d_metadata = nullptr;
    bool ownsHostMemory = false;
    bool ownsDeviceMemory = false;
};

template <typename FloatType, int BlockSize>
struct BSRMatrix {
    int numRows = 0, numCols = 0, numBlockRows = 0, numBlockCols = 0, numBlocks = 0;
    int blockSize = BlockSize;
    int* rowPtr = nullptr;
    int* colIdx = nullptr;
    FloatType* values = nullptr;
    int* d_rowPtr = nullptr;
    int* d_colIdx = nullptr;
    FloatType* d_values = nullptr;
    bool ownsHostMemory = false;
    bool ownsDeviceMemory = false;

    BSRMatrix() = default;
    BSRMatrix(const BSRMatrix&) = delete;
    BSRMatrix& operator=(const BSRMatrix&) = delete;
    ~BSRMatrix() {
        if (ownsHostMemory) {
            std::free(rowPtr);
            std::free(colIdx);
            std::free(values);
        }
        if (ownsDeviceMemory) {
            cudaFree(d_rowPtr);
            cudaFree(d_colIdx);
            cudaFree(d_values);
        }
    }
};

template <typename FloatType>
struct ELLPACKMatrix {
    int numRows = 0, numCols = 0, numElements = 0, nnz = 0;
    int* d_colIdx = nullptr;
    FloatType* d_values = nullptr;
    long long truncatedRows = 0;  // rows longer than numElements (their tails are dropped)
};

// ---------------------------------------------------------------------------
// Execution
// ---------------------------------------------------------------------------
inline spmv_status_t csr_call(const CSRMatrix<float>& A, const float* x, float* y, float a, float b,
                              const spmv_opts_t& o) {
    return spmv_csr_f32(A.numRows, A.numCols, A.nnz, A.d_rowPtr, A.d_colIdx, A.d_values, x, y, a, b, &o);
}
inline spmv_status_t csr_call(const CSRMatrix<double>& A, const double* x, double* y, double a, double b,
                              const spmv_opts_t& o) {
    return spmv_csr_f64(A.numRows, A.numCols, A.nnz, A.d_rowPtr, A.d_colIdx, A.d_values, x, y, a, b, &o);
}

template <typename FloatType>
spmv_status_t spmv_csr(const CSRMatrix<FloatType>& matrix, const FloatType* x, FloatType* y, FloatType alpha,
                       FloatType beta, const spmv_opts_t& opts) {
    static_assert(detail::is_supported<FloatType>::value, "float or double");
    return csr_call(matrix, x, y, alpha, beta, opts);
}

template <typename FloatType>
inline spmv_status_t spmv_csr_exec(const CSRMatrix<FloatType>& A, const FloatType* x, FloatType* y,
                                   FloatType alpha = 1.0, FloatType beta = 0.0,
                                   const spmv_opts_t& opts = spmv_default_opts()) {
    return spmv_csr<FloatType>(A, x, y, alpha, beta, opts);
}

inline spmv_status_t merge_call(const CSRMatrix<float>& A, const float* x, float* y, cudaStream_t s) {
    return spmv_merge_based_f32(A.numRows, A.numCols, A.nnz, A.d_rowPtr, A.d_colIdx, A.d_values, x, y, s);
}
inline spmv_status_t merge_call(const CSRMatrix<double>& A, const double* x, double* y, cudaStream_t s) {
    return spmv_merge_based_f64(A.numRows, A.numCols, A.nnz, A.d_rowPtr, A.d_colIdx, A.d_values, x, y, s);
}

template <typename FloatType>
spmv_status_t spmv_merge_based(const CSRMatrix<FloatType>& matrix, const FloatType* x, FloatType* y,
                               cudaStream_t stream) {
    return merge_call(matrix, x, y, stream);
}

// spmv_sparse_optimized<T> (src/spmv/csr/spmv_sparse_optimized.cuh:29-33):
// the reference picks a light / virtual-warp / merge kernel by mean row
// length; here every matrix takes the stateless default (per-call CSR5 tiles,
// nonzero-balanced, so short and long rows alike), y = A*x on `stream`.
template <typename FloatType>
spmv_status_t spmv_sparse_optimized(const CSRMatrix<FloatType>& matrix, const FloatType* x, FloatType* y,
                                    cudaStream_t stream) {
    spmv_opts_t o = spmv_default_opts();
    o.stream = reinterpret_cast<void*>(stream);
    return spmv_csr<FloatType>(matrix, x, y, FloatType(1), FloatType(0), o);
}

template <typename FloatType>
spmv_status_t csr5_preprocess(const CSRMatrix<FloatType>& csr, CSR5Matrix<FloatType>& csr5, int sigma,
                              cudaStream_t stream) {
    if (csr.nnz == 0) return SPMV_SUCCESS;
    csr5.referenceFromCSR(csr);
    csr5.sigma = sigma > 0 ? sigma : spmv_csr5_default_sigma();
    csr5.allocateTileMetadata(spmv_csr5_num_tiles(csr.nnz, csr5.sigma));
    csr5.allocateDeviceTileMetadata();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, stream);
    const spmv_status_t st = spmv_csr5_preprocess(csr.d_rowPtr, csr.numRows, csr.nnz, csr5.sigma,
                                                  csr5.d_tile_row_ptr, csr5.d_tile_nnz_offset, stream);
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    csr5.conversionTimeMs = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st == SPMV_SUCCESS) {
        csr5.copyTileMetadataToHost(stream);
        cudaStreamSynchronize(stream);
    }
    return st;
}

inline spmv_status_t csr5_call(const CSR5Matrix<float>& m, const float* x, float* y, float a, float b,
                               const spmv_opts_t& o) {
    return spmv_csr5_f32(m.numRows, m.numCols, m.nnz, m.d_rowPtr, m.d_colIdx, m.d_values, m.sigma, m.d_tile_row_ptr,
                         m.d_tile_nnz_offset, x, y, a, b, &o);
}
inline spmv_status_t csr5_call(const CSR5Matrix<double>& m, const double* x, double* y, double a, double b,
                               const spmv_opts_t& o) {
    return spmv_csr5_f64(m.numRows, m.numCols, m.nnz, m.d_rowPtr, m.d_colIdx, m.d_values, m.sigma, m.d_tile_row_ptr,
                         m.d_tile_nnz_offset, x, y, a, b, &o);
}

template <typename FloatType>
spmv_status_t spmv_csr5(const CSR5Matrix<FloatType>& matrix, const FloatType* x, FloatType* y, FloatType alpha,
                        FloatType beta, const spmv_opts_t& opts) {
    return csr5_call(matrix, x, y, alpha, beta, opts);
}

inline spmv_status_t ell_conv(const CSRMatrix<float>& A, int W, int* c, float* v, long long* t, cudaStream_t s) {
    return spmv_csr_to_ell_f32(A.numRows, A.nnz, A.d_rowPtr, A.d_colIdx, A.d_values, W, c, v, t, s);
}
inline spmv_status_t ell_conv(const CSRMatrix<double>& A, int W, int* c, double* v, long long* t, cudaStream_t s) {
    return spmv_csr_to_ell_f64(A.numRows, A.nnz, A.d_rowPtr, A.d_colIdx, A.d_values, W, c, v, t, s);
}

// The reference converts from the host arrays and uploads; this converts on
// the device from the device arrays (both must be populated, as the
// reference's callers do before calling it).
template <typename FloatType>
spmv_status_t csr_to_ellpack(const CSRMatrix<FloatType>& csr, ELLPACKMatrix<FloatType>& ellpack,
                             int maxElements = 0) {
    int W = maxElements;
    if (W <= 0) {
        const spmv_status_t st = spmv_max_row_length(csr.d_rowPtr, csr.numRows, &W, 0);
        if (st != SPMV_SUCCESS) return st;
    }
    ellpack.numRows = csr.numRows;
    ellpack.numCols = csr.numCols;
    ellpack.numElements = W;
    ellpack.nnz = csr.nnz;
    const size_t slots = (size_t)csr.numRows * (size_t)W;
    if (cudaMalloc(&ellpack.d_colIdx, sizeof(int) * (slots ? slots : 1)) != cudaSuccess ||
        cudaMalloc(&ellpack.d_values, sizeof(FloatType) * (slots ? slots : 1)) != cudaSuccess)
        return SPMV_ERROR_MEMORY_ALLOC;
    return ell_conv(csr, W, ellpack.d_colIdx, ellpack.d_values, &ellpack.truncatedRows, 0);
}

inline spmv_status_t ell_call(const ELLPACKMatrix<float>& e, const float* x, float* y, cudaStream_t s) {
    return spmv_ellpack_f32(e.numRows, e.numElements, e.d_colIdx, e.d_values, x, y, 1.0f, 0.0f, s);
}
inline spmv_status_t ell_call(const ELLPACKMatrix<double>& e, const double* x, double* y, cudaStream_t s) {
    return spmv_ellpack_f64(e.numRows, e.numElements, e.d_colIdx, e.d_values, x, y, 1.0, 0.0, s);
}

template <typename FloatType>
spmv_status_t spmv_ellpack(const ELLPACKMatrix<FloatType>& ellpack, const FloatType* d_x, FloatType* d_y,
                           cudaStream_t stream) {
    return ell_call(ellpack, d_x, d_y, stream);
}

// CSR -> BSR on the device (columns sorted within rows); the BSR owns its
// device arrays.
template <typename FloatType, int BlockSize>
spmv_status_t csr_to_bsr(const CSRMatrix<FloatType>& csr, BSRMatrix<FloatType, BlockSize>& bsr,
                         cudaStream_t stream = 0) {
    static_assert(BlockSize == 2 || BlockSize == 4 || BlockSize == 8, "block size 2, 4 or 8");
    bsr.numRows = csr.numRows;
    bsr.numCols = csr.numCols;
    bsr.numBlockRows = (csr.numRows + BlockSize - 1) / BlockSize;
    bsr.numBlockCols = (csr.numCols + BlockSize - 1) / BlockSize;
    if (cudaMalloc(&bsr.d_rowPtr, sizeof(int) * ((size_t)bsr.numBlockRows + 1)) != cudaSuccess)
        return SPMV_ERROR_MEMORY_ALLOC;
    bsr.ownsDeviceMemory = true;
    spmv_status_t st = spmv_csr_to_bsr_count(csr.numRows, csr.numCols, csr.nnz, csr.d_rowPtr, csr.d_colIdx, BlockSize,
                                             bsr.d_rowPtr, &bsr.numBlocks, stream);
    if (st != SPMV_SUCCESS) return st;
    const size_t nb = (size_t)(bsr.numBlocks > 0 ? bsr.numBlocks : 1);
    if (cudaMalloc(&bsr.d_colIdx, sizeof(int) * nb) != cudaSuccess ||
        cudaMalloc(&bsr.d_values, sizeof(FloatType) * nb * BlockSize * BlockSize) != cudaSuccess)
        return SPMV_ERROR_MEMORY_ALLOC;
    if (std::is_same<FloatType, float>::value)
        return spmv_csr_to_bsr_f32(csr.numRows, csr.numCols, csr.nnz, csr.d_rowPtr, csr.d_colIdx,
                                   reinterpret_cast<const float*>(csr.d_values), BlockSize, bsr.d_rowPtr, bsr.d_colIdx,
                                   reinterpret_cast<float*>(bsr.d_values), stream);
    return spmv_csr_to_bsr_f64(csr.numRows, csr.numCols, csr.nnz, csr.d_rowPtr, csr.d_colIdx,
                               reinterpret_cast<const double*>(csr.d_values), BlockSize, bsr.d_rowPtr, bsr.d_colIdx,
                               reinterpret_cast<double*>(bsr.d_values), stream);
}

namespace detail {
template <typename FloatType>
inline spmv_status_t bsr_call(int R, int C, int B, int nbr, const int* rp, const int* ci, const FloatType* v,
                              const FloatType* x, FloatType* y, FloatType alpha, FloatType beta, cudaStream_t s) {
    if (std::is_same<FloatType, float>::value)
        return spmv_bsr_f32(R, C, B, nbr, rp, ci, reinterpret_cast<const float*>(v), reinterpret_cast<const float*>(x),
                            reinterpret_cast<float*>(y), (float)alpha, (float)beta, s);
    return spmv_bsr_f64(R, C, B, nbr, rp, ci, reinterpret_cast<const double*>(v), reinterpret_cast<const double*>(x),
                        reinterpret_cast<double*>(y), (double)alpha, (double)beta, s);
}
}  // namespace detail

template <typename FloatType, int BlockSize>
spmv_status_t spmv_bsr(const BSRMatrix<FloatType, BlockSize>& bsr, const FloatType* x, FloatType* y,
                       cudaStream_t stream = 0, FloatType alpha = 1, FloatType beta = 0) {
    return detail::bsr_call<FloatType>(bsr.numRows, bsr.numCols, BlockSize, bsr.numBlockRows, bsr.d_rowPtr,
                                       bsr.d_colIdx, bsr.d_values, x, y, alpha, beta, stream);
}

// spmv_exec<T> (spmv_api.h:57-65, declared but not defined by the reference):
// `matrix` points to a CSRMatrix<T>, CSR5Matrix<T>, COOMatrix<T>,
// BSRMatrix<T, B> or ELLPACKMatrix<T> according to `format`; runs on the
// handle's stream and options.  CSR2 is refused.
template <typename FloatType>
spmv_status_t spmv_exec(spmv_handle_t* handle, spmv_format_t format, const void* matrix, const FloatType* x,
                        FloatType* y, FloatType alpha = 1.0, FloatType beta = 0.0) {
    if (!handle) return SPMV_ERROR_INVALID_HANDLE;
    if (!matrix) return SPMV_ERROR_INVALID_MATRIX;
    spmv_opts_t o = handle->opts;
    o.stream = reinterpret_cast<void*>(handle->stream);
    switch (format) {
        case SPMV_FORMAT_CSR:
            return spmv_csr<FloatType>(*static_cast<const CSRMatrix<FloatType>*>(matrix), x, y, alpha, beta, o);
        case SPMV_FORMAT_CSR5:
            return spmv_csr5<FloatType>(*static_cast<const CSR5Matrix<FloatType>*>(matrix), x, y, alpha, beta, o);
        case SPMV_FORMAT_BSR: {
            // every BSRMatrix<T, B> has the same layout; blockSize gives B
            const auto& b = *static_cast<const BSRMatrix<FloatType, 2>*>(matrix);
            return detail::bsr_call<FloatType>(b.numRows, b.numCols, b.blockSize, b.numBlockRows, b.d_rowPtr,
                                               b.d_colIdx, b.d_values, x, y, alpha, beta, handle->stream);
        }
        case SPMV_FORMAT_COO: {
            const auto& c = *static_cast<const COOMatrix<FloatType>*>(matrix);
            if (std::is_same<FloatType, float>::value)
                return spmv_coo_f32(c.numRows, c.numCols, c.nnz, c.d_rowIdx, c.d_colIdx,
                                    reinterpret_cast<const float*>(c.d_values), reinterpret_cast<const float*>(x),
                                    reinterpret_cast<float*>(y), (float)alpha, (float)beta, &o);
            return spmv_coo_f64(c.numRows, c.numCols, c.nnz, c.d_rowIdx, c.d_colIdx,
                                reinterpret_cast<const double*>(c.d_values), reinterpret_cast<const double*>(x),
                                reinterpret_cast<double*>(y), (double)alpha, (double)beta, &o);
        }
        case SPMV_FORMAT_ELL: {
            const auto& e = *static_cast<const ELLPACKMatrix<FloatType>*>(matrix);
            if (std::is_same<FloatType, float>::value)
                return spmv_ellpack_f32(e.numRows, e.numElements, e.d_colIdx,
                                        reinterpret_cast<const float*>(e.d_values), reinterpret_cast<const float*>(x),
                                        reinterpret_cast<float*>(y), (float)alpha, (float)beta, handle->stream);
            return spmv_ellpack_f64(e.numRows, e.numElements, e.d_colIdx, reinterpret_cast<const double*>(e.d_values),
                                    reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y), (double)alpha,
                                    (double)beta, handle->stream);
        }
        default:
            return SPMV_ERROR_UNSUPPORTED_FORMAT;
    }
}

// spmv_exec_transpose<T> (spmv_api.h:70-78, declared there without a
// definition): y = alpha*A^T*x + beta*y for CSR matrices (x: numRows
// entries, y: numCols), on the handle's stream; other formats are refused.
template <typename FloatType>
spmv_status_t spmv_exec_transpose(spmv_handle_t* handle, spmv_format_t format, const void* matrix,
                                  const FloatType* x, FloatType* y, FloatType alpha = 1.0, FloatType beta = 0.0) {
    static_assert(detail::is_supported<FloatType>::value, "float or double");
    if (!handle) return SPMV_ERROR_INVALID_HANDLE;
    if (format != SPMV_FORMAT_CSR) return SPMV_ERROR_UNSUPPORTED_FORMAT;
    const CSRMatrix<FloatType>& A = *static_cast<const CSRMatrix<FloatType>*>(matrix);
    spmv_opts_t o = handle->opts;
    o.operation = SPMV_OP_TRANSPOSE;
    o.stream = (void*)handle->stream;
    if (std::is_same<FloatType, float>::value)
        return spmv_csr_f32(A.numRows, A.numCols, A.nnz, A.d_rowPtr, A.d_colIdx,
                            reinterpret_cast<const float*>(A.d_values), reinterpret_cast<const float*>(x),
                            reinterpret_cast<float*>(y), (float)alpha, (float)beta, &o);
    return spmv_csr_f64(A.numRows, A.numCols, A.nnz, A.d_rowPtr, A.d_colIdx, reinterpret_cast<const double*>(A.d_values),
                        reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y), (double)alpha, (double)beta,
                        &o);
}

// ---------------------------------------------------------------------------
// Preprocessing (column_reorder.cuh).  The reference runs these on the host
// arrays; here the host arrays are staged to the device, reordered there,
// and copied back, so callers see the same host-side results.
// ---------------------------------------------------------------------------
struct ColumnReorderStats {
    int numReorders;
    float avgDistanceBefore;
    float avgDistanceAfter;
    float improvementRatio;
};

template <typename FloatType>
spmv_status_t reorderColumns(const CSRMatrix<FloatType>& matrix, CSRMatrix<FloatType>& reorderedMatrix,
                             std::vector<int>& forwardMap, ColumnReorderStats& stats) {
    if (!matrix.rowPtr) return SPMV_ERROR_INVALID_MATRIX;
    const int R = matrix.numRows, C = matrix.numCols, N = matrix.nnz;
    int *dRp = nullptr, *dCol = nullptr, *dPerm = nullptr, *dNew = nullptr;
    cudaMalloc(&dRp, sizeof(int) * (size_t)(R + 1));
    cudaMalloc(&dCol, sizeof(int) * (size_t)(N > 0 ? N : 1));
    cudaMalloc(&dPerm, sizeof(int) * (size_t)(C > 0 ? C : 1));
    cudaMalloc(&dNew, sizeof(int) * (size_t)(N > 0 ? N : 1));
    cudaMemcpy(dRp, matrix.rowPtr, sizeof(int) * (size_t)(R + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(dCol, matrix.colIdx, sizeof(int) * (size_t)N, cudaMemcpyHostToDevice);
    spmv_status_t st = spmv_column_perm(SPMV_COLPERM_CENTER_OF_MASS, R, C, N, dRp, dCol, dPerm, nullptr, 0);
    if (st == SPMV_SUCCESS) st = spmv_apply_column_perm(C, N, dPerm, dCol, dNew, 0);
    reorderedMatrix.allocateHost(R, C, N);
    forwardMap.resize(C);
    if (st == SPMV_SUCCESS) {
        cudaMemcpy(forwardMap.data(), dPerm, sizeof(int) * (size_t)C, cudaMemcpyDeviceToHost);
        cudaMemcpy(reorderedMatrix.colIdx, dNew, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost);
        std::memcpy(reorderedMatrix.rowPtr, matrix.rowPtr, sizeof(int) * (size_t)(R + 1));
        std::memcpy(reorderedMatrix.values, matrix.values, sizeof(FloatType) * (size_t)N);
        // Statistics over the first 10,000 rows (column_reorder.cuh:120-138).
        double before = 0, after = 0;
        long long count = 0;
        for (int r = 0; r < R && r < 10000; ++r)
            for (int j = matrix.rowPtr[r]; j < matrix.rowPtr[r + 1] - 1; ++j) {
                before += std::abs(matrix.colIdx[j + 1] - matrix.colIdx[j]);
                after += std::abs(reorderedMatrix.colIdx[j + 1] - reorderedMatrix.colIdx[j]);
                ++count;
            }
        if (count > 0) {
            stats.avgDistanceBefore = (float)(before / count);
            stats.avgDistanceAfter = (float)(after / count);
            stats.improvementRatio = stats.avgDistanceBefore /
                                     (stats.avgDistanceAfter > 1.0f ? stats.avgDistanceAfter : 1.0f);
        }
    }
    cudaFree(dRp);
    cudaFree(dCol);
    cudaFree(dPerm);
    cudaFree(dNew);
    return st;
}

template <typename FloatType>
void reorderXVector(const FloatType* h_x, FloatType* h_x_reordered, const std::vector<int>& forwardMap) {
    for (size_t i = 0; i < forwardMap.size(); ++i) h_x_reordered[i] = h_x[forwardMap[i]];
}

template <typename FloatType>
spmv_status_t sortColumnsWithinRows(CSRMatrix<FloatType>& matrix) {
    const int R = matrix.numRows, N = matrix.nnz;
    int *dRp = nullptr, *dCol = nullptr;
    FloatType* dVal = nullptr;
    cudaMalloc(&dRp, sizeof(int) * (size_t)(R + 1));
    cudaMalloc(&dCol, sizeof(int) * (size_t)(N > 0 ? N : 1));
    cudaMalloc(&dVal, sizeof(FloatType) * (size_t)(N > 0 ? N : 1));
    cudaMemcpy(dRp, matrix.rowPtr, sizeof(int) * (size_t)(R + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(dCol, matrix.colIdx, sizeof(int) * (size_t)N, cudaMemcpyHostToDevice);
    cudaMemcpy(dVal, matrix.values, sizeof(FloatType) * (size_t)N, cudaMemcpyHostToDevice);
    spmv_status_t st;
    if (std::is_same<FloatType, float>::value)
        st = spmv_sort_columns_within_rows_f32(R, matrix.numCols, N, dRp, dCol, reinterpret_cast<float*>(dVal), 0);
    else
        st = spmv_sort_columns_within_rows_f64(R, matrix.numCols, N, dRp, dCol, reinterpret_cast<double*>(dVal), 0);
    if (st == SPMV_SUCCESS) {
        cudaMemcpy(matrix.colIdx, dCol, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost);
        cudaMemcpy(matrix.values, dVal, sizeof(FloatType) * (size_t)N, cudaMemcpyDeviceToHost);
    }
    cudaFree(dRp);
    cudaFree(dCol);
    cudaFree(dVal);
    return st;
}

// Matrix Market I/O: src/generators/mtx_io.h:22-85 (namespace muxi_spmv::io).
namespace io {

struct MTXHeader {
    bool isSymmetric;
    bool isComplex;
    bool isPattern;
    bool isInteger;
    int numRows;
    int numCols;
    int nnz;
};

inline spmv_status_t readMTXHeader(const char* filename, MTXHeader& header) {
    spmv_mtx_header_t h;
    const spmv_status_t st = spmv_mtx_read_header(filename, &h);
    if (st != SPMV_SUCCESS) return st;
    header = MTXHeader{h.isSymmetric != 0, h.isComplex != 0, h.isPattern != 0, h.isInteger != 0, h.numRows,
                       h.numCols, h.nnz};
    return SPMV_SUCCESS;
}

// Fills the host arrays of `matrix` (it takes ownership of them).
template <typename FloatType>
spmv_status_t readMTXFile(const char* filename, CSRMatrix<FloatType>& matrix, bool expandSymmetric = true) {
    spmv_host_csr_t h;
    const spmv_status_t st = spmv_mtx_read(filename, detail::type_of<FloatType>(), expandSymmetric ? 1 : 0, &h);
    if (st != SPMV_SUCCESS) return st;
    if (matrix.ownsHostMemory) {
        std::free(matrix.rowPtr);
        std::free(matrix.colIdx);
        std::free(matrix.values);
    }
    matrix.numRows = h.numRows;
    matrix.numCols = h.numCols;
    matrix.nnz = h.nnz;
    matrix.rowPtr = h.rowPtr;
    matrix.colIdx = h.colIdx;
    matrix.values = static_cast<FloatType*>(h.values);
    matrix.ownsHostMemory = true;
    return SPMV_SUCCESS;
}

template <typename FloatType>
spmv_status_t writeMTXFile(const char* filename, const CSRMatrix<FloatType>& matrix, bool writeSymmetric = false) {
    spmv_host_csr_t h{matrix.numRows, matrix.numCols, matrix.nnz, matrix.rowPtr, matrix.colIdx,
                      static_cast<void*>(matrix.values), detail::type_of<FloatType>()};
    return spmv_mtx_write(filename, &h, writeSymmetric ? 1 : 0);
}

}  // namespace io

}  // namespace muxi_spmv

#endif  // MUXI_SPMV_HPP_
