/*
 * muxi_spmv.h -- C ABI of the GB300 (sm_103a) SpMV library.
 *
 * This is the drop-in boundary for the muxi_spmv "handle / matrix / format
 * conversion / execute" path.  Every entry point takes plain pointers and
 * sizes (device pointers unless the name says "host"), returns a
 * spmv_status_t and never throws.  The reference exposes the same operations
 * as C++ templates in namespace muxi_spmv; include/muxi_spmv.hpp maps those
 * template names onto the _f32 / _f64 entry points declared here.
 *
 * Reference interfaces replaced (paths inside the muxi_spmv project):
 *   src/utils/common.h:31-94          status / format / type / op enums, opts
 *   src/api/spmv_api.h:18-92          handle, spmv_exec (spmv_convert +
 *                                      spmv_exec_* here), spmv_csr_exec
 *   src/spmv/csr/spmv_csr.cu:52-249   spmv_csr<T> dispatcher
 *   src/spmv/csr5/spmv_csr5.cu:223-362  csr5_preprocess<T>, spmv_csr5<T>
 *   src/spmv/csr5/spmv_csr5.cu:497-533,912-1014  merge-path search,
 *                                      partitions, spmv_merge_based<T>
 *   src/spmv/ellpack/spmv_ellpack.cu:11-91  csr_to_ellpack<T>, spmv_ellpack<T>
 *   src/preprocessing/column_reorder.cuh:42-201  column reorders
 *   tests/test_row_reordering.cu:99-143, tests/test_combined_optimizations.cu:176-181
 *   tests/test_column_reordering.cu:116-199  row / "RCM" / frequency reorders
 *   src/generators/matrix_generator.h:19-102  synthetic matrix generators
 *   src/generators/mtx_io.h:22-85     Matrix Market reader / writer
 *   src/formats/sparse_formats.h:113-162  COOMatrix (declared there, no kernel)
 *   src/formats/sparse_formats.h:207-269  BSRMatrix (declared there, no kernel)
 *   src/spmv/csr/spmv_csr.cuh:105-107, src/api/spmv_api.h:70-78  transpose SpMV
 *   tests/test_pinned_memory.cu:245-380  host-memory SpMV (pipelines here)
 *   tests/test_multi_stream.cu:121-236   multi-stream SpMV (batches here)
 * and adds plans, the learned kernel selector and batched SpMV / SpMM.
 *
 * Threading: a handle is not thread safe (same as the reference).  All device
 * work is asynchronous on the stream given (opts->stream or the handle's
 * stream) unless opts->sync is set.
 */
#ifndef MUXI_SPMV_H_
#define MUXI_SPMV_H_

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MUXI_SPMV_ABI_VERSION 1

#if defined(__GNUC__)
#define SPMV_API __attribute__((visibility("default")))
#else
#define SPMV_API
#endif

/* ------------------------------------------------------------------ */
/* Enums and options: same names and numeric values as                 */
/* src/utils/common.h:31-94.                                            */
/* ------------------------------------------------------------------ */
typedef enum {
    SPMV_SUCCESS = 0,
    SPMV_ERROR_INVALID_HANDLE = -1,
    SPMV_ERROR_INVALID_MATRIX = -2,
    SPMV_ERROR_INVALID_VECTOR = -3,
    SPMV_ERROR_MEMORY_ALLOC = -4,
    SPMV_ERROR_MEMORY_COPY = -5,
    SPMV_ERROR_DEVICE = -6,
    SPMV_ERROR_UNSUPPORTED_FORMAT = -7,
    SPMV_ERROR_UNSUPPORTED_TYPE = -8,
    SPMV_ERROR_INTERNAL = -9
} spmv_status_t;

/* common.h:45-53; ELL has no value in the reference and takes 5 here. */
typedef enum {
    SPMV_FORMAT_CSR = 0,
    SPMV_FORMAT_COO = 1,
    SPMV_FORMAT_CSR2 = 2,
    SPMV_FORMAT_BSR = 3,
    SPMV_FORMAT_CSR5 = 4,
    SPMV_FORMAT_ELL = 5,
    SPMV_FORMAT_UNKNOWN = -1
} spmv_format_t;

/* common.h:55-63 */
typedef enum {
    SPMV_TYPE_FLOAT = 0,
    SPMV_TYPE_DOUBLE = 1,
    SPMV_TYPE_HALF = 2,
    SPMV_TYPE_BF16 = 3,
    SPMV_TYPE_TF32 = 4,
    SPMV_TYPE_UNKNOWN = -1
} spmv_type_t;

/* common.h:65-70 */
typedef enum {
    SPMV_OP_NORMAL = 0,
    SPMV_OP_TRANSPOSE = 1,
    SPMV_OP_CONJUGATE = 2
} spmv_operation_t;

/* common.h:73-94, field for field.  `stream` holds a cudaStream_t value
 * (NULL = legacy default stream).  The reference's spmv_set_stream stored a
 * pointer to the handle's stream member here (spmv_api.cu:53-54); this
 * library stores the stream itself. */
typedef struct {
    spmv_operation_t operation;
    int sync;
    int check_inputs;
    int use_tensor_core;
    int use_streaming;
    int stream_id;
    void* stream;
} spmv_opts_t;

/* common.h:84-94 */
SPMV_API spmv_opts_t spmv_default_opts(void);

/* ------------------------------------------------------------------ */
/* Handle: src/api/spmv_api.h:18-43.  The leading fields are the        */
/* reference's, in its order; the rest are GB300 additions.            */
/* ------------------------------------------------------------------ */
typedef struct spmv_handle_t {
    int deviceId;
    cudaStream_t stream;
    spmv_opts_t opts;
    int warpSize;
    int smCount;
    int maxThreadsPerBlock;
    size_t sharedMemPerSM;
    /* additions */
    size_t l2CacheBytes;
    size_t sharedMemPerBlockOptin;
    int ccMajor;
    int ccMinor;
    void* internal;
} spmv_handle_t;

/* spmv_api.cu:11-37 */
SPMV_API spmv_status_t spmv_create_handle(spmv_handle_t** handle);
/* spmv_api.cu:39-46 */
SPMV_API spmv_status_t spmv_destroy_handle(spmv_handle_t* handle);
/* spmv_api.cu:48-56 (stores the stream by value) */
SPMV_API spmv_status_t spmv_set_stream(spmv_handle_t* handle, cudaStream_t stream);

/* Text of the last error raised on the calling host thread ("" if none). */
SPMV_API const char* spmv_last_error(void);
/* Library ABI version (MUXI_SPMV_ABI_VERSION). */
SPMV_API int spmv_abi_version(void);

/* ------------------------------------------------------------------ */
/* CSR SpMV, y = alpha*A*x + beta*y.                                    */
/* Replaces spmv_csr<T> (src/spmv/csr/spmv_csr.cu:52-249,              */
/* declared spmv_csr.cuh:1100-1106) and spmv_csr_exec<T>                */
/* (src/api/spmv_api.h:82-92).  Unlike the reference, alpha and beta    */
/* are applied; beta == 0 never reads y.  nnz == 0 still writes         */
/* y = beta*y.  The call is stateless: it finds CSR5 tiles of 256       */
/* nonzeros for this call, runs the ordered tile kernel and the carry    */
/* fix-up (merge-path tiles beyond 2^31 - 32769 nonzeros), and takes its */
/* scratch from the stream-ordered allocator of the call's stream.      */
/* ------------------------------------------------------------------ */
SPMV_API spmv_status_t spmv_csr_f32(int numRows, int numCols, int nnz,
                           const int* rowPtr, const int* colIdx, const float* values,
                           const float* x, float* y, float alpha, float beta,
                           const spmv_opts_t* opts);
SPMV_API spmv_status_t spmv_csr_f64(int numRows, int numCols, int nnz,
                           const int* rowPtr, const int* colIdx, const double* values,
                           const double* x, double* y, double alpha, double beta,
                           const spmv_opts_t* opts);

/* opts->operation == SPMV_OP_TRANSPOSE computes y = alpha*A^T*x + beta*y
 * (x: numRows entries, y: numCols entries) by building A^T in stream-ordered
 * scratch (spmv_csr_transpose_*) and running it as a normal SpMV; the
 * reference declares spmv_exec_transpose (spmv_api.h:70-78) without a
 * definition and scatters with float atomics in its transpose kernel. */

/* CSR of A^T on the device: tRowPtr[numCols+1], tColIdx/tValues[nnz]; row c
 * of A^T lists the rows of A holding column c in ascending order. */
SPMV_API spmv_status_t spmv_csr_transpose_f32(int numRows, int numCols, int nnz, const int* rowPtr,
                                              const int* colIdx, const float* values, int* tRowPtr, int* tColIdx,
                                              float* tValues, cudaStream_t stream);
SPMV_API spmv_status_t spmv_csr_transpose_f64(int numRows, int numCols, int nnz, const int* rowPtr,
                                              const int* colIdx, const double* values, int* tRowPtr, int* tColIdx,
                                              double* tValues, cudaStream_t stream);

/* COO (src/formats/sparse_formats.h:113-162, COOMatrix: declared there
 * without a kernel).  spmv_coo_to_csr_* orders the entries by (row, column);
 * entries with equal (row, column) stay separate, in input order, and add.
 * Entries outside the matrix are refused with SPMV_ERROR_INVALID_MATRIX (the
 * check synchronises the stream).  spmv_coo_* converts in stream-ordered
 * scratch and runs the stateless CSR SpMV. */
SPMV_API spmv_status_t spmv_coo_to_csr_f32(int numRows, int numCols, int nnz, const int* rowIdx, const int* colIdx,
                                           const float* values, int* rowPtr, int* outColIdx, float* outValues,
                                           cudaStream_t stream);
SPMV_API spmv_status_t spmv_coo_to_csr_f64(int numRows, int numCols, int nnz, const int* rowIdx, const int* colIdx,
                                           const double* values, int* rowPtr, int* outColIdx, double* outValues,
                                           cudaStream_t stream);
SPMV_API spmv_status_t spmv_coo_f32(int numRows, int numCols, int nnz, const int* rowIdx, const int* colIdx,
                                    const float* values, const float* x, float* y, float alpha, float beta,
                                    const spmv_opts_t* opts);
SPMV_API spmv_status_t spmv_coo_f64(int numRows, int numCols, int nnz, const int* rowIdx, const int* colIdx,
                                    const double* values, const double* x, double* y, double alpha, double beta,
                                    const spmv_opts_t* opts);

/* BSR (src/formats/sparse_formats.h:207-269, BSRMatrix: declared there
 * without a conversion or kernel), block size B = 2, 4 or 8, blocks dense
 * B x B row-major, numBlockRows = ceil(numRows / B).  Conversion from a CSR
 * whose columns are sorted within rows, in two calls:
 * spmv_csr_to_bsr_count fills bRowPtr[numBlockRows + 1] and returns the block
 * count (synchronises the stream; unsorted rows give
 * SPMV_ERROR_INVALID_MATRIX); spmv_csr_to_bsr_* then fills bColIdx[numBlocks]
 * and bValues[numBlocks * B * B] (entries of one row at the same column add).
 * spmv_bsr_*: y = alpha*A*x + beta*y. */
SPMV_API spmv_status_t spmv_csr_to_bsr_count(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                                             int B, int* bRowPtr, int* numBlocks, cudaStream_t stream);
SPMV_API spmv_status_t spmv_csr_to_bsr_f32(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                                           const float* values, int B, const int* bRowPtr, int* bColIdx,
                                           float* bValues, cudaStream_t stream);
SPMV_API spmv_status_t spmv_csr_to_bsr_f64(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                                           const double* values, int B, const int* bRowPtr, int* bColIdx,
                                           double* bValues, cudaStream_t stream);
SPMV_API spmv_status_t spmv_bsr_f32(int numRows, int numCols, int B, int numBlockRows, const int* bRowPtr,
                                    const int* bColIdx, const float* bValues, const float* x, float* y, float alpha,
                                    float beta, cudaStream_t stream);
SPMV_API spmv_status_t spmv_bsr_f64(int numRows, int numCols, int B, int numBlockRows, const int* bRowPtr,
                                    const int* bColIdx, const double* bValues, const double* x, double* y,
                                    double alpha, double beta, cudaStream_t stream);

/* FP32 CSR SpMV that allocates no device memory (no counterpart in the
 * reference).  It runs the kernels of spmv_csr_f32 given the SPMV_KERNEL_MERGE
 * variant {256, 0, 8, 4} (merge-path tiles plus carry fix-up; a default
 * spmv_csr_f32 call runs CSR5 tiles instead, so the two agree within the FP32
 * row bound, not bit for bit).  It is for callers that cannot allocate:
 * code running under a device-memory budget owned by another allocator, or a
 * real-time loop that must not pay an allocation or the synchronisation it
 * can cause.  The caller passes inputs and outputs; the scratch (tile
 * coordinates and carries) is a fixed 8 MiB device array inside the library,
 * so numRows + nnz may reach about 1.07e9 when colIdx and values are 16-byte
 * aligned and about 0.94e9 otherwise -- larger matrices are rejected with
 * SPMV_ERROR_MEMORY_ALLOC and a message that states the limit.  Every GPU
 * that loads the library keeps that array until the process exits.  The
 * first call on a device looks up the array's address (cudaGetSymbolAddress)
 * and keeps it; do not use the entry point on a device after
 * cudaDeviceReset.  All calls share the one
 * array, which keeps the last call's contents (nothing in it needs to start
 * at zero): calls that can overlap on the GPU (different streams without
 * ordering) race and must be serialised by the caller. */
SPMV_API spmv_status_t spmv_csr_noalloc_f32(int numRows, int numCols, int nnz,
                                            const int* rowPtr, const int* colIdx, const float* values,
                                            const float* x, float* y, float alpha, float beta,
                                            cudaStream_t stream);

/* Kernel variants of the CSR family (the autotuner's search space).
 * Replaces the reference's fixed choice between spmv_csr_scalar_kernel,
 * spmv_csr_vector_kernel and the N-threads-per-row family
 * (spmv_csr.cuh:83-208, tests/test_block_optimization.cu:97-145). */
typedef enum {
    SPMV_KERNEL_AUTO = 0,      /* plan: selector decides                    */
    SPMV_KERNEL_SCALAR = 1,    /* one thread per row                        */
    SPMV_KERNEL_VECTOR = 2,    /* threadsPerRow lanes per row, 2..32       */
    SPMV_KERNEL_MERGE = 3,     /* merge-path CTA tiles + carry fix-up       */
    SPMV_KERNEL_CSR5 = 4,      /* sigma-nnz tiles (CSR5 metadata)           */
    SPMV_KERNEL_ELL = 5,       /* column-major ELLPACK                      */
    SPMV_KERNEL_HEURISTIC = 6, /* plan: the reference's avgNnz rule, restated */
    SPMV_KERNEL_BAND = 7,      /* ordered CSR5 tiles of 32*itemsPerThread nonzeros; each
                                  CTA owns a range of consecutive tiles and serves the
                                  gathers that fall in a bulk-copied shared-memory
                                  window of x around its rows from there (FP32 at
                                  1024 threads and 8 per lane: one CTA per SM, the
                                  next tile's loads in flight, 16-byte tile loads
                                  when colIdx and values are 16-byte aligned).  The
                                  launch sets the kernel's shared-memory carve-out
                                  preference to what its CTAs use              */
    SPMV_KERNEL_STREAM = 8     /* ordered CSR5 tiles of 32*itemsPerThread nonzeros, one
                                  CTA per SM over a contiguous tile range; each warp's
                                  next tiles are bulk-copied (TMA) into a ring of
                                  threadsPerRow shared-memory slots ahead of use    */
} spmv_kernel_t;

/* CSR5 (vectorWidth field): gathers in nonzero order, and the same with the
 * next tile's column indices and values requested before the current tile is
 * computed (block ranges only). */
#define SPMV_CSR5_ORDERED 32
#define SPMV_CSR5_ORDERED_PREFETCH 64
/* CSR5 block ranges (threadsPerRow field): one range per resident block. */
#define SPMV_RANGE_PER_RESIDENT_BLOCK (1 << 20)

/* One launch configuration of a kernel family. */
typedef struct {
    spmv_kernel_t kernel;
    int blockSize;       /* threads per CTA: SCALAR/VECTOR 64..1024 (powers
                            of two), MERGE 128/256, CSR5 with vectorWidth
                            32 128..1024, BAND 256/512/1024 (0: 512),
                            STREAM FP32 512 (ipt 16, 3 stages), 768 (ipt
                            16, 2 stages), 1024 (ipt 8, 2 or 3 stages),
                            STREAM FP64 512 (3) or 1024 (2) with ipt 8
                            (0: 512), others 256 or 512                   */
    int threadsPerRow;   /* VECTOR: 1,2,4,8,16,32; CSR5 with vectorWidth 32:
                            0 = one tile per warp; n > 0 = block ranges:
                            a block of blockSize 256/384/512/640/1024
                            threads owns about n tiles per warp of
                            consecutive tiles (fitted so the blocks fill
                            whole waves; n beyond the tiles per resident
                            block gives each resident block one range),
                            which its warps take one at a time; BAND: target
                            tiles per warp of a CTA's range (0: 8), fitted
                            so the CTAs fill whole waves; STREAM: shared-
                            memory slots per warp (0: 3 at 512 threads,
                            else 2)                                       */
    int itemsPerThread;  /* MERGE: merge items per thread (tile = block*ipt);
                            CSR5: nonzeros per lane (tile = 32*ipt);
                            BAND: 8 or 16 (0: 16 for FP32, 8 for FP64)   */
    int vectorWidth;     /* VECTOR/MERGE: 1 or 4 elements per load;
                            CSR5: 32 = gathers issued in nonzero order
                            (32 consecutive nonzeros per instruction), 64 =
                            the same with the next tile's loads issued
                            before the current tile's compute (block ranges
                            of 512, 768 or 1024 threads);
                            BAND: x window in units of 1,024 elements
                            (0: 16, or the largest the CTA shape fits if
                            smaller)                                      */
} spmv_variant_t;

/* Run one explicit variant (no plan, no selector).  MERGE variants take
 * their scratch like spmv_csr_*; CSR5/ELL are not accepted here. */
SPMV_API spmv_status_t spmv_csr_variant_f32(const spmv_variant_t* variant,
                                   int numRows, int numCols, int nnz,
                                   const int* rowPtr, const int* colIdx, const float* values,
                                   const float* x, float* y, float alpha, float beta,
                                   const spmv_opts_t* opts);
SPMV_API spmv_status_t spmv_csr_variant_f64(const spmv_variant_t* variant,
                                   int numRows, int numCols, int nnz,
                                   const int* rowPtr, const int* colIdx, const double* values,
                                   const double* x, double* y, double alpha, double beta,
                                   const spmv_opts_t* opts);

/* ------------------------------------------------------------------ */
/* Merge path (src/spmv/csr5/spmv_csr5.cu:497-533, 912-1014).           */
/* ------------------------------------------------------------------ */
/* Partition count the reference picks for warp 32 (spmv_csr5.cu:941-972):
 * max(1, min((numRows+nnz)/32, 128*8*8)). */
SPMV_API int spmv_merge_default_partitions(int numRows, int nnz);

/* compute_merge_partitions_kernel (spmv_csr5.cu:912-925):
 * pos[t] = min(t*ceil(L/P), L), t = 0..P, L = numRows+nnz.  pos has P+1
 * entries.  Bit-exact with the reference (int64 arithmetic inside, so L up
 * to 2^31-1 never overflows). */
SPMV_API spmv_status_t spmv_merge_partitions(int numRows, int nnz, int numPartitions,
                                    int* pos, cudaStream_t stream);

/* merge_path_search (spmv_csr5.cu:497-533) for each of `count` diagonals:
 * (rowIdx[i], nnzIdx[i]) with rowIdx+nnzIdx = diag[i] and
 * rowPtr[rowIdx] <= nnzIdx <= rowPtr[rowIdx+1].  Bit-exact. */
SPMV_API spmv_status_t spmv_merge_path_search(const int* rowPtr, int numRows, int nnz,
                                     const int* diag, int count,
                                     int* rowIdx, int* nnzIdx, cudaStream_t stream);

/* spmv_merge_based<T> (spmv_csr5.cu:930-1014), with a correct consumer
 * (the reference double-counts rows split by a partition) and no
 * per-call cudaMalloc.  y = A*x. */
SPMV_API spmv_status_t spmv_merge_based_f32(int numRows, int numCols, int nnz,
                                   const int* rowPtr, const int* colIdx, const float* values,
                                   const float* x, float* y, cudaStream_t stream);
SPMV_API spmv_status_t spmv_merge_based_f64(int numRows, int numCols, int nnz,
                                   const int* rowPtr, const int* colIdx, const double* values,
                                   const double* x, double* y, cudaStream_t stream);

/* ------------------------------------------------------------------ */
/* CSR5 (src/spmv/csr5/spmv_csr5.cu:13-58, 223-362;                     */
/* src/formats/sparse_formats.h:284-386).                               */
/* ------------------------------------------------------------------ */
/* Tile size getCSR5Config picks for warp 32 (spmv_csr5.cu:13-32): 128. */
SPMV_API int spmv_csr5_default_sigma(void);
/* ceil(nnz / sigma). */
SPMV_API int spmv_csr5_num_tiles(int nnz, int sigma);
/* csr5_compute_tile_boundaries_kernel (spmv_csr5.cu:36-58): for tile t,
 * tile_row_ptr[t] = last row r in [0,numRows) with rowPtr[r] <= t*sigma and
 * tile_nnz_offset[t] = t*sigma - rowPtr[r].  Arrays hold
 * spmv_csr5_num_tiles() entries (device).  Bit-exact. */
SPMV_API spmv_status_t spmv_csr5_preprocess(const int* rowPtr, int numRows, int nnz, int sigma,
                                            int* tile_row_ptr, int* tile_nnz_offset, cudaStream_t stream);
/* spmv_csr5<T> (spmv_csr5.cu:277-362): SpMV over sigma-nnz tiles described
 * by the metadata above; y = alpha*A*x + beta*y, no atomics (split rows are
 * joined by a carry fix-up in tile order).  sigma must be 128, 256 or 512. */
SPMV_API spmv_status_t spmv_csr5_f32(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                                     const float* values, int sigma, const int* tile_row_ptr,
                                     const int* tile_nnz_offset, const float* x, float* y, float alpha,
                                     float beta, const spmv_opts_t* opts);
SPMV_API spmv_status_t spmv_csr5_f64(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                                     const double* values, int sigma, const int* tile_row_ptr,
                                     const int* tile_nnz_offset, const double* x, double* y, double alpha,
                                     double beta, const spmv_opts_t* opts);

/* ------------------------------------------------------------------ */
/* ELLPACK (src/spmv/ellpack/spmv_ellpack.{cuh,cu}).                    */
/* ------------------------------------------------------------------ */
/* Longest row (the width csr_to_ellpack auto-detects,
 * spmv_ellpack.cu:17-24); *maxLen is host memory. */
SPMV_API spmv_status_t spmv_max_row_length(const int* rowPtr, int numRows, int* maxLen, cudaStream_t stream);
/* csr_to_ellpack (spmv_ellpack.cu:11-70) on the device: ellCol/ellVal hold
 * numRows*width entries, slot (r, i) at r + i*numRows, padding col -1 and
 * value 0.  Rows longer than width keep their first width entries, as the
 * reference does; *truncatedRows (host, may be NULL) counts them.
 * Bit-exact with the reference. */
SPMV_API spmv_status_t spmv_csr_to_ell_f32(int numRows, int nnz, const int* rowPtr, const int* colIdx,
                                           const float* values, int width, int* ellCol, float* ellVal,
                                           long long* truncatedRows, cudaStream_t stream);
SPMV_API spmv_status_t spmv_csr_to_ell_f64(int numRows, int nnz, const int* rowPtr, const int* colIdx,
                                           const double* values, int width, int* ellCol, double* ellVal,
                                           long long* truncatedRows, cudaStream_t stream);
/* spmv_ellpack<T> (spmv_ellpack.cu:72-91): y = alpha*A*x + beta*y over the
 * column-major ELL arrays; slots with col < 0 are skipped. */
SPMV_API spmv_status_t spmv_ellpack_f32(int numRows, int width, const int* ellCol, const float* ellVal,
                                        const float* x, float* y, float alpha, float beta, cudaStream_t stream);
SPMV_API spmv_status_t spmv_ellpack_f64(int numRows, int width, const int* ellCol, const double* ellVal,
                                        const double* x, double* y, double alpha, double beta,
                                        cudaStream_t stream);

/* ------------------------------------------------------------------ */
/* Reorders (device).  Reference: reorderMatrixByRowLength             */
/* (tests/test_row_reordering.cu:99-143), restoreOrder                  */
/* (tests/test_combined_optimizations.cu:176-181), reorderColumns,      */
/* reorderXVector, sortColumnsWithinRows                                */
/* (src/preprocessing/column_reorder.cuh:42-201), reorderColumnsRCM and */
/* reorderColumnsByFrequency (tests/test_column_reordering.cu:116-199). */
/* ------------------------------------------------------------------ */
typedef enum {
    SPMV_COLPERM_CENTER_OF_MASS = 0,  /* key: float mean of the rows touching the column (0 if none),
                                         summed in row order; ties by column id            */
    SPMV_COLPERM_MIN_ROW = 1,         /* the reference's "RCM": key = first row touching the column
                                         (numRows if none); ties by column id               */
    SPMV_COLPERM_FREQUENCY = 2        /* nonzeros per column, descending; ties by column id  */
} spmv_colperm_t;

/* Stable sort of rows by length: rowMap[new] = old, newRowPtr (numRows+1),
 * rows copied in that order.  Bit-exact with std::stable_sort. */
SPMV_API spmv_status_t spmv_reorder_rows_by_length_f32(int numRows, int nnz, const int* rowPtr, const int* colIdx,
                                                       const float* values, int* rowMap, int* newRowPtr,
                                                       int* newColIdx, float* newValues, cudaStream_t stream);
SPMV_API spmv_status_t spmv_reorder_rows_by_length_f64(int numRows, int nnz, const int* rowPtr, const int* colIdx,
                                                       const double* values, int* rowMap, int* newRowPtr,
                                                       int* newColIdx, double* newValues, cudaStream_t stream);
/* y[rowMap[i]] = yPerm[i]. */
SPMV_API spmv_status_t spmv_restore_order_f32(int numRows, const float* yPerm, const int* rowMap, float* y,
                                              cudaStream_t stream);
SPMV_API spmv_status_t spmv_restore_order_f64(int numRows, const double* yPerm, const int* rowMap, double* y,
                                              cudaStream_t stream);
/* Column permutation perm[new] = old (numCols entries).  keys (optional,
 * device): float per column for CENTER_OF_MASS, int per column otherwise.
 * The centre-of-mass order is bit-exact with reorderColumns; for MIN_ROW and
 * FREQUENCY the reference's std::sort leaves tie order unspecified, and
 * this library breaks ties by ascending column id. */
SPMV_API spmv_status_t spmv_column_perm(spmv_colperm_t kind, int numRows, int numCols, int nnz,
                                        const int* rowPtr, const int* colIdx, int* perm, void* keys,
                                        cudaStream_t stream);
/* newColIdx[j] = inv[colIdx[j]] with inv[perm[i]] = i. */
SPMV_API spmv_status_t spmv_apply_column_perm(int numCols, int nnz, const int* perm, const int* colIdx,
                                              int* newColIdx, cudaStream_t stream);
/* xr[i] = x[perm[i]] (reorderXVector). */
SPMV_API spmv_status_t spmv_permute_x_f32(int numCols, const int* perm, const float* x, float* xr,
                                          cudaStream_t stream);
SPMV_API spmv_status_t spmv_permute_x_f64(int numCols, const int* perm, const double* x, double* xr,
                                          cudaStream_t stream);
/* In place: each row's (column, value) pairs ordered by column, then value
 * (pair ordering of std::sort on pair<int, T>). */
SPMV_API spmv_status_t spmv_sort_columns_within_rows_f32(int numRows, int numCols, int nnz, const int* rowPtr,
                                                         int* colIdx, float* values, cudaStream_t stream);
SPMV_API spmv_status_t spmv_sort_columns_within_rows_f64(int numRows, int numCols, int nnz, const int* rowPtr,
                                                         int* colIdx, double* values, cudaStream_t stream);

/* ------------------------------------------------------------------ */
/* Plans: a matrix plus everything one kernel needs precomputed         */
/* (tile coordinates, scratch, format copies).  This is the GB300       */
/* native replacement for spmv_exec<T>(handle, format, matrix, ...)     */
/* (src/api/spmv_api.h:57-65, declared but never defined there).        */
/* The plan borrows the CSR arrays; they must outlive it.               */
/* ------------------------------------------------------------------ */
typedef struct spmv_plan_s* spmv_plan_t;

SPMV_API spmv_status_t spmv_plan_create(spmv_handle_t* handle, spmv_type_t type,
                               int numRows, int numCols, int nnz,
                               const int* rowPtr, const int* colIdx, const void* values,
                               const spmv_variant_t* variant, spmv_plan_t* plan);
/* Matrix ownership of a plan (the reference's CSR5Matrix borrows the CSR
 * arrays, sparse_formats.h:351-362): SPMV_PLAN_BORROW (0, as spmv_plan_create)
 * keeps the caller's arrays, which must outlive the plan; SPMV_PLAN_COPY
 * copies them into memory the plan owns (synchronises the handle's stream
 * before returning, so the caller may free its arrays). */
#define SPMV_PLAN_BORROW 0
#define SPMV_PLAN_COPY 1
SPMV_API spmv_status_t spmv_plan_create_ex(spmv_handle_t* handle, spmv_type_t type, int numRows, int numCols,
                                           int nnz, const int* rowPtr, const int* colIdx, const void* values,
                                           const spmv_variant_t* variant, int flags, spmv_plan_t* plan);
SPMV_API spmv_status_t spmv_plan_destroy(spmv_plan_t plan);
/* The variant the plan runs (after AUTO / HEURISTIC resolution). */
SPMV_API spmv_status_t spmv_plan_get_variant(spmv_plan_t plan, spmv_variant_t* variant);
/* Device bytes the plan holds beyond the borrowed CSR arrays. */
SPMV_API spmv_status_t spmv_plan_get_workspace_bytes(spmv_plan_t plan, size_t* bytes);
SPMV_API spmv_status_t spmv_plan_exec_f32(spmv_handle_t* handle, spmv_plan_t plan, float alpha,
                                 const float* x, float beta, float* y);
SPMV_API spmv_status_t spmv_plan_exec_f64(spmv_handle_t* handle, spmv_plan_t plan, double alpha,
                                 const double* x, double beta, double* y);

/* y = alpha*op(A)*x + beta*y with op = SPMV_OP_NORMAL (as spmv_plan_exec_*)
 * or SPMV_OP_TRANSPOSE (x: numRows entries, y: numCols).  The transpose is
 * built from the matrix's values on the first transposed call and kept with
 * the plan (a caller that changes the values recreates the plan).  That first
 * call allocates and synchronises the handle's stream: make it before
 * capturing transposed executions into a CUDA graph.
 * SPMV_OP_CONJUGATE: SPMV_ERROR_UNSUPPORTED_FORMAT. */
SPMV_API spmv_status_t spmv_plan_exec_op_f32(spmv_handle_t* handle, spmv_plan_t plan, spmv_operation_t op,
                                             float alpha, const float* x, float beta, float* y);
SPMV_API spmv_status_t spmv_plan_exec_op_f64(spmv_handle_t* handle, spmv_plan_t plan, spmv_operation_t op,
                                             double alpha, const double* x, double beta, double* y);

/* The conversion and execute calls of a format-generic ABI (the
 * reference's csr5_preprocess + spmv_csr5, csr_to_ellpack + spmv_ellpack and
 * its declared-only spmv_exec, src/api/spmv_api.h:57-65, as one pair).
 * spmv_convert builds a plan of the CSR arrays in `format`:
 *   SPMV_FORMAT_CSR   any CSR kernel (`params`: a variant; NULL: AUTO);
 *   SPMV_FORMAT_CSR5  CSR5 tiles (`params`: blockSize / itemsPerThread =
 *                     sigma/32 / vectorWidth 32 for nonzero-order gathers;
 *                     NULL: the default tile shape);
 *   SPMV_FORMAT_ELL   column-major ELLPACK (refused beyond 2x padding).
 * Other formats: SPMV_ERROR_UNSUPPORTED_FORMAT (COO and BSR have their own
 * conversions above).  spmv_exec_* = spmv_plan_exec_op_*. */
SPMV_API spmv_status_t spmv_convert(spmv_handle_t* handle, spmv_type_t type, int numRows, int numCols, int nnz,
                                    const int* rowPtr, const int* colIdx, const void* values, spmv_format_t format,
                                    const spmv_variant_t* params, spmv_plan_t* plan);
SPMV_API spmv_status_t spmv_exec_f32(spmv_handle_t* handle, spmv_plan_t plan, spmv_operation_t op, float alpha,
                                     const float* x, float beta, float* y);
SPMV_API spmv_status_t spmv_exec_f64(spmv_handle_t* handle, spmv_plan_t plan, spmv_operation_t op, double alpha,
                                     const double* x, double beta, double* y);

/* Device-side failure word of a plan.  The BAND and STREAM kernels wait for
 * bulk copies with a bound: a wait that gives up (about 2 s) raises this word
 * (code 2: BAND window, code 3: STREAM tile slot), lets its copies land and
 * returns without computing.
 * Synchronises; *code = 0 when clean, else the raised code (the call then
 * returns SPMV_ERROR_DEVICE and clears the word). */
SPMV_API spmv_status_t spmv_plan_device_error(spmv_plan_t plan, int* code);

/* Fault injection for tests (no reference counterpart; the reference has no
 * bounded waits).  enable != 0: the following executions of a BAND or STREAM
 * plan initialise their copy barriers with one arrival held back and wait for
 * it at most `limitCycles` SM clocks (0: 100,000), so the waits run out; the
 * kernel then makes the held-back arrivals itself, waits for its copies to
 * land and returns, and spmv_plan_device_error reports code 2 (BAND) or 3
 * (STREAM).  The GPU context stays usable.  enable = 0 restores normal
 * executions.  Plans of other kernels have no waits:
 * SPMV_ERROR_UNSUPPORTED_FORMAT. */
SPMV_API spmv_status_t spmv_plan_inject_wait_timeout(spmv_plan_t plan, int enable, long long limitCycles);

/* Device-memory accounting and allocation-failure injection for tests (no
 * reference counterpart; the reference's status contract,
 * src/utils/common.h:31-43, names SPMV_ERROR_MEMORY_ALLOC but nothing raises
 * it).  Every device allocation the library makes -- plans, pipelines,
 * batches, selector models, stateless scratch -- is counted while live:
 * spmv_debug_device_memory reports the live bytes and allocations.
 * spmv_debug_fail_allocation(n), n >= 1: the n-th device allocation from now
 * fails as if the device were out of memory (the CUDA driver is not asked); the
 * call that made it returns SPMV_ERROR_MEMORY_ALLOC after releasing what it
 * had taken.  n = 0 turns injection off.  Process-wide, not thread-local. */
SPMV_API spmv_status_t spmv_debug_fail_allocation(long long n);
SPMV_API spmv_status_t spmv_debug_device_memory(long long* liveBytes, long long* liveAllocations);

/* Kernel timing on the launching stream (the role of the reference's
 * GpuTimer, src/utils/timer.h:17-47, moved into the plan): while enabled,
 * each exec records a CUDA event pair around the plan's main kernel only
 * (not the carry fix-up).  spmv_plan_profile_read waits for the recorded
 * events and returns the summed main-kernel time and the launch count, then
 * starts a new window.  Enabling resets the window. */
SPMV_API spmv_status_t spmv_plan_profile(spmv_plan_t plan, int enable);
SPMV_API spmv_status_t spmv_plan_profile_read(spmv_plan_t plan, double* kernel_ms, int* launches);

/* ------------------------------------------------------------------ */
/* Matrix statistics.                                                   */
/* ------------------------------------------------------------------ */
/* Number of distinct column indices present in colIdx (device bitmap).
 * Used for the algorithmic-byte count of the x gather. */
SPMV_API spmv_status_t spmv_count_distinct_columns(int numCols, int nnz, const int* colIdx,
                                          long long* distinct, cudaStream_t stream);
/* Validates a device CSR: rowPtr[0]==0, rowPtr monotone, rowPtr[R]==nnz,
 * 0<=col<numCols.  *bad = number of violations found (0 = valid). */
SPMV_API spmv_status_t spmv_validate_csr(int numRows, int numCols, int nnz, const int* rowPtr,
                                const int* colIdx, long long* bad, cudaStream_t stream);

/* ------------------------------------------------------------------ */
/* Seeded synthetic generators (host, multi-threaded, deterministic for */
/* a given seed whatever the thread count).  Replaces the libc-rand()   */
/* generators of src/generators/matrix_generator.h:19-102.              */
/* Two steps: spmv_gen_row_ptr fills rowPtr (numRows+1, host) and       */
/* returns nnz; spmv_gen_fill_* then fills colIdx/values (host).        */
/* ------------------------------------------------------------------ */
typedef enum {
    SPMV_GEN_POISSON_UNIFORM = 0,  /* Poisson(p0) lengths clamped to [p1,p2];
                                      columns uniform without replacement,
                                      sorted; values U[-1,1]                  */
    SPMV_GEN_POWERLAW = 1,         /* Zipf(p0) lengths truncated to [1,p1];
                                      fraction p3 of columns within +-p2 of
                                      the diagonal, rest uniform; sorted;
                                      values N(0,1)                           */
    SPMV_GEN_STENCIL2D = 2,        /* 5-point on a p0 x p1 grid; 4 / -1       */
    SPMV_GEN_STENCIL3D = 3,        /* 27-point on a p0 x p1 x p2 grid; N(0,1) */
    SPMV_GEN_BANDED = 4,           /* lengths Poisson(p0) clamped [1,p1],
                                      columns within the band of width p1    */
    SPMV_GEN_BLOCKDIAG = 5,        /* p0 diagonal blocks; Poisson(p1) lengths
                                      clamped to the block; columns uniform
                                      inside the block                        */
    SPMV_GEN_ZIPF_UNIFORM = 6,     /* Zipf(p0) lengths truncated to [1,p1],
                                      plus p2 on every row (0 = none), capped
                                      at numCols; columns uniform without
                                      replacement                             */
    SPMV_GEN_DIAGONAL = 7          /* identity pattern, values 1              */
} spmv_gen_kind_t;

typedef struct {
    spmv_gen_kind_t kind;
    int numRows;
    int numCols;
    double p0, p1, p2, p3;
    unsigned long long seed;
    int threads;                   /* 0 = all hardware threads */
} spmv_gen_params_t;

/* Fills rowPtr[0..numRows] and returns nnz in *nnz (int64; the call fails
 * with SPMV_ERROR_INVALID_MATRIX if nnz >= 2^31). */
SPMV_API spmv_status_t spmv_gen_row_ptr(const spmv_gen_params_t* p, int* rowPtr, long long* nnz);
SPMV_API spmv_status_t spmv_gen_fill_f32(const spmv_gen_params_t* p, const int* rowPtr,
                                int* colIdx, float* values);
SPMV_API spmv_status_t spmv_gen_fill_f64(const spmv_gen_params_t* p, const int* rowPtr,
                                int* colIdx, double* values);
/* Dense vector with entries U[lo,hi] (host). */
SPMV_API spmv_status_t spmv_gen_vector_f32(long long n, unsigned long long seed, double lo, double hi,
                                  float* out, int threads);
SPMV_API spmv_status_t spmv_gen_vector_f64(long long n, unsigned long long seed, double lo, double hi,
                                  double* out, int threads);

/* Device-side generators for corpora and batches: same length laws as the
 * host generators for SPMV_GEN_POISSON_UNIFORM, SPMV_GEN_ZIPF_UNIFORM,
 * SPMV_GEN_BANDED and SPMV_GEN_BLOCKDIAG, drawn on the GPU (values differ
 * from the host generators'), and the host generators' SPMV_GEN_STENCIL2D
 * and SPMV_GEN_STENCIL3D operators (3D values drawn here).  Columns are
 * sorted within a row and may repeat where a row is dense in its range.  All pointers are device
 * pointers; spmv_gen_device_row_ptr synchronises the stream to read nnz and
 * fails with SPMV_ERROR_INVALID_MATRIX when nnz >= 2^31. */
SPMV_API spmv_status_t spmv_gen_device_row_ptr(const spmv_gen_params_t* p, int* rowPtr, long long* nnz,
                                               cudaStream_t stream);
SPMV_API spmv_status_t spmv_gen_device_fill_f32(const spmv_gen_params_t* p, const int* rowPtr, int* colIdx,
                                                float* values, cudaStream_t stream);
SPMV_API spmv_status_t spmv_gen_device_vector_f32(long long n, unsigned long long seed, double lo, double hi,
                                                  float* out, cudaStream_t stream);

/* ------------------------------------------------------------------ */
/* Matrix Market files <-> host CSR (src/generators/mtx_io.h:22-85).     */
/* The reader follows readMTXFile (mtx_io.cu:111-222): 1-based entries,  */
/* pattern -> 1, symmetric files mirrored unless expandSymmetric is 0,   */
/* entries sorted by (row, column), duplicates kept in file order.       */
/* Complex files are refused; skew-symmetric mirrors are negated.  The   */
/* writer emits a banner the reader accepts and exact values.            */
/* ------------------------------------------------------------------ */
typedef struct {
    int isSymmetric;
    int isSkew;
    int isComplex;
    int isPattern;
    int isInteger;
    int numRows;
    int numCols;
    int nnz;          /* entries stored in the file */
} spmv_mtx_header_t;

/* Host CSR owned by the library after spmv_mtx_read (free with
 * spmv_host_csr_free); values are float or double per `type`. */
typedef struct {
    int numRows;
    int numCols;
    int nnz;
    int* rowPtr;
    int* colIdx;
    void* values;
    spmv_type_t type;
} spmv_host_csr_t;

SPMV_API spmv_status_t spmv_mtx_read_header(const char* path, spmv_mtx_header_t* header);
SPMV_API spmv_status_t spmv_mtx_read(const char* path, spmv_type_t type, int expandSymmetric, spmv_host_csr_t* out);
/* writeSymmetric: write the upper triangle (column >= row) only, as the
 * reference's writer does (mtx_io.cu:245-262). */
SPMV_API spmv_status_t spmv_mtx_write(const char* path, const spmv_host_csr_t* m, int writeSymmetric);
SPMV_API void spmv_host_csr_free(spmv_host_csr_t* m);

/* ------------------------------------------------------------------ */
/* Kernel selection.  The reference selects by a fixed rule on the     */
/* integer mean row length (src/spmv/csr/spmv_csr.cu:115-153, exposed  */
/* here as SPMV_KERNEL_HEURISTIC); this library adds an exhaustive     */
/* autotuner over a fixed variant space and a learned selector (an MLP  */
/* over matrix features, trained on the autotuner's timings).          */
/* ------------------------------------------------------------------ */
#define SPMV_NUM_FEATURES 32

/* Writes SPMV_NUM_FEATURES floats describing a device CSR matrix to the
 * DEVICE buffer `features` (asynchronous on `stream`).  Reads rowPtr in
 * full and the columns of at most 4096 sampled rows. */
SPMV_API spmv_status_t spmv_matrix_features(spmv_type_t type, int numRows, int numCols, int nnz,
                                            const int* rowPtr, const int* colIdx, float* features,
                                            cudaStream_t stream);

/* Copies the variant search space (at most `capacity` entries) to `out`
 * and returns its size; out may be NULL to query the size.  The order is
 * fixed: a selector model's outputs index it. */
SPMV_API int spmv_variant_space(spmv_variant_t* out, int capacity);

/* Times every candidate (the whole space when candidates is NULL) as a
 * plan on this matrix: one warm-up, then `repeats` executions (repeats <= 0:
 * as many as fill about 2 ms, 3 to 500), on the handle's stream.  Variants
 * whose warm-up is 20x slower than the best so far keep the warm-up time.
 * msOut[i] = mean milliseconds, or -1 where the variant does not apply
 * (plan creation refused it); *bestIndex = the fastest. */
SPMV_API spmv_status_t spmv_autotune(spmv_handle_t* handle, spmv_type_t type, int numRows, int numCols, int nnz,
                                     const int* rowPtr, const int* colIdx, const void* values,
                                     const spmv_variant_t* candidates, int numCandidates, int repeats,
                                     float* msOut, int* bestIndex);

/* Selector network: in -> h1 -> h2 -> out, ReLU, trained on the GPU with
 * Adam on a masked mean squared error.  X, T, M, Y are DEVICE row-major
 * [batch x in] / [batch x out] arrays; inputs are standardised with the
 * model's mean/std before the first layer.  Parameters are laid out
 * W1[h1 x in], b1, W2[h2 x h1], b2, W3[out x h2], b3. */
typedef struct spmv_mlp_s* spmv_mlp_t;
SPMV_API spmv_status_t spmv_mlp_create(int in, int h1, int h2, int out, unsigned long long seed,
                                       spmv_mlp_t* model);
SPMV_API spmv_status_t spmv_mlp_destroy(spmv_mlp_t model);
SPMV_API int spmv_mlp_num_params(spmv_mlp_t model);
SPMV_API spmv_status_t spmv_mlp_shape(spmv_mlp_t model, int* in, int* h1, int* h2, int* out);
SPMV_API spmv_status_t spmv_mlp_get_params(spmv_mlp_t model, float* host, int count);
SPMV_API spmv_status_t spmv_mlp_set_params(spmv_mlp_t model, const float* host, int count);
/* Host arrays of `in` floats; std entries below 1e-6 are taken as 1. */
SPMV_API spmv_status_t spmv_mlp_set_normalization(spmv_mlp_t model, const float* mean, const float* std);
SPMV_API spmv_status_t spmv_mlp_forward(spmv_mlp_t model, const float* X, float* Y, int batch,
                                        cudaStream_t stream);
/* Loss and gradients of one batch without updating the model; grads is a
 * HOST array of spmv_mlp_num_params floats (may be NULL). Synchronises. */
SPMV_API spmv_status_t spmv_mlp_gradients(spmv_mlp_t model, const float* X, const float* T, const float* M,
                                          int batch, float* loss, float* grads, cudaStream_t stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) at learning rate lr;
 * *loss (if not NULL) receives the batch loss before the step. */
SPMV_API spmv_status_t spmv_mlp_train_step(spmv_mlp_t model, const float* X, const float* T, const float* M,
                                           int batch, float lr, float* loss, cudaStream_t stream);
/* Model file: magic, version, layer sizes, parameters, normalisation and
 * a 64-bit checksum; loading verifies all of them. */
SPMV_API spmv_status_t spmv_mlp_save(spmv_mlp_t model, const char* path);
SPMV_API spmv_status_t spmv_mlp_load(const char* path, spmv_mlp_t* model);

typedef enum {
    SPMV_SELECT_HEURISTIC = 0,     /* the reference's mean-row-length rule      */
    SPMV_SELECT_LEARNED = 1,       /* features + MLP, argmin of predictions     */
    SPMV_SELECT_AUTOTUNE = 2,      /* time the whole space                      */
    SPMV_SELECT_LEARNED_TOPK = 3,  /* time only the model's topK best guesses   */
    SPMV_SELECT_LEARNED_FALLBACK = 4 /* learned pick; when other variants are
                                        predicted within 12% of it (low
                                        confidence), time those too (at most
                                        topK candidates, default 4) and take
                                        the fastest */
} spmv_select_mode_t;

/* Picks a variant for a device CSR matrix.  `model` is needed by the
 * learned modes, `values` by the timing modes.  *spaceIndex = index into
 * spmv_variant_space (-1 when the heuristic's pick is not in the space).
 * Learned modes never return a variant that plan creation would refuse
 * (ELL over 2x padding, unsupported shapes). */
SPMV_API spmv_status_t spmv_select(spmv_handle_t* handle, spmv_select_mode_t mode, spmv_mlp_t model, int topK,
                                   spmv_type_t type, int numRows, int numCols, int nnz, const int* rowPtr,
                                   const int* colIdx, const void* values, spmv_variant_t* out, int* spaceIndex);
/* Registers (model != NULL) or clears a selector model on the handle: FP32
 * plans created with SPMV_KERNEL_AUTO then take the learned pick (the model
 * is trained on FP32 timings; FP64 AUTO plans keep their own rule: one
 * range of tiles per SM on large matrices whose nonzeros mostly lie within
 * 4,096 columns of the diagonal, else 256-nonzero tiles per warp).  The
 * handle borrows the model; it must outlive the handle's use of it. */
SPMV_API spmv_status_t spmv_set_selector(spmv_handle_t* handle, spmv_mlp_t model);
/* How AUTO plans on this handle use the registered model:
 * SPMV_SELECT_LEARNED (default: the model's pick, about 0.15 ms) or
 * SPMV_SELECT_LEARNED_FALLBACK (plan creation also times the variants
 * predicted within 12% of the pick, at most four candidates). */
SPMV_API spmv_status_t spmv_set_selector_mode(spmv_handle_t* handle, spmv_select_mode_t mode);

/* ------------------------------------------------------------------ */
/* Batched SpMV / SpMM over many independent FP32 CSR matrices:          */
/* Y_i = alpha*A_i*X_i + beta*Y_i, X_i numCols_i x k and Y_i numRows_i x k */
/* row-major on the device, k in {1, 2, 4, 8, 16}.  No counterpart in    */
/* the reference (its multi-stream test splits one matrix,               */
/* tests/test_multi_stream.cu:121-236).  The batch borrows the matrices; */
/* colIdx and values must be 16-byte aligned, X_i and Y_i aligned to     */
/* min(k,4)*4 bytes.  Results are deterministic (no atomics).            */
/* ------------------------------------------------------------------ */
typedef struct spmv_batch_s* spmv_batch_t;
typedef struct {
    int numRows;
    int numCols;
    int nnz;
    const int* rowPtr;
    const int* colIdx;
    const float* values;
} spmv_batch_matrix_t;

typedef enum {
    SPMV_BATCH_PERSISTENT = 0,        /* one launch over all matrices (+ fix-up)   */
    SPMV_BATCH_PERSISTENT_GRAPH = 1,  /* the same, replayed from a CUDA graph       */
    SPMV_BATCH_LOOP = 2,              /* one launch per matrix (baseline)           */
    SPMV_BATCH_LOOP_GRAPH = 3         /* the per-matrix loop replayed from a graph  */
} spmv_batch_mode_t;

/* Launch shape of a batch (0 in a field = its default): consecutive
 * nonzeros per slot of lanes (8, or 4; default 8), resident 256-thread blocks
 * per SM the kernel is compiled for (2; 3 with 4 nonzeros per slot; default
 * 2), and nonzeros per work chunk handed to a warp (a multiple of the tile,
 * which is nnzPerSlot * 32 / (k/4 rounded up to 1); default 2048).
 * ordered = 1 (k = 1 only): every matrix is cut into CSR5 tiles of
 * 32 * nnzPerSlot nonzeros (16, default, or 8) and each warp runs one tile
 * with loads and gathers in nonzero order, as a single-matrix plan does
 * (128-thread blocks, blocksPerSM 10 or 8 for 16 nonzeros per lane, 16 or
 * 12 for 8; chunkNnz is ignored), joined by a per-tile carry fix-up. */
typedef struct {
    int nnzPerSlot;
    int blocksPerSM;
    int chunkNnz;
    int ordered;
} spmv_batch_variant_t;

/* `mats` is a host array of `count` descriptors (device pointers).  Builds
 * the tile table (synchronises the handle's stream). */
SPMV_API spmv_status_t spmv_batch_create(spmv_handle_t* handle, int count, const spmv_batch_matrix_t* mats, int k,
                                         spmv_batch_t* batch);
SPMV_API spmv_status_t spmv_batch_create_ex(spmv_handle_t* handle, int count, const spmv_batch_matrix_t* mats,
                                            int k, const spmv_batch_variant_t* variant, spmv_batch_t* batch);
SPMV_API spmv_status_t spmv_batch_get_variant(spmv_batch_t batch, spmv_batch_variant_t* variant);
SPMV_API spmv_status_t spmv_batch_destroy(spmv_batch_t batch);
/* x, y: host arrays of `count` device pointers.  Binds the vectors used by
 * every later execution (graphs stay valid; synchronous copy). */
SPMV_API spmv_status_t spmv_batch_set_vectors_f32(spmv_batch_t batch, const float* const* x, float* const* y);
SPMV_API spmv_status_t spmv_batch_exec_f32(spmv_handle_t* handle, spmv_batch_t batch, float alpha, float beta,
                                           spmv_batch_mode_t mode);
SPMV_API spmv_status_t spmv_batch_info(spmv_batch_t batch, long long* tiles, int* warps, long long* nnzTotal);

/* Batch group: matrices with their own number of right-hand sides k[i]
 * (1, 2, 4, 8 or 16 each).  One batch per distinct k; execution runs them
 * back to back (the graph modes in one graph).  `variants` is NULL or 5 launch
 * shapes, for k = 1, 2, 4, 8 and 16.  x[i] / y[i] are numCols_i x k[i] /
 * numRows_i x k[i], row-major, as for a single batch. */
typedef struct spmv_batch_group_s* spmv_batch_group_t;
SPMV_API spmv_status_t spmv_batch_group_create(spmv_handle_t* handle, int count, const spmv_batch_matrix_t* mats,
                                               const int* k, const spmv_batch_variant_t* variants,
                                               spmv_batch_group_t* group);
SPMV_API spmv_status_t spmv_batch_group_destroy(spmv_batch_group_t group);
SPMV_API spmv_status_t spmv_batch_group_set_vectors_f32(spmv_batch_group_t group, const float* const* x,
                                                        float* const* y);
SPMV_API spmv_status_t spmv_batch_group_exec_f32(spmv_handle_t* handle, spmv_batch_group_t group, float alpha,
                                                 float beta, spmv_batch_mode_t mode);
SPMV_API spmv_status_t spmv_batch_group_info(spmv_batch_group_t group, int* batches, long long* nnzTotal);

/* ------------------------------------------------------------------ */
/* Host-to-host pipeline: x in pinned host memory -> y in pinned host   */
/* memory, with the copies overlapping the SpMV.  Replaces the pinned-  */
/* memory / multi-stream path of tests/test_pinned_memory.cu:245-380    */
/* (testPinnedAsync, testPinnedMultiStream: one stream per row range,   */
/* whole-vector copies before and after the kernels).                   */
/*                                                                      */
/* The matrix (device CSR, borrowed) is cut into `slices` row slices of  */
/* equal rows + nonzeros; slice s of y is copied out as soon as slice s  */
/* is computed, while later slices run.  Up to `depth` requests are in  */
/* flight, each with its own device x and y, so the next request's x    */
/* copy runs under the current SpMV.  Every slice runs the variant       */
/* chosen for the whole matrix (NULL or AUTO: as spmv_plan_create).     */
/* slices <= 0: 1; depth <= 0: 2 (limits 256 and 8).  Throughput comes  */
/* from depth >= 2 (copies hidden under the neighbouring requests);     */
/* slices > 1 shorten one request's latency at about 5 us per slice.    */
/*                                                                      */
/* submit only enqueues work (on the pipeline's own streams): hx must    */
/* stay unchanged and hy unread until spmv_pipeline_wait returns.  With  */
/* pageable host memory the copies are correct but do not overlap.  With */
/* beta != 0 hy is read (copied in) before the request's SpMV.           */
/* ------------------------------------------------------------------ */
typedef struct spmv_pipeline_s* spmv_pipeline_t;

SPMV_API spmv_status_t spmv_pipeline_create(spmv_handle_t* handle, spmv_type_t type, int numRows, int numCols,
                                            int nnz, const int* rowPtr, const int* colIdx, const void* values,
                                            const spmv_variant_t* variant, int slices, int depth,
                                            spmv_pipeline_t* pipeline);
SPMV_API spmv_status_t spmv_pipeline_destroy(spmv_pipeline_t pipeline);
SPMV_API spmv_status_t spmv_pipeline_submit_f32(spmv_pipeline_t pipeline, float alpha, const float* hx, float beta,
                                                float* hy);
SPMV_API spmv_status_t spmv_pipeline_submit_f64(spmv_pipeline_t pipeline, double alpha, const double* hx,
                                                double beta, double* hy);
/* Waits for every submitted request (their hy are then complete). */
SPMV_API spmv_status_t spmv_pipeline_wait(spmv_pipeline_t pipeline);
/* Later submissions start after the work queued on `stream` so far. */
SPMV_API spmv_status_t spmv_pipeline_order_after(spmv_pipeline_t pipeline, cudaStream_t stream);
/* Work queued on `stream` from now on waits for every submitted request. */
SPMV_API spmv_status_t spmv_pipeline_join(spmv_pipeline_t pipeline, cudaStream_t stream);
/* Slices kept (boundaries inside one row are dropped), depth, the slices'
 * variant, device bytes held, kernel launches per request. */
SPMV_API spmv_status_t spmv_pipeline_info(spmv_pipeline_t pipeline, int* slices, int* depth,
                                          spmv_variant_t* variant, size_t* deviceBytes, int* launchesPerRequest);

#ifdef __cplusplus
}
#endif

#endif /* MUXI_SPMV_H_ */
