// Launch wrappers exported by the kernel translation units to api.cu.
#pragma once

#include <cuda_runtime.h>
#include "muxi_spmv.h"

namespace mxs {

template <typename T>
struct RowsArgs {
    int numRows;
    int nnz;
    const int* rowPtr;
    const int* colIdx;
    const T* values;
    const T* x;
    T* y;
    T alpha;
    T beta;
    int betaZero;
    int noEmptyRows = 0;  // set by plans that checked every row holds a nonzero
};

// Scalar / vector CSR kernels (csr_kernels.cu).
template <typename T>
spmv_status_t run_rows(int block, int tpr, int vec, const RowsArgs<T>& a, cudaStream_t s);
// y = beta*y.
template <typename T>
spmv_status_t run_scale(long long n, T* y, T beta, cudaStream_t s);

// ---- merge path (merge_kernels.cu) ----
// Merge-path tile geometry for a given block size / items per thread.
// vec == 0: per-item merge consumer (ipt merge items per thread).
// vec == 4: nonzero-vectorised consumer (ipt consecutive nonzeros per thread,
//           16-byte loads); a tile holds block*ipt - 4 merge items so the
//           16-byte-aligned cover of its nonzeros fits the CTA.
struct MergeGeom {
    int block;
    int ipt;
    int vec = 0;
    long long tile() const { return (long long)block * ipt - (vec ? 4 : 0); }
};
// Builds the geometry of a MERGE variant (defaults filled in).
MergeGeom merge_geom_of(const spmv_variant_t& v);
bool merge_geom_supported(const MergeGeom& g);
// The per-item consumer with the same block size: what runs when a 16-byte
// vectorised geometry meets colIdx / values that are not 16-byte aligned.
inline MergeGeom merge_unaligned_geom(const MergeGeom& g) { return MergeGeom{g.block, 7, 0}; }
// Number of tiles for a matrix: ceil((R+N)/tile), at least 1.
long long merge_tile_count(int numRows, int nnz, const MergeGeom& g);
// Bytes of scratch the merge path needs for P tiles and value size vsize:
// (P+1) start rows, (P+1) start nnz, P carry rows, P carry values.
size_t merge_scratch_bytes(long long P, size_t vsize);

struct MergeScratch {
    int* tileRow;   // P+1
    int* tileNnz;   // P+1
    int* carryRow;  // P
    void* carryVal; // P values
};
// Carves the four arrays out of one buffer of merge_scratch_bytes().
MergeScratch merge_carve(void* base, long long P, size_t vsize);

// Tile start coordinates: diagonal min(t*tile, R+N) for t = 0..P.
spmv_status_t merge_tile_coords(const int* rowPtr, int numRows, int nnz, const MergeGeom& g,
                                long long P, int* tileRow, int* tileNnz, cudaStream_t s);

// Tile kernel then carry fix-up; `afterMain` (optional) is recorded between them.
template <typename T>
spmv_status_t run_merge(const MergeGeom& g, long long P, const MergeScratch& sc, const RowsArgs<T>& a,
                        cudaStream_t s, cudaEvent_t afterMain = nullptr);

// Carry fix-up of a merge-path launch (adds carries of split rows in tile order).
template <typename T>
spmv_status_t run_merge_fixup(long long P, const MergeScratch& sc, const RowsArgs<T>& a, cudaStream_t s);

// Range length (tiles per CTA) of a block-range launch: about `target`
// tiles, adjusted so that the CTA count is a whole number of waves of
// `resident` CTAs (CTAs of equal nonzero counts then end together); at least
// `minPer`.
inline long long fitted_range(long long tiles, long long target, long long resident, long long minPer) {
    if (resident < 1) resident = 1;
    if (target < 1) target = 1;
    long long waves = (tiles + target * resident - 1) / (target * resident);
    if (waves < 1) waves = 1;
    const long long per = (tiles + waves * resident - 1) / (waves * resident);
    return per < minPer ? minPer : per;
}

// Reference-compatible partitioning (spmv_csr5.cu:912-925) and search (:497-533).
spmv_status_t merge_partitions(int numRows, int nnz, int P, int* pos, cudaStream_t s);
spmv_status_t merge_search(const int* rowPtr, int numRows, int nnz, const int* diag, int count,
                           int* rowIdx, int* nnzIdx, cudaStream_t s);

// ---- statistics (stats_kernels.cu) ----
spmv_status_t count_distinct_columns(int numCols, int nnz, const int* colIdx, long long* out,
                                     cudaStream_t s);
spmv_status_t validate_csr(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                           long long* bad, cudaStream_t s);

// Stream-ordered scratch from the library's per-device memory pool.
spmv_status_t scratch_alloc(void** p, size_t bytes, cudaStream_t s);
spmv_status_t scratch_free(void* p, cudaStream_t s);

}  // namespace mxs
