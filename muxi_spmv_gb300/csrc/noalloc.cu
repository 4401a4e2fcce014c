// spmv_csr_noalloc_f32: a stateless FP32 CSR SpMV (merge-path tiles plus
// carry fix-up: spmv_csr_f32's kernels when that call is given the
// SPMV_KERNEL_MERGE variant {256, 0, 8, 4}) for callers that must not
// allocate device memory.  Examples: code running under a strict
// device-memory budget owned by another allocator, a real-time loop where an
// allocation (and the synchronisation it can cause) is not allowed, or a
// library callback that has no allocator handed to it.
//
// The tile coordinates and carries live in one file-scope device array of
// kNoAllocScratchBytes.  Every GPU that loads this library reserves that
// array for the life of the process.  Its device address is looked up with
// cudaGetSymbolAddress once per device, on the first call made with that
// device current.  The address stays cached for the process: after a cudaDeviceReset the module is
// reloaded and the array may move, so do not call this entry point on a
// device that has been reset.
#include <mutex>
#include <vector>

#include "internal.h"
#include "kernels.h"

namespace mxs {
namespace {

// 8 MiB: 16 bytes per merge tile (plus alignment), so up to 524,224 tiles:
// numRows + nnz up to about 1.07e9 with 16-byte-aligned colIdx / values
// (2,044-item tiles), about 0.94e9 otherwise (1,792-item tiles).
constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;

// Largest numRows + nnz the array serves with tiles of geometry g.
long long max_items(const MergeGeom& g) {
    long long P = (long long)(kNoAllocScratchBytes / 16);
    while (P > 1 && merge_scratch_bytes(P, sizeof(float)) > kNoAllocScratchBytes) --P;
    return P * g.tile();
}
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
std::vector<void*> g_addr;  // per device; nullptr until looked up

spmv_status_t scratch_address(void** out) {
    int dev = 0;
    MXS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_addr.size() <= dev) g_addr.resize(dev + 1, nullptr);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)", __FILE__, __LINE__);
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return SPMV_SUCCESS;
}

}  // namespace
}  // namespace mxs

using namespace mxs;

extern "C" spmv_status_t spmv_csr_noalloc_f32(int numRows, int numCols, int nnz, const int* rowPtr,
                                              const int* colIdx, const float* values, const float* x, float* y,
                                              float alpha, float beta, cudaStream_t stream) {
    clear_error();
    if (numRows < 0 || numCols < 0 || nnz < 0)
        MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension (R=%d C=%d nnz=%d)", numRows, numCols, nnz);
    MergeGeom g{256, 8, 4};
    if (nnz > 0 && !(aligned16(colIdx) && aligned16(values))) g = merge_unaligned_geom(g);
    const long long tiles = merge_tile_count(numRows, nnz, g);
    const size_t need = merge_scratch_bytes(tiles, sizeof(float));
    if (need > kNoAllocScratchBytes)
        MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC,
                 "matrix needs %zu bytes of scratch (%lld merge tiles); the no-allocation entry point has a fixed "
                 "%zu-byte array (numRows + nnz up to %lld for this call's colIdx / values alignment)",
                 need, tiles, kNoAllocScratchBytes, max_items(g));
    if (numRows > 0 && (!rowPtr || !y)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr or y is NULL");
    if (nnz > 0 && (!colIdx || !values || !x)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx, values or x is NULL");
    if (numRows == 0) return SPMV_SUCCESS;
    if (nnz == 0) return run_scale<float>(numRows, y, beta, stream);
    void* base = nullptr;
    MXS_TRY(scratch_address(&base));
    // Nothing in the array needs to start at zero: the coordinate kernel
    // writes all tiles+1 entries and every tile writes its carry.
    const MergeScratch sc = merge_carve(base, tiles, sizeof(float));
    MXS_TRY(merge_tile_coords(rowPtr, numRows, nnz, g, tiles, sc.tileRow, sc.tileNnz, stream));
    const RowsArgs<float> a{numRows, nnz, rowPtr, colIdx, values, x, y, alpha, beta, beta == 0.0f};
    return run_merge<float>(g, tiles, sc, a, stream);
}
