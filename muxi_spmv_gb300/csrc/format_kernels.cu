// SpMV over the CSR5 tile metadata and over column-major ELLPACK.
//
// CSR5 (reference: spmv_csr5_warp32_kernel, src/spmv/csr5/spmv_csr5.cu:148-219)
// gives every warp one tile of sigma consecutive nonzeros.  The reference
// gives each lane sigma/32 contiguous nonzeros, searches every lane's row in
// global memory and adds every row change with a float atomic (results vary
// run to run).  Here:
//   * a lane's sigma/32 nonzeros are one or two aligned 16-byte loads (the tile
//     start t*sigma is a multiple of 128 elements);
//   * the lane's first row is searched only inside [tile_row_ptr[t],
//     tile_row_ptr[t+1]];
//   * rows are summed per lane, joined across lanes by a segmented warp scan,
//     and a row that runs past the tile end leaves a carry that a second
//     kernel adds in tile order -- no atomics;
//   * empty rows get y = beta*y from the tile whose row range holds them.
//
// ELL (reference: spmv_ellpack_kernel, src/spmv/ellpack/spmv_ellpack.cuh:85-111)
// keeps one thread per row over column-major slots (coalesced by layout) and
// adds streaming loads, unrolled slots and the alpha/beta epilogue.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "formats.h"
#include "csr5_tile.cuh"
#include "csr5_ordered.cuh"
#include "sort.h"

namespace mxs {

template <typename T, int E>
__global__ void __launch_bounds__(256)
csr5_tile_kernel(int numRows, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                 const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                 int betaZero, const int* __restrict__ tileRow, long long tiles, int* __restrict__ carryRow,
                 T* __restrict__ carryVal) {
    __shared__ int sRp[8][csr5_rp_cap<E>()];
    const long long t = ((long long)blockIdx.x * 256 + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= tiles) return;  // uniform per warp
    Csr5Load<T, E> L;
    csr5_load<T, E>(L, t, lane, nnz, tiles, numRows, tileRow, rowPtr, colIdx, values);
    csr5_compute<T, E>(L, t, lane, numRows, nnz, rowPtr, y, alpha, beta, betaZero != 0, carryRow, carryVal,
                       sRp[threadIdx.x >> 5], [x](int c) { return ld_x(x + c); });
}

// Row-start masks of a CSR5 tiling (see csr5_tile_rows_bits); matrices
// without empty rows only.  bits: tiles * E words, zeroed before.
__global__ void tile_bits_kernel(const int* __restrict__ rowPtr, int numRows, int sigma, int words, long long tiles,
                                 unsigned* __restrict__ bits) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) atomicOr(bits + (tiles - 1) * words, 1u);  // the last tile's last row ends at its end
    if (r < 1 || r >= numRows) return;
    const int pos = rowPtr[r];
    const long long t = pos / sigma;
    const int k = pos - (int)(t * sigma);
    if (k) atomicOr(bits + t * words + (k >> 5), 1u << (k & 31));
    else atomicOr(bits + (t - 1) * words, 1u);  // row r starts tile t: tile t-1's last row ends at its end
}

spmv_status_t csr5_tile_bits(const int* rowPtr, int numRows, int sigma, long long tiles, void** buf, cudaStream_t s) {
    *buf = nullptr;
    if (tiles <= 0) return SPMV_SUCCESS;
    const int words = sigma / 32;
    const size_t bytes = sizeof(unsigned) * (size_t)tiles * words;
    MXS_CUDA(dev_malloc(buf, bytes));
    cudaError_t e = cudaMemsetAsync(*buf, 0, bytes, s);
    if (e == cudaSuccess) {
        tile_bits_kernel<<<grid_for(numRows > 0 ? numRows : 1, 256), 256, 0, s>>>(rowPtr, numRows, sigma, words,
                                                                                 tiles, static_cast<unsigned*>(*buf));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        dev_free(*buf);
        *buf = nullptr;
        return cuda_fail(e, "tile row masks", __FILE__, __LINE__);
    }
    return SPMV_SUCCESS;
}

// One tile per warp, BLOCK threads per block, MINB resident blocks per SM
// (the launch bound sets the register budget: 128x16, 512x4 and 1024x2 keep
// 64 warps per SM at 32 registers, 256x6 keeps 48 at 40).  Larger blocks put
// more consecutive tiles on one SM, so their gathers share that SM's L1.
template <typename T, int E, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB)
csr5_ordered_kernel(int numRows, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                    const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                    int betaZero, const int* __restrict__ tileRow, long long tiles, int* __restrict__ carryRow,
                    T* __restrict__ carryVal, int noEmptyRows, const unsigned* __restrict__ tileBits) {
    constexpr int WARPS = BLOCK / 32;
    __shared__ int sRpAll[WARPS][kOrderedRpCap];
    __shared__ __align__(16) T sPAll[WARPS][ordered_slots<T, E>()];
    pdl_trigger();  // the carry fix-up may be scheduled behind the last wave
    const long long t = ((long long)blockIdx.x * BLOCK + threadIdx.x) >> 5;
    if (t >= tiles) return;  // uniform per warp
    const int w = threadIdx.x >> 5;
    csr5_ordered_tile<T, E>(t, threadIdx.x & 31, numRows, nnz, rowPtr, colIdx, values, x, y, alpha, beta,
                            betaZero != 0, tileRow, tiles, carryRow, carryVal, noEmptyRows != 0, tileBits, sRpAll[w],
                            sPAll[w], betaZero == kPlainAxpby);
}

// Block ranges: block b owns the `perBlock` consecutive tiles from
// b*perBlock; its warps take them one at a time from a shared counter, so the
// warps of a block work on neighbouring rows (the near-diagonal x they gather
// stays in the SM's L1) and a warp that drew short tiles takes more of them
// (no block waits for a slow tile while others idle, as one-tile-per-warp
// launches of large blocks do).
// PREFETCH: the next tile's column indices and values are requested before
// the current tile's gathers and row logic (a second tile's loads held in
// registers), so the matrix stream's memory latency overlaps this tile's work
// instead of preceding it.
template <typename T, int E, int BLOCK, int MINB, bool PREFETCH = false>
__global__ void __launch_bounds__(BLOCK, MINB)
csr5_ordered_range_kernel(int numRows, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                          const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                          int betaZero, const int* __restrict__ tileRow, long long tiles, int* __restrict__ carryRow,
                          T* __restrict__ carryVal, int noEmptyRows, int perBlock,
                          const unsigned* __restrict__ tileBits) {
    constexpr int WARPS = BLOCK / 32;
    __shared__ int sRpAll[WARPS][kOrderedRpCap];
    __shared__ __align__(16) T sPAll[WARPS][ordered_slots<T, E>()];
    __shared__ int sNext, sEnd;  // next tile to hand out, end of the range (shared: fewer live registers)
    pdl_trigger();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Tile counts fit in int: plans cap nnz below 2^31.
    int t = blockIdx.x * perBlock + w;
    if (threadIdx.x == 0) {
        sNext = blockIdx.x * perBlock + WARPS;
        sEnd = min(blockIdx.x * perBlock + perBlock, (int)tiles);
    }
    __syncthreads();
    if constexpr (PREFETCH) {
        const int end = sEnd;
        OrderedLoad<T, E> cur, nxt;
        if (t < end) csr5_ordered_load<T, E>(cur, t, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
        while (t < end) {
            int next = 0;
            if (lane == 0) next = atomicAdd(&sNext, 1);
            next = __shfl_sync(0xffffffffu, next, 0);
            if (next < end)
                csr5_ordered_load<T, E>(nxt, next, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
            csr5_ordered_compute<T, E, true>(cur, t, lane, nnz, rowPtr, GlobalGather<T>{x}, y, alpha, beta,
                                             betaZero != 0, tiles, carryRow, carryVal, noEmptyRows != 0, sRpAll[w],
                                             sPAll[w], tileBits != nullptr, betaZero == kPlainAxpby);
            cur = nxt;
            t = next;
        }
        return;
    }
    while (t < sEnd) {
        OrderedLoad<T, E> L;
        csr5_ordered_load<T, E>(L, t, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
        int next = 0;  // drawn before the compute so its latency hides under the loads
        if (lane == 0) next = atomicAdd(&sNext, 1);
        csr5_ordered_compute<T, E, true>(L, t, lane, nnz, rowPtr, GlobalGather<T>{x}, y, alpha, beta, betaZero != 0, tiles,
                                         carryRow, carryVal, noEmptyRows != 0, sRpAll[w], sPAll[w],
                                         tileBits != nullptr, betaZero == kPlainAxpby);
        t = __shfl_sync(0xffffffffu, next, 0);
    }
}

// Row still open at the end of each tile (-1 if the tile's last row ends in it).
__global__ void carry_rows_kernel(const int* __restrict__ rowPtr, int numRows, int nnz, int sigma,
                                  const int* __restrict__ tileRow, long long tiles, int* __restrict__ carry) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    const long long tEnd = (t + 1) * sigma < nnz ? (t + 1) * sigma : nnz;
    int lo = tileRow[t], hi = t + 1 < tiles ? tileRow[t + 1] : numRows - 1;
    while (lo < hi) {  // last row with rowPtr <= tEnd - 1: the row holding the tile's last nonzero
        const int mid = (lo + hi + 1) >> 1;
        if (rowPtr[mid] <= tEnd - 1) lo = mid;
        else hi = mid - 1;
    }
    carry[t] = rowPtr[lo + 1] > tEnd ? lo : -1;
}

__global__ void chain_flags_kernel(const int* __restrict__ carry, long long tiles, unsigned* __restrict__ isStart,
                                   unsigned* __restrict__ isEnd) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    const int c = carry[t];
    isStart[t] = c >= 0 && (t == 0 || carry[t - 1] != c);
    isEnd[t] = c >= 0 && (t + 1 == tiles || carry[t + 1] != c);
}

__global__ void chain_compact_kernel(const int* __restrict__ carry, const unsigned* __restrict__ isStart,
                                     const unsigned* __restrict__ startPos, const unsigned* __restrict__ isEnd,
                                     const unsigned* __restrict__ endPos, long long tiles, int* __restrict__ start,
                                     int* __restrict__ end, int* __restrict__ row) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    if (isStart[t]) {
        start[startPos[t]] = (int)t;
        row[startPos[t]] = carry[t];
    }
    if (isEnd[t]) end[endPos[t]] = (int)t;
}

spmv_status_t csr5_chains(const int* rowPtr, int numRows, int nnz, int sigma, const int* tileRow, long long tiles,
                          void** buf, Csr5Chains* out, cudaStream_t s) {
    *buf = nullptr;
    out->n = 0;
    if (tiles <= 0) return SPMV_SUCCESS;
    void* tmp = nullptr;
    const size_t a = ((sizeof(unsigned) * tiles) + 255) & ~size_t(255);
    MXS_TRY(scratch_alloc(&tmp, 5 * a + 256, s));
    char* b = static_cast<char*>(tmp);
    int* carry = reinterpret_cast<int*>(b);
    unsigned* isStart = reinterpret_cast<unsigned*>(b + a);
    unsigned* isEnd = reinterpret_cast<unsigned*>(b + 2 * a);
    unsigned* startPos = reinterpret_cast<unsigned*>(b + 3 * a);
    unsigned* endPos = reinterpret_cast<unsigned*>(b + 4 * a);
    unsigned* total = reinterpret_cast<unsigned*>(b + 5 * a);
    const unsigned g = grid_for(tiles, 256);
    carry_rows_kernel<<<g, 256, 0, s>>>(rowPtr, numRows, nnz, sigma, tileRow, tiles, carry);
    chain_flags_kernel<<<g, 256, 0, s>>>(carry, tiles, isStart, isEnd);
    spmv_status_t st = cudaGetLastError() == cudaSuccess ? SPMV_SUCCESS : SPMV_ERROR_DEVICE;
    if (st == SPMV_SUCCESS) st = scan_exclusive_u32(isStart, startPos, tiles, total, s);
    unsigned n = 0;
    if (st == SPMV_SUCCESS) st = scan_exclusive_u32(isEnd, endPos, tiles, nullptr, s);
    if (st == SPMV_SUCCESS) {
        cudaError_t e = cudaMemcpyAsync(&n, total, sizeof(n), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "carry chains", __FILE__, __LINE__);
    }
    if (st == SPMV_SUCCESS && n > 0) {
        cudaError_t e = dev_malloc(buf, 3 * sizeof(int) * (size_t)n);
        if (e != cudaSuccess) {
            *buf = nullptr;
            st = cuda_fail(e, "carry chain table", __FILE__, __LINE__);
        } else {
            int* start = static_cast<int*>(*buf);
            chain_compact_kernel<<<g, 256, 0, s>>>(carry, isStart, startPos, isEnd, endPos, tiles, start, start + n,
                                                   start + 2 * n);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) st = cuda_fail(e, "carry chains", __FILE__, __LINE__);
            out->start = start;
            out->end = start + n;
            out->row = start + 2 * n;
        }
    }
    scratch_free(tmp, s);
    if (st != SPMV_SUCCESS) {
        if (*buf) dev_free(*buf);
        *buf = nullptr;
        out->n = -1;
        return st;
    }
    out->n = n;
    return SPMV_SUCCESS;
}

// Adds each chain's carries to its row.  A thread sums a chain of up to
// kShortChain tiles in tile order; a longer chain (a row over more tiles) is
// queued in shared memory and summed by a whole warp: lane-strided partial
// sums, then the butterfly of group_sum.  Which warp takes a queued chain
// varies, but each chain's order of additions is fixed, so results are
// identical run to run -- and one 65,536-nonzero row no longer makes a single
// thread walk 256 carries while the rest of the GPU idles.
constexpr int kShortChain = 8;
template <typename T>
__global__ void __launch_bounds__(256)
csr5_chain_fixup_kernel(long long chains, const int* __restrict__ start, const int* __restrict__ end,
                        const int* __restrict__ row, const T* __restrict__ carryVal, T* __restrict__ y, T alpha) {
    __shared__ int sLong[256];
    __shared__ int sCount;
    pdl_wait();  // the tile kernel's carries and y are complete
    if (threadIdx.x == 0) sCount = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * 256;
    const long long c = base + threadIdx.x;
    if (c < chains) {
        const int b = start[c], e = end[c];
        if (e - b < kShortChain) {
            T s = T(0);
#pragma unroll 4
            for (int u = b; u <= e; ++u) s += carryVal[u];
            y[row[c]] += alpha * s;
        } else {
            sLong[atomicAdd(&sCount, 1)] = threadIdx.x;
        }
    }
    __syncthreads();
    const int n = sCount, lane = threadIdx.x & 31;
    for (int i = threadIdx.x >> 5; i < n; i += 8) {
        const long long cc = base + sLong[i];
        const int b = start[cc], e = end[cc];
        T s = T(0);
        for (int u = b + lane; u <= e; u += 32) s += carryVal[u];
        s = group_sum<32>(s);
        if (lane == 0) y[row[cc]] += alpha * s;
    }
}

// Adds each split row's carries (rows with carry -1 skipped), for callers
// without a chain table: the thread at the first tile of a run of equal
// carry rows walks it.  Runs of up to kShortChain tiles are summed in tile
// order by that thread; longer ones go to a warp exactly as in
// csr5_chain_fixup_kernel (same additions, so both fix-ups give the same bits).
template <typename T>
__global__ void __launch_bounds__(256)
csr5_fixup_kernel(long long tiles, const int* __restrict__ carryRow, const T* __restrict__ carryVal,
                  T* __restrict__ y, T alpha) {
    __shared__ int sLong[256];
    __shared__ int sCount;
    pdl_wait();
    if (threadIdx.x == 0) sCount = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * 256;
    const long long t = base + threadIdx.x;
    if (t < tiles) {
        const int r = carryRow[t];
        if (r >= 0 && (t == 0 || carryRow[t - 1] != r)) {
            T s = T(0);
            long long u = t;
            for (; u < tiles && u - t < kShortChain && carryRow[u] == r; ++u) s += carryVal[u];
            if (u - t == kShortChain && u < tiles && carryRow[u] == r)
                sLong[atomicAdd(&sCount, 1)] = threadIdx.x;
            else
                y[r] += alpha * s;
        }
    }
    __syncthreads();
    const int n = sCount, lane = threadIdx.x & 31;
    for (int i = threadIdx.x >> 5; i < n; i += 8) {
        const long long t0 = base + sLong[i];
        const int r = carryRow[t0];
        T s = T(0);
        for (long long b = t0;; b += 32) {  // the run is contiguous: its lanes form a prefix
            const long long u = b + lane;
            const bool in = u < tiles && carryRow[u] == r;
            if (in) s += carryVal[u];
            if (!__all_sync(kFull, in)) break;
        }
        s = group_sum<32>(s);
        if (lane == 0) y[r] += alpha * s;
    }
}

// Block-range launch: about `chunk` tiles per warp, fitted so the CTAs fill
// whole waves of the CTAs resident at once (a chunk beyond tiles / resident
// gives one range per resident CTA: each SM works through contiguous ranges).
template <typename T, int E, int B, int M, bool PF = false>
static spmv_status_t launch_range(const int* tileRow, long long tiles, int* carryRow, T* carryVal,
                                  const RowsArgs<T>& a, int chunk, const unsigned* bits, int bzFlags, cudaStream_t s) {
    auto kern = csr5_ordered_range_kernel<T, E, B, M, PF>;
    int perSm = 0;
    MXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, B, 0));
    const long long resident = (long long)(perSm > 0 ? perSm : 1) * current_sm_count();
    const long long per = fitted_range(tiles, (long long)chunk * (B / 32), resident, B / 32);
    if (per > 0x7fffffffLL) MXS_FAIL(SPMV_ERROR_INTERNAL, "CSR5 block range too large");
    kern<<<grid_for(tiles, (int)per), B, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha,
                                                 a.beta, bzFlags, tileRow, tiles, carryRow, carryVal, a.noEmptyRows,
                                                 (int)per, bits);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

template <typename T, int E>
static spmv_status_t launch_ordered(const int* tileRow, long long tiles, int* carryRow, T* carryVal,
                                    const RowsArgs<T>& a, int block, int chunk, const unsigned* bits, cudaStream_t s,
                                    bool prefetch) {
    const int bzFlags = a.betaZero ? (a.alpha == T(1) ? kPlainAxpby : 1) : 0;
    if (chunk <= 0) {
        constexpr bool wide = E * sizeof(T) >= 64;  // 16 doubles or floats per lane: fewer, larger blocks
#define MXS_ORDERED(B, M)                                                                                        \
    csr5_ordered_kernel<T, E, B, M><<<grid_for(tiles * 32, B), B, 0, s>>>(                                        \
        a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha, a.beta, bzFlags, tileRow, tiles,   \
        carryRow, carryVal, a.noEmptyRows, bits)
        switch (block) {
            // 16 four-byte or 8 eight-byte values per lane: 10 blocks (48
            // registers, 40 warps) measured best; 16 doubles (the FP64 FMA
            // hand-off holds a lane's 16 values) fit 96 registers at 5.
            case 128: MXS_ORDERED(128, E * sizeof(T) >= 128 ? 5 : (wide ? 10 : 16)); break;
            case 256: MXS_ORDERED(256, E * sizeof(T) >= 128 ? 3 : (wide ? 5 : 6)); break;
            case 512: MXS_ORDERED(512, wide ? 2 : 4); break;
            case 1024: MXS_ORDERED(1024, wide ? 1 : 2); break;
            default: MXS_FAIL(SPMV_ERROR_INTERNAL, "ordered CSR5 block must be 128, 256, 512 or 1024 (got %d)", block);
        }
#undef MXS_ORDERED
        return SPMV_SUCCESS;
    }
    if (prefetch) {  // block ranges with the next tile's loads in flight (two tiles' loads in registers)
        constexpr bool small = E * sizeof(T) <= 32;  // 8 four-byte values per lane: two 512-thread blocks fit
        switch (block) {
            case 512:
                if constexpr (small) return launch_range<T, E, 512, 2, true>(tileRow, tiles, carryRow, carryVal, a, chunk, bits, bzFlags, s);
                else return launch_range<T, E, 512, 1, true>(tileRow, tiles, carryRow, carryVal, a, chunk, bits, bzFlags, s);
            case 768: return launch_range<T, E, 768, 1, true>(tileRow, tiles, carryRow, carryVal, a, chunk, bits, bzFlags, s);
            case 1024: return launch_range<T, E, 1024, 1, true>(tileRow, tiles, carryRow, carryVal, a, chunk, bits, bzFlags, s);
            default: MXS_FAIL(SPMV_ERROR_INTERNAL, "prefetching block ranges need 512, 768 or 1024 threads (got %d)", block);
        }
    }
    // Block ranges of about `chunk` tiles per warp.  Resident blocks per SM
    // (the register budget): 16 four-byte or 8 eight-byte values per lane
    // ("wide") take the first figure, smaller tiles the second.
    constexpr bool wide = E * sizeof(T) >= 64;
#define MXS_RANGE(B, MW, MN)                                                                                    \
    if constexpr (wide) return launch_range<T, E, B, MW>(tileRow, tiles, carryRow, carryVal, a, chunk, bits,   \
                                                         bzFlags, s);                                          \
    else return launch_range<T, E, B, MN>(tileRow, tiles, carryRow, carryVal, a, chunk, bits, bzFlags, s)
    switch (block) {
        case 256: MXS_RANGE(256, 3, 8);
        case 384: MXS_RANGE(384, 3, 5);
        case 512: MXS_RANGE(512, 2, 4);
        case 640: MXS_RANGE(640, 2, 3);
        case 1024: MXS_RANGE(1024, 1, 2);
        default: MXS_FAIL(SPMV_ERROR_INTERNAL, "block-range CSR5 block must be 256, 384, 512, 640 or 1024 (got %d)", block);
    }
#undef MXS_RANGE
}

template <typename T>
spmv_status_t run_csr5(int sigma, const int* tileRow, long long tiles, int* carryRow, T* carryVal,
                       const RowsArgs<T>& a, cudaStream_t s, cudaEvent_t afterMain, bool ordered, int block,
                       int chunk, const Csr5Chains* chains, const unsigned* tileBits, bool prefetch) {
    // The lane-contiguous kernel reads 16-byte quads; on arrays that are not
    // 16-byte aligned the ordered kernel (4-byte loads) runs the same tiles.
    if (!ordered && !(aligned16(a.colIdx) && aligned16(a.values))) {
        ordered = true;
        block = 128;
        chunk = 0;
        tileBits = nullptr;
    }
    if (ordered) {
        if (sigma == 128) MXS_TRY((launch_ordered<T, 4>(tileRow, tiles, carryRow, carryVal, a, block, chunk, tileBits, s, prefetch)));
        else if (sigma == 256) MXS_TRY((launch_ordered<T, 8>(tileRow, tiles, carryRow, carryVal, a, block, chunk, tileBits, s, prefetch)));
        else if (sigma == 512) MXS_TRY((launch_ordered<T, 16>(tileRow, tiles, carryRow, carryVal, a, block, chunk, tileBits, s, prefetch)));
        else MXS_FAIL(SPMV_ERROR_INTERNAL, "CSR5 sigma must be 128, 256 or 512 (got %d)", sigma);
    } else {
        const unsigned g = grid_for(tiles * 32, 256);
        if (sigma == 128) {
            csr5_tile_kernel<T, 4><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y,
                                                     a.alpha, a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
        } else if (sigma == 256) {
            csr5_tile_kernel<T, 8><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y,
                                                     a.alpha, a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
        } else if (sigma == 512) {
            csr5_tile_kernel<T, 16><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y,
                                                      a.alpha, a.beta, a.betaZero, tileRow, tiles, carryRow,
                                                      carryVal);
        } else {
            MXS_FAIL(SPMV_ERROR_INTERNAL, "CSR5 sigma must be 128, 256 or 512 (got %d)", sigma);
        }
    }
    MXS_LAUNCH_CHECK();
    // the lane-contiguous kernel does not trigger a programmatic launch
    return run_csr5_fixups<T>(tiles, carryRow, carryVal, a, s, afterMain, chains, ordered);
}

template <typename T>
spmv_status_t run_csr5_fixups(long long tiles, const int* carryRow, const T* carryVal, const RowsArgs<T>& a,
                              cudaStream_t s, cudaEvent_t afterMain, const Csr5Chains* chains, bool programmatic) {
    if (afterMain) MXS_CUDA(cudaEventRecord(afterMain, s));
    // Right behind an ordered tile kernel (no event between them) the fix-up
    // launches programmatically: its blocks are scheduled while the tile
    // kernel's last wave runs and start when it completes.
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(256);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (programmatic && !afterMain) ? 1 : 0;
    if (chains && chains->n >= 0) {
        if (chains->n > 0) {
            cfg.gridDim = dim3(grid_for(chains->n, 256));
            MXS_CUDA(cudaLaunchKernelEx(&cfg, csr5_chain_fixup_kernel<T>, (long long)chains->n,
                                        (const int*)chains->start, (const int*)chains->end, (const int*)chains->row,
                                        (const T*)carryVal, a.y, a.alpha));
        }
        return SPMV_SUCCESS;
    }
    cfg.gridDim = dim3(grid_for(tiles, 256));
    MXS_CUDA(cudaLaunchKernelEx(&cfg, csr5_fixup_kernel<T>, tiles, (const int*)carryRow, (const T*)carryVal, a.y,
                                a.alpha));
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t run_csr5_fixup(long long tiles, const int* carryRow, const T* carryVal, const RowsArgs<T>& a,
                             cudaStream_t s) {
    csr5_fixup_kernel<T><<<grid_for(tiles, 256), 256, 0, s>>>(tiles, carryRow, carryVal, a.y, a.alpha);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
template spmv_status_t run_csr5_fixup<float>(long long, const int*, const float*, const RowsArgs<float>&,
                                             cudaStream_t);
template spmv_status_t run_csr5_fixup<double>(long long, const int*, const double*, const RowsArgs<double>&,
                                              cudaStream_t);
template spmv_status_t run_csr5_fixups<float>(long long, const int*, const float*, const RowsArgs<float>&,
                                              cudaStream_t, cudaEvent_t, const Csr5Chains*, bool);
template spmv_status_t run_csr5_fixups<double>(long long, const int*, const double*, const RowsArgs<double>&,
                                               cudaStream_t, cudaEvent_t, const Csr5Chains*, bool);
template spmv_status_t run_csr5<float>(int, const int*, long long, int*, float*, const RowsArgs<float>&,
                                       cudaStream_t, cudaEvent_t, bool, int, int, const Csr5Chains*,
                                       const unsigned*, bool);
template spmv_status_t run_csr5<double>(int, const int*, long long, int*, double*, const RowsArgs<double>&,
                                        cudaStream_t, cudaEvent_t, bool, int, int, const Csr5Chains*,
                                        const unsigned*, bool);

// ---------------------------------------------------------------------------
// ELL
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256)
ell_kernel(int numRows, int width, const int* __restrict__ ellCol, const T* __restrict__ ellVal,
           const T* __restrict__ x, T* __restrict__ y, T alpha, T beta, int betaZero) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= numRows) return;
    T sum = T(0);
    int i = 0;
    for (; i + 4 <= width; i += 4) {
        int c[4];
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long idx = r + (long long)(i + u) * numRows;
            c[u] = ld_stream(ellCol + idx);
            v[u] = ld_stream(ellVal + idx);
        }
        // Padding (col -1) gathers x[0] and discards it: unconditional
        // gathers keep the four loads in flight together.
        T g[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) g[u] = ld_x(x + (c[u] >= 0 ? c[u] : 0));
#pragma unroll
        for (int u = 0; u < 4; ++u) sum += c[u] >= 0 ? v[u] * g[u] : T(0);
    }
    for (; i < width; ++i) {
        const long long idx = r + (long long)i * numRows;
        const int c = ld_stream(ellCol + idx);
        const T v = ld_stream(ellVal + idx);
        const T g = ld_x(x + (c >= 0 ? c : 0));
        sum += c >= 0 ? v * g : T(0);
    }
    y[r] = axpby(alpha, sum, beta, betaZero != 0, y + r);
}

template <typename T>
spmv_status_t run_ell(int numRows, int width, const int* ellCol, const T* ellVal, const T* x, T* y, T alpha, T beta,
                      cudaStream_t s) {
    if (numRows <= 0) return SPMV_SUCCESS;
    if (width == 0) return run_scale<T>(numRows, y, beta, s);
    ell_kernel<T><<<grid_for(numRows, 256), 256, 0, s>>>(numRows, width, ellCol, ellVal, x, y, alpha, beta,
                                                         beta == T(0));
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
template spmv_status_t run_ell<float>(int, int, const int*, const float*, const float*, float*, float, float,
                                      cudaStream_t);
template spmv_status_t run_ell<double>(int, int, const int*, const double*, const double*, double*, double, double,
                                       cudaStream_t);

}  // namespace mxs
