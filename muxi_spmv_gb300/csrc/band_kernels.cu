// CSR5-tile SpMV with a shared-memory window of x per CTA (the BAND kernel).
//
// A CTA of NW warps takes NW*TPW consecutive CSR5 tiles (SIGMA = 32*E
// nonzeros each); warp w walks TPW consecutive tiles of that block.  Before
// the gathers, the CTA copies the slice of x around its rows into shared
// memory with one bulk copy (cp.async.bulk completing on an mbarrier):
// for rows [R0, R1] the window is [R0 - b, R1 + b] with b chosen so the slice
// fills WCAP entries.  Gathers whose column lies in the window read shared
// memory; all others read x from global memory, so results never depend on
// the window -- only speed.  Banded and diagonally dominant matrices (the
// stencils, the near-diagonal 70% of the power-law workload) turn most
// gathers into shared-memory reads, relieving the L1 data pipe that random
// global gathers saturate, while the window stays small enough for about
// 48 warps per SM.
//
// The tile data of a warp's first tile is requested before the window wait.
// The wait gives up after about two seconds: the CTA raises *errFlag and
// returns (its copy, if still in flight, completes into the CTA's own shared
// memory first because every thread waits on the same barrier).
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "formats.h"
#include "csr5_tile.cuh"

namespace mxs {

template <typename T, int NW, int E, int TPW, int WCAP>
__global__ void __launch_bounds__(NW * 32)
band_block_kernel(int numRows, int numCols, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                  const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                  int betaZero, const int* __restrict__ tileRow, long long tiles, int useWindow,
                  int* __restrict__ carryRow, T* __restrict__ carryVal, int* __restrict__ errFlag) {
    extern __shared__ __align__(128) unsigned char smem[];
    T* win = reinterpret_cast<T*>(smem);
    __shared__ int sRpAll[NW][csr5_rp_cap<E>()];
    __shared__ __align__(8) unsigned long long bar;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool bz = betaZero != 0;

    const long long tb = (long long)blockIdx.x * NW * TPW;
    const long long te = tb + NW * TPW < tiles ? tb + NW * TPW : tiles;

    // Window bounds (uniform per CTA), multiples of 4 elements.
    int wlo = 0, wspan = 0;
    if (useWindow) {
        const int R0 = __ldg(tileRow + tb);
        const int R1 = te < tiles ? __ldg(tileRow + te) : numRows - 1;
        const long long rows = (long long)R1 - R0 + 1;
        const long long b = rows < WCAP ? (WCAP - rows) / 2 : 0;
        long long lo = (long long)R0 - b;
        lo = lo < 0 ? 0 : lo & ~3LL;
        long long hi = lo + WCAP;
        const long long cols4 = numCols & ~3LL;
        if (hi > cols4) hi = cols4;
        if (hi < lo) hi = lo;
        wlo = (int)lo;
        wspan = (int)(hi - lo);
    }
    if (tid == 0 && wspan > 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (tid == 0 && wspan > 0) {
        mbar_arrive_expect_tx(&bar, (unsigned)(wspan * sizeof(T)));
        bulk_g2s(win, x + wlo, (unsigned)(wspan * sizeof(T)), &bar);
    }

    long long t = tb + (long long)warp * TPW;
    const long long tw = t + TPW < te ? t + TPW : te;
    Csr5Load<T, E> cur;
    if (t < tw) csr5_load<T, E>(cur, t, lane, nnz, tiles, numRows, tileRow, rowPtr, colIdx, values);
    if (wspan > 0 && !mbar_wait_bounded(&bar, 0)) {
        if (tid == 0) atomicExch(errFlag, 1);
        return;
    }
    int* sRp = sRpAll[warp];
    for (; t < tw; ++t) {
        csr5_compute<T, E>(cur, t, lane, numRows, nnz, rowPtr, y, alpha, beta, bz, carryRow, carryVal, sRp,
                           [x, win, wlo, wspan](int c) {
                               const unsigned o = (unsigned)(c - wlo);
                               return o < (unsigned)wspan ? win[o] : ld_x(x + c);
                           });
        __syncwarp();
        if (t + 1 < tw) csr5_load<T, E>(cur, t + 1, lane, nnz, tiles, numRows, tileRow, rowPtr, colIdx, values);
    }
}

template <typename T> constexpr int block_window_cap() { return sizeof(T) == 4 ? 8192 : 4096; }

bool band_shape_supported(int block, int E) {
    return (block == 256 || block == 512) && (E == 4 || E == 8);
}

template <typename T, int NW, int E>
static spmv_status_t launch_block(const int* tileRow, long long tiles, int* carryRow, T* carryVal, int* errFlag,
                                  const RowsArgs<T>& a, int numCols, cudaStream_t s) {
    constexpr int TPW = 4;
    constexpr int WCAP = block_window_cap<T>();
    const bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0;
    const size_t smem = aligned ? sizeof(T) * WCAP : 0;
    auto kern = band_block_kernel<T, NW, E, TPW, WCAP>;
    static bool attr[64] = {false};
    int dev = 0;
    MXS_CUDA(cudaGetDevice(&dev));
    if (dev >= 64 || !attr[dev]) {
        MXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(T) * WCAP)));
        // Prefer the largest shared-memory carve-out so several CTAs' windows fit per SM.
        MXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        if (dev < 64) attr[dev] = true;
    }
    const long long perCta = (long long)NW * TPW;
    const long long grid = (tiles + perCta - 1) / perCta;
    if (grid > 0x7fffffffLL) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "too many tiles");
    kern<<<(unsigned)grid, NW * 32, smem, s>>>(a.numRows, numCols, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y,
                                               a.alpha, a.beta, a.betaZero, tileRow, tiles, aligned ? 1 : 0,
                                               carryRow, carryVal, errFlag);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t run_band(int block, int E, const int* tileRow, long long tiles, int* carryRow, T* carryVal,
                       int* errFlag, const RowsArgs<T>& a, int numCols, cudaStream_t s, cudaEvent_t afterMain) {
    if (tiles <= 0) return SPMV_SUCCESS;
    spmv_status_t st;
    if (block == 512 && E == 8) st = launch_block<T, 16, 8>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols, s);
    else if (block == 512 && E == 4) st = launch_block<T, 16, 4>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols, s);
    else if (block == 256 && E == 8) st = launch_block<T, 8, 8>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols, s);
    else if (block == 256 && E == 4) st = launch_block<T, 8, 4>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols, s);
    else MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported band shape block=%d ept=%d", block, E);
    MXS_TRY(st);
    if (afterMain) MXS_CUDA(cudaEventRecord(afterMain, s));
    return run_csr5_fixup<T>(tiles, carryRow, carryVal, a, s);
}

template spmv_status_t run_band<float>(int, int, const int*, long long, int*, float*, int*, const RowsArgs<float>&,
                                       int, cudaStream_t, cudaEvent_t);
template spmv_status_t run_band<double>(int, int, const int*, long long, int*, double*, int*,
                                        const RowsArgs<double>&, int, cudaStream_t, cudaEvent_t);

}  // namespace mxs
