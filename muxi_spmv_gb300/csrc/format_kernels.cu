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

// Adds each split row's carries in tile order (rows with carry -1 skipped).
template <typename T>
__global__ void csr5_fixup_kernel(long long tiles, const int* __restrict__ carryRow, const T* __restrict__ carryVal,
                                  T* __restrict__ y, T alpha) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tiles) return;
    const int r = carryRow[t];
    if (r < 0) return;
    if (t > 0 && carryRow[t - 1] == r) return;
    T s = T(0);
    for (long long u = t; u < tiles && carryRow[u] == r; ++u) s += carryVal[u];
    y[r] += alpha * s;
}

template <typename T>
spmv_status_t run_csr5(int sigma, const int* tileRow, long long tiles, int* carryRow, T* carryVal,
                       const RowsArgs<T>& a, cudaStream_t s, cudaEvent_t afterMain) {
    const unsigned g = grid_for(tiles * 32, 256);
    if (sigma == 128) {
        csr5_tile_kernel<T, 4><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha,
                                                 a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
    } else if (sigma == 256) {
        csr5_tile_kernel<T, 8><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha,
                                                 a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
    } else if (sigma == 512) {
        csr5_tile_kernel<T, 16><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha,
                                                  a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
    } else {
        MXS_FAIL(SPMV_ERROR_INTERNAL, "CSR5 sigma must be 128, 256 or 512 (got %d)", sigma);
    }
    MXS_LAUNCH_CHECK();
    if (afterMain) MXS_CUDA(cudaEventRecord(afterMain, s));
    return run_csr5_fixup<T>(tiles, carryRow, carryVal, a, s);
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
template spmv_status_t run_csr5<float>(int, const int*, long long, int*, float*, const RowsArgs<float>&,
                                       cudaStream_t, cudaEvent_t);
template spmv_status_t run_csr5<double>(int, const int*, long long, int*, double*, const RowsArgs<double>&,
                                        cudaStream_t, cudaEvent_t);

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
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (c[u] >= 0) sum += v[u] * ld_x(x + c[u]);
    }
    for (; i < width; ++i) {
        const long long idx = r + (long long)i * numRows;
        const int c = ld_stream(ellCol + idx);
        if (c >= 0) sum += ld_stream(ellVal + idx) * ld_x(x + c);
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
