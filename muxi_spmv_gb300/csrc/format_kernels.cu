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

namespace mxs {

template <typename T, int SIGMA>
__global__ void __launch_bounds__(256)
csr5_tile_kernel(int numRows, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                 const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                 int betaZero, const int* __restrict__ tileRow, long long tiles, int* __restrict__ carryRow,
                 T* __restrict__ carryVal) {
    constexpr int E = SIGMA / 32;
    const long long t = ((long long)blockIdx.x * 256 + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= tiles) return;  // uniform per warp
    const bool bz = betaZero != 0;
    const long long tStart = t * SIGMA;
    const long long tEnd = tStart + SIGMA < nnz ? tStart + SIGMA : nnz;
    const int rFirst = tileRow[t];
    const int rLast = t + 1 < tiles ? tileRow[t + 1] : numRows - 1;

    // Empty rows of this tile's range: (rFirst, rLast], plus leading rows for tile 0.
    {
        const int lo = t == 0 ? 0 : rFirst + 1;
        for (int r = lo + lane; r <= rLast; r += 32)
            if (__ldg(rowPtr + r) == __ldg(rowPtr + r + 1)) y[r] = bz ? T(0) : beta * y[r];
    }

    const long long j0 = tStart + (long long)lane * E;
    const long long laneEnd = j0 + E < tEnd ? j0 + E : tEnd;
    const bool has = j0 < tEnd;

    int key = 0x7fffffff;  // lanes without elements sort last in the scan
    T run = T(0), headVal = T(0);
    int headRow = -1, startRow = -1;
    long long rowEnd = 0;
    if (has) {
        int lo = rFirst, hi = rLast;  // last row with rowPtr <= j0
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(rowPtr + mid) <= j0) lo = mid;
            else hi = mid - 1;
        }
        key = startRow = lo;
        rowEnd = __ldg(rowPtr + lo + 1);
        T p[E];
        if (j0 + E <= nnz) {
#pragma unroll
            for (int q = 0; q < E; q += 4) {
                const int4 c = ld_stream4(colIdx + j0 + q);
                const Quad<T> v = ld_stream_quad(values + j0 + q);
                p[q + 0] = v.v[0] * ld_x(x + c.x);
                p[q + 1] = v.v[1] * ld_x(x + c.y);
                p[q + 2] = v.v[2] * ld_x(x + c.z);
                p[q + 3] = v.v[3] * ld_x(x + c.w);
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e)
                p[e] = j0 + e < tEnd ? ld_stream(values + j0 + e) * ld_x(x + ld_stream(colIdx + j0 + e)) : T(0);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const long long j = j0 + e;
            if (j < laneEnd) {
                if (j >= rowEnd) {
                    // `key` is complete; rows skipped on the way are empty.
                    if (headRow < 0) {
                        headRow = key;
                        headVal = run;
                    } else {
                        y[key] = axpby(alpha, run, beta, bz, y + key);
                    }
                    do {
                        ++key;
                        rowEnd = __ldg(rowPtr + key + 1);
                    } while (j >= rowEnd);
                    run = T(0);
                }
                run += p[e];
            }
        }
    }

    // Segmented inclusive scan over lanes of (tail row, partial).
    T incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int k2 = __shfl_up_sync(kFull, key, off);
        const T v2 = __shfl_up_sync(kFull, incl, off);
        if (lane >= off && k2 == key) incl += v2;
    }
    const int prevKey = __shfl_up_sync(kFull, key, 1);
    const T prevIncl = __shfl_up_sync(kFull, incl, 1);
    if (!has) return;
    const T cin = (lane > 0 && prevKey == startRow) ? prevIncl : T(0);
    if (headRow >= 0) y[headRow] = axpby(alpha, headVal + cin, beta, bz, y + headRow);
    if (rowEnd == laneEnd) {
        y[key] = axpby(alpha, incl, beta, bz, y + key);  // tail row ends in this lane
    }
    if (laneEnd == tEnd) {  // the lane holding the tile's last nonzero
        carryRow[t] = rowEnd > laneEnd ? key : -1;
        carryVal[t] = incl;
    }
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
        csr5_tile_kernel<T, 128><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha,
                                                   a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
    } else if (sigma == 256) {
        csr5_tile_kernel<T, 256><<<g, 256, 0, s>>>(a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha,
                                                   a.beta, a.betaZero, tileRow, tiles, carryRow, carryVal);
    } else {
        MXS_FAIL(SPMV_ERROR_INTERNAL, "CSR5 sigma must be 128 or 256 (got %d)", sigma);
    }
    MXS_LAUNCH_CHECK();
    if (afterMain) MXS_CUDA(cudaEventRecord(afterMain, s));
    csr5_fixup_kernel<T><<<grid_for(tiles, 256), 256, 0, s>>>(tiles, carryRow, carryVal, a.y, a.alpha);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
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
