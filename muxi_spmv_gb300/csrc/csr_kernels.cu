// Row-parallel CSR kernels: one thread per row ("scalar") and groups of
// threadsPerRow lanes per row ("vector", optionally with 16-byte loads).
//
// These replace spmv_csr_scalar_kernel / spmv_csr_vector_kernel and the
// N-threads-per-row family of the reference (src/spmv/csr/spmv_csr.cuh:83-208,
// tests/test_block_optimization.cu:97-145, tests/test_extreme_optimizations.cu:
// 380-423).  Differences that matter for results: every row is covered (no
// 65535-block clamp, spmv_csr.cu:44-49), alpha/beta are applied, and the
// group reduction is a butterfly over aligned lane groups.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"

namespace mxs {

// TPR lanes per row; VEC = 1 (scalar loads) or 4 (aligned 16-byte quads).
// Lanes of one row walk its nnz with stride TPR*VEC; the quad path rounds the
// row start down to a multiple of 4 elements and masks elements outside
// [start, end), so every vector load is 16-byte aligned.
template <typename T, int TPR, int VEC, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
csr_rows_kernel(int numRows, int nnz, const int* __restrict__ rowPtr,
                const int* __restrict__ colIdx, const T* __restrict__ values,
                const T* __restrict__ x, T* __restrict__ y, T alpha, T beta, int betaZero) {
    const long long gtid = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long row = gtid / TPR;
    const int sub = threadIdx.x & (TPR - 1);
    const bool valid = row < numRows;
    int js = 0, je = 0;
    if (valid) {
        js = __ldg(rowPtr + row);
        je = __ldg(rowPtr + row + 1);
    }
    T sum = T(0);
    if (VEC == 1) {
        for (int j = js + sub; j < je; j += TPR)
            sum += ld_stream(values + j) * ld_x(x + ld_stream(colIdx + j));
    } else {
        const int base = js & ~3;
        for (int q = base + sub * 4; q < je; q += TPR * 4) {
            if (q + 4 <= nnz) {
                const int4 c = ld_stream4(colIdx + q);
                const Quad<T> v = ld_stream_quad(values + q);
                const int cc[4] = {c.x, c.y, c.z, c.w};
                T part = T(0);
                T g[4];  // every quad column is a valid index (q + 4 <= nnz)
#pragma unroll
                for (int e = 0; e < 4; ++e) g[e] = ld_x(x + cc[e]);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (q + e >= js && q + e < je) part += v.v[e] * g[e];
                sum += part;
            } else {
                // Last partial quad of the arrays: element loads, never past nnz.
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = q + e;
                    if (j >= js && j < je) sum += ld_stream(values + j) * ld_x(x + ld_stream(colIdx + j));
                }
            }
        }
    }
    if (TPR > 1) sum = group_sum<TPR>(sum);
    if (valid && sub == 0) y[row] = axpby(alpha, sum, beta, betaZero != 0, y + row);
}

template <typename T, int TPR, int VEC, int BLOCK>
static void launch_rows(const RowsArgs<T>& a, cudaStream_t s) {
    const long long threads = (long long)a.numRows * TPR;
    csr_rows_kernel<T, TPR, VEC, BLOCK><<<grid_for(threads, BLOCK), BLOCK, 0, s>>>(
        a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha, a.beta, a.betaZero);
}

template <typename T, int BLOCK>
static bool dispatch_tpr(int tpr, int vec, const RowsArgs<T>& a, cudaStream_t s) {
    if (vec == 4) {
        switch (tpr) {
            case 1: launch_rows<T, 1, 4, BLOCK>(a, s); return true;
            case 2: launch_rows<T, 2, 4, BLOCK>(a, s); return true;
            case 4: launch_rows<T, 4, 4, BLOCK>(a, s); return true;
            case 8: launch_rows<T, 8, 4, BLOCK>(a, s); return true;
            case 16: launch_rows<T, 16, 4, BLOCK>(a, s); return true;
            case 32: launch_rows<T, 32, 4, BLOCK>(a, s); return true;
        }
    } else {
        switch (tpr) {
            case 1: launch_rows<T, 1, 1, BLOCK>(a, s); return true;
            case 2: launch_rows<T, 2, 1, BLOCK>(a, s); return true;
            case 4: launch_rows<T, 4, 1, BLOCK>(a, s); return true;
            case 8: launch_rows<T, 8, 1, BLOCK>(a, s); return true;
            case 16: launch_rows<T, 16, 1, BLOCK>(a, s); return true;
            case 32: launch_rows<T, 32, 1, BLOCK>(a, s); return true;
        }
    }
    return false;
}

template <typename T>
spmv_status_t run_rows(int block, int tpr, int vec, const RowsArgs<T>& a, cudaStream_t s) {
    if (a.numRows <= 0) return SPMV_SUCCESS;
    // Quads need 16-byte aligned column and value arrays.
    if (vec == 4 && ((reinterpret_cast<uintptr_t>(a.colIdx) & 15) ||
                     (reinterpret_cast<uintptr_t>(a.values) & 15)))
        vec = 1;
    bool ok = false;
    switch (block) {  // the reference's family spans blocks of 64 to 1024 threads
        case 64: ok = dispatch_tpr<T, 64>(tpr, vec, a, s); break;
        case 128: ok = dispatch_tpr<T, 128>(tpr, vec, a, s); break;
        case 256: ok = dispatch_tpr<T, 256>(tpr, vec, a, s); break;
        case 512: ok = dispatch_tpr<T, 512>(tpr, vec, a, s); break;
        case 1024: ok = dispatch_tpr<T, 1024>(tpr, vec, a, s); break;
        default: ok = false;
    }
    if (!ok) MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported row-kernel shape block=%d tpr=%d vec=%d", block, tpr, vec);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

template spmv_status_t run_rows<float>(int, int, int, const RowsArgs<float>&, cudaStream_t);
template spmv_status_t run_rows<double>(int, int, int, const RowsArgs<double>&, cudaStream_t);

// y = beta*y (used when a matrix has no nonzeros).
template <typename T>
__global__ void scale_kernel(long long n, T* __restrict__ y, T beta, int betaZero) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        y[i] = betaZero ? T(0) : beta * y[i];
}

template <typename T>
spmv_status_t run_scale(long long n, T* y, T beta, cudaStream_t s) {
    if (n <= 0) return SPMV_SUCCESS;
    const unsigned g = grid_for(n, 256);
    scale_kernel<T><<<g < 65535u * 8 ? g : 65535u * 8, 256, 0, s>>>(n, y, beta, beta == T(0));
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
template spmv_status_t run_scale<float>(long long, float*, float, cudaStream_t);
template spmv_status_t run_scale<double>(long long, double*, double, cudaStream_t);

}  // namespace mxs
