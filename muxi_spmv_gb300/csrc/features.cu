// Matrix features for the learned kernel selector, computed on the device
// from rowPtr (all rows) and colIdx (up to 4096 sampled rows, 1024 nonzeros
// each).  Cost: one pass over rowPtr plus a few MB of column indices, i.e.
// microseconds, against milliseconds for an exhaustive autotune.
//
// Feature vector (SPMV_NUM_FEATURES = 32 floats):
//   0 log2(R+1)   1 log2(C+1)   2 log2(nnz+1)   3 log2(mean row length + 1)
//   4 coefficient of variation of row length   5 log2(max row length + 1)
//   6 log2(max/mean + 1)   7 fraction of empty rows
//   8..19 fraction of rows with length in [0], [1], [2,4), [4,8), [8,16),
//         [16,32), [32,64), [64,128), [128,256), [256,1024), [1024,4096), >=4096
//   20 fraction of nonzeros in rows of length >= 1024
//   21 fraction of nonzeros in rows of length >= 256
//   22 mean |col - diagonal| / C over sampled nonzeros (diagonal = row*C/R)
//   23..25 fraction of sampled nonzeros within 64, 4096 and C/64 of the diagonal
//   26 mean (max col - min col) / C over sampled rows
//   27 log2(mean gap between consecutive sampled columns + 1)
//   28 fraction of consecutive sampled pairs with gap <= 8
//   29 log2(x bytes / L2 bytes)   30 log2(matrix bytes / L2 bytes)   31 log2(R / C)
#include <cmath>

#include "internal.h"
#include "device.cuh"
#include "kernels.h"

namespace mxs {

struct FeatAcc {
    unsigned long long sumLen, maxLen, empty, long1024, long256;
    double sumLen2;
    unsigned long long hist[12];
    // sampled columns
    double sumDist;
    unsigned long long sampled, near64, near4096, nearFrac, pairs, close8;
    double sumSpan, sumGap;
    unsigned long long spanRows;
};

__device__ __forceinline__ int len_bin(unsigned l) {
    if (l == 0) return 0;
    if (l == 1) return 1;
    if (l < 4) return 2;
    if (l < 8) return 3;
    if (l < 16) return 4;
    if (l < 32) return 5;
    if (l < 64) return 6;
    if (l < 128) return 7;
    if (l < 256) return 8;
    if (l < 1024) return 9;
    if (l < 4096) return 10;
    return 11;
}

__global__ void feat_rows_kernel(const int* __restrict__ rowPtr, int numRows, FeatAcc* acc) {
    __shared__ unsigned long long sHist[12];
    if (threadIdx.x < 12) sHist[threadIdx.x] = 0;
    __syncthreads();
    unsigned long long s = 0, mx = 0, em = 0, l1k = 0, l256 = 0;
    double s2 = 0.0;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < numRows;
         r += (long long)gridDim.x * blockDim.x) {
        const unsigned l = (unsigned)(rowPtr[r + 1] - rowPtr[r]);
        s += l;
        s2 += (double)l * l;
        mx = l > mx ? l : mx;
        em += l == 0;
        if (l >= 1024) l1k += l;
        if (l >= 256) l256 += l;
        atomicAdd(&sHist[len_bin(l)], 1ull);
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_xor_sync(kFull, s, off);
        s2 += __shfl_xor_sync(kFull, s2, off);
        const unsigned long long m2 = __shfl_xor_sync(kFull, mx, off);
        mx = m2 > mx ? m2 : mx;
        em += __shfl_xor_sync(kFull, em, off);
        l1k += __shfl_xor_sync(kFull, l1k, off);
        l256 += __shfl_xor_sync(kFull, l256, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc->sumLen, s);
        atomicAdd(&acc->sumLen2, s2);
        atomicMax(&acc->maxLen, mx);
        atomicAdd(&acc->empty, em);
        atomicAdd(&acc->long1024, l1k);
        atomicAdd(&acc->long256, l256);
    }
    __syncthreads();
    if (threadIdx.x < 12 && sHist[threadIdx.x]) atomicAdd(&acc->hist[threadIdx.x], sHist[threadIdx.x]);
}

// Warp per sampled row.
__global__ void feat_cols_kernel(const int* __restrict__ rowPtr, const int* __restrict__ colIdx, int numRows,
                                 int numCols, int samples, FeatAcc* acc) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= samples) return;
    const long long r = samples >= numRows ? w : (long long)w * numRows / samples;
    const int s = rowPtr[r], e0 = rowPtr[r + 1];
    const int e = e0 - s > 1024 ? s + 1024 : e0;
    const double diag = (double)r * numCols / (numRows > 0 ? numRows : 1);
    const double fracWin = numCols / 64.0;
    double dist = 0.0, gap = 0.0;
    unsigned long long n = 0, n64 = 0, n4k = 0, nfr = 0, pairs = 0, close = 0;
    int cmin = 0x7fffffff, cmax = -1;
    for (int j = s + lane; j < e; j += 32) {
        const int c = colIdx[j];
        const double d = fabs((double)c - diag);
        dist += d;
        ++n;
        n64 += d <= 64.0;
        n4k += d <= 4096.0;
        nfr += d <= fracWin;
        cmin = min(cmin, c);
        cmax = max(cmax, c);
        if (j + 1 < e) {
            const int g = abs(colIdx[j + 1] - c);
            gap += g;
            ++pairs;
            close += g <= 8;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        dist += __shfl_xor_sync(kFull, dist, off);
        gap += __shfl_xor_sync(kFull, gap, off);
        n += __shfl_xor_sync(kFull, n, off);
        n64 += __shfl_xor_sync(kFull, n64, off);
        n4k += __shfl_xor_sync(kFull, n4k, off);
        nfr += __shfl_xor_sync(kFull, nfr, off);
        pairs += __shfl_xor_sync(kFull, pairs, off);
        close += __shfl_xor_sync(kFull, close, off);
        cmin = min(cmin, __shfl_xor_sync(kFull, cmin, off));
        cmax = max(cmax, __shfl_xor_sync(kFull, cmax, off));
    }
    if (lane == 0) {
        atomicAdd(&acc->sumDist, dist);
        atomicAdd(&acc->sampled, n);
        atomicAdd(&acc->near64, n64);
        atomicAdd(&acc->near4096, n4k);
        atomicAdd(&acc->nearFrac, nfr);
        atomicAdd(&acc->pairs, pairs);
        atomicAdd(&acc->close8, close);
        atomicAdd(&acc->sumGap, gap);
        if (n > 0) {
            atomicAdd(&acc->sumSpan, (double)(cmax - cmin) / (numCols > 0 ? numCols : 1));
            atomicAdd(&acc->spanRows, 1ull);
        }
    }
}

__global__ void feat_finish_kernel(const FeatAcc* __restrict__ a, int R, int C, long long N, double l2,
                                   double vsize, float* __restrict__ f) {
    const double Rd = R > 0 ? R : 1, mean = (double)a->sumLen / Rd;
    const double var = a->sumLen2 / Rd - mean * mean;
    const double sd = var > 0 ? sqrt(var) : 0.0;
    const double nn = N > 0 ? (double)N : 1.0;
    f[0] = (float)log2(R + 1.0);
    f[1] = (float)log2(C + 1.0);
    f[2] = (float)log2(N + 1.0);
    f[3] = (float)log2(mean + 1.0);
    f[4] = (float)(mean > 0 ? sd / mean : 0.0);
    f[5] = (float)log2((double)a->maxLen + 1.0);
    f[6] = (float)log2((mean > 0 ? (double)a->maxLen / mean : 0.0) + 1.0);
    f[7] = (float)(a->empty / Rd);
    for (int i = 0; i < 12; ++i) f[8 + i] = (float)(a->hist[i] / Rd);
    f[20] = (float)(a->long1024 / nn);
    f[21] = (float)(a->long256 / nn);
    const double ns = a->sampled > 0 ? (double)a->sampled : 1.0;
    f[22] = (float)(a->sumDist / ns / (C > 0 ? C : 1));
    f[23] = (float)(a->near64 / ns);
    f[24] = (float)(a->near4096 / ns);
    f[25] = (float)(a->nearFrac / ns);
    f[26] = (float)(a->spanRows > 0 ? a->sumSpan / a->spanRows : 0.0);
    f[27] = (float)log2((a->pairs > 0 ? a->sumGap / a->pairs : 0.0) + 1.0);
    f[28] = (float)(a->pairs > 0 ? (double)a->close8 / a->pairs : 0.0);
    f[29] = (float)log2((C * vsize + 1.0) / l2);
    f[30] = (float)log2((N * (vsize + 4.0) + (R + 1.0) * 4.0 + 1.0) / l2);
    f[31] = (float)log2((R + 1.0) / (C + 1.0));
}

spmv_status_t matrix_features(int R, int C, int N, const int* rowPtr, const int* colIdx, size_t vsize, float* dOut,
                              cudaStream_t s, long long* maxLenOut) {
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (!dOut) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "output is NULL");
    if ((R > 0 && !rowPtr) || (N > 0 && !colIdx)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL CSR array");
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(FeatAcc), s));
    FeatAcc* acc = static_cast<FeatAcc*>(buf);
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(FeatAcc), s);
    if (e == cudaSuccess && R > 0) {
        const unsigned g = grid_for(R, 256);
        feat_rows_kernel<<<g < 2048u ? g : 2048u, 256, 0, s>>>(rowPtr, R, acc);
        const int samples = R < 4096 ? R : 4096;
        if (N > 0) feat_cols_kernel<<<grid_for((long long)samples * 32, 256), 256, 0, s>>>(rowPtr, colIdx, R, C, samples, acc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        int dev = 0;
        cudaGetDevice(&dev);
        const double l2 = (double)(device_props(dev).l2_bytes ? device_props(dev).l2_bytes : (size_t)128 << 20);
        feat_finish_kernel<<<1, 1, 0, s>>>(acc, R, C, N, l2, (double)vsize, dOut);
        e = cudaGetLastError();
    }
    unsigned long long maxLen = 0;
    if (e == cudaSuccess && maxLenOut) {
        e = cudaMemcpyAsync(&maxLen, &acc->maxLen, sizeof(maxLen), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        *maxLenOut = (long long)maxLen;
    }
    scratch_free(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "features", __FILE__, __LINE__);
    return SPMV_SUCCESS;
}

}  // namespace mxs

using namespace mxs;

extern "C" spmv_status_t spmv_matrix_features(spmv_type_t type, int R, int C, int N, const int* rowPtr,
                                              const int* colIdx, float* features, cudaStream_t stream) {
    clear_error();
    if (type != SPMV_TYPE_FLOAT && type != SPMV_TYPE_DOUBLE) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "float or double");
    return matrix_features(R, C, N, rowPtr, colIdx, type == SPMV_TYPE_FLOAT ? 4 : 8, features, stream, nullptr);
}
