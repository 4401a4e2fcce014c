// Batched SpMV / SpMM over many independent CSR matrices: Y_i = alpha*A_i*X_i
// + beta*Y_i for i < count, X_i numCols_i x k and Y_i numRows_i x k row-major,
// k in {1, 2, 4, 8, 16}.  The reference has no multi-matrix batching (its
// closest piece splits one matrix over streams, tests/test_multi_stream.cu:
// 121-236).
//
// Work: every matrix is cut into tiles of 256 consecutive nonzeros (at least
// one tile per matrix, so empty matrices still get y = beta*y).  A tile's
// first row comes from the CSR5 tile search done once at plan creation.  One
// persistent launch gives each warp a contiguous range of the batch's tiles
// (equal nonzero counts per warp, whatever the matrix sizes).  Inside a tile
// the 32 lanes form S = 32/L slots of L lanes; a slot owns 256/S consecutive
// nonzeros and each of its lanes owns Q = min(k, 4) of the k columns, so one
// float4 gather per lane serves a nonzero's columns (k = 16: 4 lanes x 4).
// Rows crossing slots are joined by a segmented warp scan; a row crossing
// tiles of the same warp is carried in registers; only the row open at the
// end of a warp's range leaves a carry in memory, which a small fix-up kernel
// adds in warp order -- results are deterministic and need no atomics.
#include <vector>

#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "preprocess.h"

struct spmv_batch_s;

namespace mxs {

constexpr int kBatchSigma = 256;

struct BatchDesc {
    const int* rowPtr;
    const int* colIdx;
    const float* values;
    const float* x;
    float* y;
    int numRows, nnz;
};

template <int Q>
struct VQ {
    float v[Q];
};

template <int Q>
__device__ __forceinline__ VQ<Q> ld_xq(const float* p) {
    VQ<Q> r;
    if constexpr (Q == 4) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(p));
        r.v[0] = a.x;
        r.v[1] = a.y;
        r.v[2] = a.z;
        r.v[3] = a.w;
    } else if constexpr (Q == 2) {
        const float2 a = __ldg(reinterpret_cast<const float2*>(p));
        r.v[0] = a.x;
        r.v[1] = a.y;
    } else {
        r.v[0] = __ldg(p);
    }
    return r;
}

// y[0..Q) = alpha*s + beta*y (y not read when beta is zero).
template <int Q>
__device__ __forceinline__ void st_yq(float* p, const float (&s)[Q], float alpha, float beta, bool bz) {
    float o[Q];
    if (bz) {
#pragma unroll
        for (int q = 0; q < Q; ++q) o[q] = alpha * s[q];
    } else {
        const VQ<Q> old = [&] {
            VQ<Q> r;
            if constexpr (Q == 4) {
                const float4 a = *reinterpret_cast<const float4*>(p);
                r.v[0] = a.x, r.v[1] = a.y, r.v[2] = a.z, r.v[3] = a.w;
            } else if constexpr (Q == 2) {
                const float2 a = *reinterpret_cast<const float2*>(p);
                r.v[0] = a.x, r.v[1] = a.y;
            } else {
                r.v[0] = *p;
            }
            return r;
        }();
#pragma unroll
        for (int q = 0; q < Q; ++q) o[q] = alpha * s[q] + beta * old.v[q];
    }
    if constexpr (Q == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
    } else if constexpr (Q == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(o[0], o[1]);
    } else {
        *p = o[0];
    }
}

// tileStart[m] = first tile of matrix m (tileStart[count] = total tiles).
// Warps of this launch split tiles [tileStart[mBegin], tileStart[mEnd]).
template <int K>
__global__ void __launch_bounds__(256)
batch_tile_kernel(const BatchDesc* __restrict__ descs, int mBegin, int mEnd, const int* __restrict__ tileStart,
                  const int* __restrict__ tileRow, int* __restrict__ carryRow, int* __restrict__ carryMat,
                  float* __restrict__ carryVal, float alpha, float beta, int betaZero) {
    constexpr int Q = K < 4 ? K : 4;  // columns per lane
    constexpr int L = K / Q;          // lanes per slot
    constexpr int S = 32 / L;         // slots per warp
    constexpr int E = kBatchSigma / S;  // nonzeros per slot (multiple of 4)
    static_assert(E % 4 == 0, "slot ranges must start on 16-byte boundaries");
    const bool bz = betaZero != 0;
    const int lane = threadIdx.x & 31, slot = lane / L, kq = lane % L;
    const long long W = (long long)gridDim.x * (blockDim.x >> 5);
    const long long w = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int tAll0 = __ldg(tileStart + mBegin);
    const long long total = (long long)__ldg(tileStart + mEnd) - tAll0;
    const int tb = tAll0 + (int)(total * w / W), te = tAll0 + (int)(total * (w + 1) / W);

    // Matrix of the first tile: last m in [mBegin, mEnd) with tileStart[m] <= tb.
    int m = mBegin;
    {
        int lo = mBegin, hi = mEnd - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tileStart + mid) <= tb) lo = mid;
            else hi = mid - 1;
        }
        m = lo;
    }
    BatchDesc d = descs[m];
    int mTile0 = __ldg(tileStart + m), mTileEnd = __ldg(tileStart + m + 1);
    int cinRow = -1;  // row carried from this warp's previous tile (same matrix)
    float cin[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) cin[q] = 0.f;

    for (int t = tb; t < te; ++t) {
        while (t >= mTileEnd) {
            ++m;
            d = descs[m];
            mTile0 = mTileEnd;
            mTileEnd = __ldg(tileStart + m + 1);
            cinRow = -1;
        }
        const int* __restrict__ rowPtr = d.rowPtr;
        float* __restrict__ y = d.y;
        const int tl = t - mTile0;
        const int tStart = tl * kBatchSigma;
        const int tEnd = min(tStart + kBatchSigma, d.nnz);
        const int rFirst = __ldg(tileRow + t);
        const int rLast = t + 1 < mTileEnd ? __ldg(tileRow + t + 1) : d.numRows - 1;
        const int colOff = kq * Q;

        // Empty rows of (rFirst, rLast] (from row 0 in a matrix's first tile).
        {
            const int lo = tl == 0 ? 0 : rFirst + 1;
            const float zero[Q] = {};
            for (int r = lo + slot; r <= rLast; r += S)
                if (__ldg(rowPtr + r) == __ldg(rowPtr + r + 1))
                    st_yq<Q>(y + (long long)r * K + colOff, zero, alpha, beta, bz);
        }

        const int j0 = tStart + slot * E;
        const int laneEnd = min(j0 + E, tEnd);
        const bool has = j0 < tEnd;
        int key = 0x7fffffff;  // slots without nonzeros sort last in the scan
        int headRow = -1, startRow = -1, rowEnd = 0;
        float run[Q], headVal[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) run[q] = headVal[q] = 0.f;
        if (has) {
            int lo = rFirst, hi = rLast;  // last row with rowPtr <= j0
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(rowPtr + mid) <= j0) lo = mid;
                else hi = mid - 1;
            }
            key = startRow = lo;
            rowEnd = __ldg(rowPtr + lo + 1);
            const float* __restrict__ xb = d.x + colOff;
#pragma unroll 2
            for (int e = 0; e < E; e += 4) {
                const int j = j0 + e;
                if (j >= laneEnd) break;
                int c[4];
                float v[4];
                if (j + 4 <= laneEnd) {
                    const int4 ci = ld_stream4(d.colIdx + j);
                    const float4 vi = ld_stream4(d.values + j);
                    c[0] = ci.x, c[1] = ci.y, c[2] = ci.z, c[3] = ci.w;
                    v[0] = vi.x, v[1] = vi.y, v[2] = vi.z, v[3] = vi.w;
                } else {
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const bool in = j + u < laneEnd;
                        c[u] = in ? ld_stream(d.colIdx + j + u) : 0;
                        v[u] = in ? ld_stream(d.values + j + u) : 0.f;
                    }
                }
                VQ<Q> xv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (j + u < laneEnd) {
                        xv[u] = ld_xq<Q>(xb + (long long)c[u] * K);
                    } else {
#pragma unroll
                        for (int q = 0; q < Q; ++q) xv[u].v[q] = 0.f;
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int jj = j + u;
                    if (jj < laneEnd) {
                        if (jj >= rowEnd) {
                            // `key` is complete; rows skipped on the way are empty.
                            if (headRow < 0) {
                                headRow = key;
#pragma unroll
                                for (int q = 0; q < Q; ++q) headVal[q] = run[q];
                            } else {
                                st_yq<Q>(y + (long long)key * K + colOff, run, alpha, beta, bz);
                            }
                            do {
                                ++key;
                                rowEnd = __ldg(rowPtr + key + 1);
                            } while (jj >= rowEnd);
#pragma unroll
                            for (int q = 0; q < Q; ++q) run[q] = 0.f;
                        }
#pragma unroll
                        for (int q = 0; q < Q; ++q) run[q] = fmaf(v[u], xv[u].v[q], run[q]);
                    }
                }
            }
        }

        // Segmented inclusive scan over slots (lanes with the same kq).
        float incl[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) incl[q] = run[q];
#pragma unroll
        for (int off = 1; off < S; off <<= 1) {
            const int k2 = __shfl_up_sync(kFull, key, off * L);
            float v2[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) v2[q] = __shfl_up_sync(kFull, incl[q], off * L);
            if (slot >= off && k2 == key) {
#pragma unroll
                for (int q = 0; q < Q; ++q) incl[q] += v2[q];
            }
        }
        const int prevKey = __shfl_up_sync(kFull, key, L);
        float prevIncl[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) prevIncl[q] = __shfl_up_sync(kFull, incl[q], L);

        // The row still open at the tile end (held by the slot with the tile's
        // last nonzero) becomes the next tile's carry.
        const int lastSlot = tEnd > tStart ? (tEnd - 1 - tStart) / E : 0;
        const int src = lastSlot * L + kq;
        const int lastKey = __shfl_sync(kFull, key, src);
        const int lastRowEnd = __shfl_sync(kFull, rowEnd, src);
        float lastIncl[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) lastIncl[q] = __shfl_sync(kFull, incl[q], src);

        if (has) {
            if (headRow >= 0) {
                float s[Q];
                const bool joinPrev = slot > 0 && prevKey == startRow;
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    s[q] = headVal[q] + (joinPrev ? prevIncl[q] : 0.f) + (headRow == cinRow ? cin[q] : 0.f);
                st_yq<Q>(y + (long long)headRow * K + colOff, s, alpha, beta, bz);
            }
            if (rowEnd == laneEnd) {  // the lane's last row ends inside it
                float s[Q];
#pragma unroll
                for (int q = 0; q < Q; ++q) s[q] = incl[q] + (key == cinRow ? cin[q] : 0.f);
                st_yq<Q>(y + (long long)key * K + colOff, s, alpha, beta, bz);
            }
        }
        if (tEnd > tStart && lastRowEnd > tEnd) {
#pragma unroll
            for (int q = 0; q < Q; ++q) cin[q] = lastIncl[q] + (lastKey == cinRow ? cin[q] : 0.f);
            cinRow = lastKey;
        } else {
            cinRow = -1;
        }
    }

    if (slot == 0) {
        if (kq == 0) {
            carryRow[w] = cinRow;
            carryMat[w] = m;
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) carryVal[w * K + kq * Q + q] = cin[q];
    }
}

// Adds the carries of warps whose range ended inside a row, in warp order.
template <int K>
__global__ void batch_fixup_kernel(const BatchDesc* __restrict__ descs, int W, const int* __restrict__ carryRow,
                                   const int* __restrict__ carryMat, const float* __restrict__ carryVal, float alpha) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    const int r = carryRow[w];
    if (r < 0) return;
    const int m = carryMat[w];
    if (w > 0 && carryRow[w - 1] == r && carryMat[w - 1] == m) return;
    float s[K];
#pragma unroll
    for (int j = 0; j < K; ++j) s[j] = 0.f;
    for (int u = w; u < W && carryRow[u] == r && carryMat[u] == m; ++u)
#pragma unroll
        for (int j = 0; j < K; ++j) s[j] += carryVal[(long long)u * K + j];
    float* y = descs[m].y + (long long)r * K;
#pragma unroll
    for (int j = 0; j < K; ++j) y[j] += alpha * s[j];
}

}  // namespace mxs

using namespace mxs;

struct spmv_batch_s {
    int count = 0, k = 0, device = 0;
    long long nnzTotal = 0;
    int tiles = 0;
    int warps = 0;  // persistent launch: warps in the grid (= carry slots)
    int blocksPerSM = 0;
    std::vector<int> hTileStart;
    std::vector<BatchDesc> hDesc;
    BatchDesc* dDesc = nullptr;
    int* dTileStart = nullptr;
    int* dTileRow = nullptr;
    int* dCarryRow = nullptr;
    int* dCarryMat = nullptr;
    float* dCarryVal = nullptr;
    bool vectorsSet = false;
    // graphs, keyed by the mode and the alpha/beta they were captured with
    struct G {
        cudaGraphExec_t exec = nullptr;
        float alpha = 0.f, beta = 0.f;
    } graph[2];
    cudaStream_t capStream = nullptr;
};

namespace mxs {
namespace {

template <int K>
spmv_status_t launch_range(const spmv_batch_s* b, int mBegin, int mEnd, int warps, float alpha, float beta,
                           cudaStream_t s) {
    const int blocks = (warps + 7) / 8;
    batch_tile_kernel<K><<<blocks, 256, 0, s>>>(b->dDesc, mBegin, mEnd, b->dTileStart, b->dTileRow, b->dCarryRow,
                                                b->dCarryMat, b->dCarryVal, alpha, beta, beta == 0.f ? 1 : 0);
    MXS_LAUNCH_CHECK();
    batch_fixup_kernel<K><<<grid_for(blocks * 8, 128), 128, 0, s>>>(b->dDesc, blocks * 8, b->dCarryRow,
                                                                     b->dCarryMat, b->dCarryVal, alpha);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

spmv_status_t launch_k(const spmv_batch_s* b, int mBegin, int mEnd, int warps, float alpha, float beta,
                       cudaStream_t s) {
    switch (b->k) {
        case 1: return launch_range<1>(b, mBegin, mEnd, warps, alpha, beta, s);
        case 2: return launch_range<2>(b, mBegin, mEnd, warps, alpha, beta, s);
        case 4: return launch_range<4>(b, mBegin, mEnd, warps, alpha, beta, s);
        case 8: return launch_range<8>(b, mBegin, mEnd, warps, alpha, beta, s);
        case 16: return launch_range<16>(b, mBegin, mEnd, warps, alpha, beta, s);
        default: MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "k must be 1, 2, 4, 8 or 16");
    }
}

template <int K>
int occupancy_blocks() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_tile_kernel<K>, 256, 0);
    return n > 0 ? n : 1;
}

// All launches of one execution: one persistent range, or one range per matrix.
spmv_status_t launch_all(const spmv_batch_s* b, bool loop, float alpha, float beta, cudaStream_t s) {
    if (!loop) return launch_k(b, 0, b->count, b->warps, alpha, beta, s);
    for (int i = 0; i < b->count; ++i) {
        const int t = b->hTileStart[i + 1] - b->hTileStart[i];
        MXS_TRY(launch_k(b, i, i + 1, t < b->warps ? t : b->warps, alpha, beta, s));
    }
    return SPMV_SUCCESS;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace
}  // namespace mxs

extern "C" {

spmv_status_t spmv_batch_destroy(spmv_batch_t b) {
    clear_error();
    if (!b) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch is NULL");
    for (auto& g : b->graph)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (b->capStream) cudaStreamDestroy(b->capStream);
    cudaFree(b->dDesc);
    cudaFree(b->dTileStart);
    cudaFree(b->dTileRow);
    cudaFree(b->dCarryRow);
    delete b;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_create(spmv_handle_t* h, int count, const spmv_batch_matrix_t* mats, int k,
                                spmv_batch_t* out) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    *out = nullptr;
    if (count <= 0 || !mats) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "count must be positive and mats non-NULL");
    if (k != 1 && k != 2 && k != 4 && k != 8 && k != 16)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "k must be 1, 2, 4, 8 or 16 (got %d)", k);
    long long tiles = 0, nnzTotal = 0;
    std::vector<int> tileStart(count + 1);
    for (int i = 0; i < count; ++i) {
        const spmv_batch_matrix_t& a = mats[i];
        if (a.numRows < 0 || a.numCols < 0 || a.nnz < 0)
            MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "matrix %d: negative dimension", i);
        if (a.nnz > 0x7fffffff - 32768) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "matrix %d: nnz above 2^31 - 32769", i);
        if (a.numRows > 0 && !a.rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "matrix %d: rowPtr is NULL", i);
        if (a.numRows == 0 && a.nnz > 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "matrix %d: nonzeros without rows", i);
        if (a.nnz > 0 && (!a.colIdx || !a.values))
            MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "matrix %d: colIdx/values is NULL", i);
        if (a.nnz > 0 && (!aligned(a.colIdx, 16) || !aligned(a.values, 16)))
            MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "matrix %d: colIdx and values must be 16-byte aligned", i);
        tileStart[i] = (int)tiles;
        tiles += a.nnz > 0 ? ((long long)a.nnz + kBatchSigma - 1) / kBatchSigma : 1;
        nnzTotal += a.nnz;
        if (tiles > 0x7fffffff - 1) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "batch has more than 2^31 tiles");
    }
    tileStart[count] = (int)tiles;

    spmv_batch_s* b = new (std::nothrow) spmv_batch_s();
    if (!b) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    b->count = count;
    b->k = k;
    b->device = h->deviceId;
    b->tiles = (int)tiles;
    b->nnzTotal = nnzTotal;
    b->hTileStart = tileStart;
    b->hDesc.resize(count);
    for (int i = 0; i < count; ++i)
        b->hDesc[i] = BatchDesc{mats[i].rowPtr, mats[i].colIdx, mats[i].values, nullptr, nullptr, mats[i].numRows,
                                mats[i].nnz};
    switch (k) {
        case 1: b->blocksPerSM = occupancy_blocks<1>(); break;
        case 2: b->blocksPerSM = occupancy_blocks<2>(); break;
        case 4: b->blocksPerSM = occupancy_blocks<4>(); break;
        case 8: b->blocksPerSM = occupancy_blocks<8>(); break;
        default: b->blocksPerSM = occupancy_blocks<16>(); break;
    }
    b->warps = current_sm_count() * b->blocksPerSM * 8;

    const cudaStream_t s = h->stream;
    int* tileOff = nullptr;
    spmv_status_t st = SPMV_SUCCESS;
    cudaError_t e = cudaMalloc(&b->dDesc, sizeof(BatchDesc) * count);
    if (e == cudaSuccess) e = cudaMalloc(&b->dTileStart, sizeof(int) * (count + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->dTileRow, sizeof(int) * tiles);
    if (e == cudaSuccess) e = cudaMalloc(&tileOff, sizeof(int) * tiles);
    // carries: row, matrix, k values per warp slot
    const size_t cb = ((sizeof(int) * 2 * b->warps + 255) & ~size_t(255)) + sizeof(float) * k * (size_t)b->warps;
    if (e == cudaSuccess) e = cudaMalloc(&b->dCarryRow, cb);
    if (e != cudaSuccess) {
        cudaFree(tileOff);
        spmv_batch_destroy(b);
        return cuda_fail(e, "batch allocation", __FILE__, __LINE__);
    }
    b->dCarryMat = b->dCarryRow + b->warps;
    b->dCarryVal = reinterpret_cast<float*>(reinterpret_cast<char*>(b->dCarryRow) +
                                            ((sizeof(int) * 2 * b->warps + 255) & ~size_t(255)));
    e = cudaMemcpyAsync(b->dTileStart, tileStart.data(), sizeof(int) * (count + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dTileRow, 0, sizeof(int) * tiles, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->dDesc, b->hDesc.data(), sizeof(BatchDesc) * count,
                                              cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) st = cuda_fail(e, "batch setup", __FILE__, __LINE__);
    for (int i = 0; i < count && st == SPMV_SUCCESS; ++i)
        if (mats[i].nnz > 0)
            st = csr5_tiles(mats[i].rowPtr, mats[i].numRows, mats[i].nnz, kBatchSigma, b->dTileRow + tileStart[i],
                            tileOff + tileStart[i], s);
    if (st == SPMV_SUCCESS) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "batch setup", __FILE__, __LINE__);
    }
    cudaFree(tileOff);
    if (st != SPMV_SUCCESS) {
        spmv_batch_destroy(b);
        return st;
    }
    *out = b;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_set_vectors_f32(spmv_batch_t b, const float* const* x, float* const* y) {
    clear_error();
    if (!b) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch is NULL");
    if (!x || !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x/y pointer arrays are NULL");
    const size_t a = (size_t)(b->k < 4 ? b->k : 4) * sizeof(float);
    for (int i = 0; i < b->count; ++i) {
        const BatchDesc& d = b->hDesc[i];
        if (d.numRows > 0 && (!y[i] || !aligned(y[i], a)))
            MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "matrix %d: y is NULL or not %zu-byte aligned", i, a);
        if (d.nnz > 0 && (!x[i] || !aligned(x[i], a)))
            MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "matrix %d: x is NULL or not %zu-byte aligned", i, a);
    }
    for (int i = 0; i < b->count; ++i) {
        b->hDesc[i].x = x[i];
        b->hDesc[i].y = y[i];
    }
    MXS_CUDA(cudaMemcpy(b->dDesc, b->hDesc.data(), sizeof(BatchDesc) * b->count, cudaMemcpyHostToDevice));
    b->vectorsSet = true;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_exec_f32(spmv_handle_t* h, spmv_batch_t b, float alpha, float beta,
                                  spmv_batch_mode_t mode) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!b) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch is NULL");
    if (!b->vectorsSet) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "spmv_batch_set_vectors_f32 was not called");
    const cudaStream_t s = h->stream;
    switch (mode) {
        case SPMV_BATCH_PERSISTENT:
            MXS_TRY(launch_all(b, false, alpha, beta, s));
            break;
        case SPMV_BATCH_LOOP:
            MXS_TRY(launch_all(b, true, alpha, beta, s));
            break;
        case SPMV_BATCH_PERSISTENT_GRAPH:
        case SPMV_BATCH_LOOP_GRAPH: {
            const bool loop = mode == SPMV_BATCH_LOOP_GRAPH;
            auto& g = b->graph[loop ? 1 : 0];
            if (g.exec && (g.alpha != alpha || g.beta != beta)) {
                cudaGraphExecDestroy(g.exec);
                g.exec = nullptr;
            }
            if (!g.exec) {
                if (!b->capStream) MXS_CUDA(cudaStreamCreateWithFlags(&b->capStream, cudaStreamNonBlocking));
                cudaGraph_t graph = nullptr;
                MXS_CUDA(cudaStreamBeginCapture(b->capStream, cudaStreamCaptureModeThreadLocal));
                const spmv_status_t st = launch_all(b, loop, alpha, beta, b->capStream);
                const cudaError_t e = cudaStreamEndCapture(b->capStream, &graph);
                if (st != SPMV_SUCCESS) {
                    if (graph) cudaGraphDestroy(graph);
                    return st;
                }
                if (e != cudaSuccess) return cuda_fail(e, "batch graph capture", __FILE__, __LINE__);
                const cudaError_t e2 = cudaGraphInstantiate(&g.exec, graph, 0);
                cudaGraphDestroy(graph);
                if (e2 != cudaSuccess) {
                    g.exec = nullptr;
                    return cuda_fail(e2, "batch graph instantiate", __FILE__, __LINE__);
                }
                g.alpha = alpha;
                g.beta = beta;
            }
            MXS_CUDA(cudaGraphLaunch(g.exec, s));
            break;
        }
        default:
            MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "unknown batch mode %d", (int)mode);
    }
    if (h->opts.sync) MXS_CUDA(cudaStreamSynchronize(s));
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_info(spmv_batch_t b, long long* tiles, int* warps, long long* nnzTotal) {
    clear_error();
    if (!b) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch is NULL");
    if (tiles) *tiles = b->tiles;
    if (warps) *warps = b->warps;
    if (nnzTotal) *nnzTotal = b->nnzTotal;
    return SPMV_SUCCESS;
}

}  // extern "C"
