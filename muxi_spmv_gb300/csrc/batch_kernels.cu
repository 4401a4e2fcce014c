// Batched SpMV / SpMM over many independent CSR matrices: Y_i = alpha*A_i*X_i
// + beta*Y_i for i < count, X_i numCols_i x k and Y_i numRows_i x k row-major,
// k in {1, 2, 4, 8, 16}.  The reference has no multi-matrix batching (its
// closest piece splits one matrix over streams, tests/test_multi_stream.cu:
// 121-236).
//
// Work: the 32 lanes of a warp form S = 32/L slots of L lanes; each lane owns
// Q = min(k, 4) of the k columns (k = 16: 4 lanes x float4 per nonzero) and a
// slot owns 8 consecutive nonzeros, so a tile is 8*S nonzeros (256 for k <= 4,
// 128 for k = 8, 64 for k = 16).  Every matrix is cut into such tiles (at
// least one, so empty matrices still get y = beta*y); a tile's first row comes
// from the CSR5 tile search done once at plan creation.  One persistent launch
// gives each warp a contiguous range of the batch's tiles -- equal nonzero
// counts per warp whatever the matrix sizes -- and the warp loads tile t+1
// (indices, values, its rowPtr slice) while it computes tile t, searching
// rows in the slice staged in shared memory.  Rows crossing slots are joined
// by a segmented warp scan; a row crossing tiles of the same warp is carried
// in registers; only the row open at the end of a warp's range leaves a carry
// in memory, which a small fix-up kernel adds in warp order -- results are
// deterministic and need no atomics.
#include <vector>

#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "preprocess.h"
#include "csr5_ordered.cuh"

struct spmv_batch_s;

namespace mxs {


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

// Lane layout for k right-hand sides: Q columns per lane, L lanes per slot,
// S slots per warp, E consecutive nonzeros per slot, tiles of SIGMA = E*S.
template <int K, int E_>
struct BatchGeom {
    static constexpr int Q = K < 4 ? K : 4;
    static constexpr int L = K / Q;
    static constexpr int S = 32 / L;
    static constexpr int E = E_;
    static constexpr int SIGMA = E * S;
    // rowPtr entries staged per warp: a tile without empty rows spans at
    // most SIGMA+1 rows (SIGMA+2 entries); larger spans read rowPtr directly.
    static constexpr int RPL = (SIGMA + 2 + 31) / 32;
    static constexpr int CAP = 32 * RPL;
};

__host__ __device__ constexpr int batch_sigma(int k, int e) { return e * (k <= 4 ? 32 : (k == 8 ? 16 : 8)); }

// Everything one tile needs from memory, loaded a tile ahead of its use.
template <int K, int E>
struct TileLoad {
    int rFirst, rLast;
    int c[E];
    float v[E];
    int rp[BatchGeom<K, E>::RPL];
};

template <int K, int E>
__device__ __forceinline__ void tile_load(TileLoad<K, E>& T, const BatchDesc& d, int t, int tl, int mTileEnd,
                                          const int* __restrict__ tileRow, int lane, int slot) {
    using G = BatchGeom<K, E>;
    T.rFirst = __ldg(tileRow + t);
    T.rLast = t + 1 < mTileEnd ? __ldg(tileRow + t + 1) : d.numRows - 1;
    const int nRp = T.rLast - T.rFirst + 2;
#pragma unroll
    for (int k = 0; k < G::RPL; ++k) {
        const int i = lane + 32 * k;
        T.rp[k] = (d.numRows > 0 && nRp <= G::CAP && i < nRp) ? __ldg(d.rowPtr + T.rFirst + i) : 0;
    }
    const int tStart = tl * G::SIGMA;
    const int tEnd = min(tStart + G::SIGMA, d.nnz);
    const int j0 = tStart + slot * E;
    if (j0 + E <= tEnd) {
#pragma unroll
        for (int q = 0; q < E; q += 4) {
            const int4 ci = ld_stream4(d.colIdx + j0 + q);
            const float4 vi = ld_stream4(d.values + j0 + q);
            T.c[q] = ci.x, T.c[q + 1] = ci.y, T.c[q + 2] = ci.z, T.c[q + 3] = ci.w;
            T.v[q] = vi.x, T.v[q + 1] = vi.y, T.v[q + 2] = vi.z, T.v[q + 3] = vi.w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const bool in = j0 + e < tEnd;
            T.c[e] = in ? ld_stream(d.colIdx + j0 + e) : 0;
            T.v[e] = in ? ld_stream(d.values + j0 + e) : 0.f;
        }
    }
}

// tileStart[m] = first tile of matrix m (tileStart[count] = total tiles).
// Tiles [tileStart[mBegin], tileStart[mEnd]) form chunks of CH consecutive
// tiles (2,048 nonzeros by default); warp w of the first numWarps takes chunks w,
// w + numWarps, ...  so the warps in flight share a window of a few matrices
// (their x blocks stay in L2), while rows crossing tiles of one chunk chain in
// registers.  Each chunk leaves one carry (the row open at its end, or -1).
template <int K, int E_, int MINB>
__global__ void __launch_bounds__(256, MINB)
batch_tile_kernel(const BatchDesc* __restrict__ descs, int mBegin, int mEnd, const int* __restrict__ tileStart,
                  const int* __restrict__ tileRow, int* __restrict__ carryRow, int* __restrict__ carryMat,
                  float* __restrict__ carryVal, float alpha, float beta, int betaZero, int numWarps, int CH) {
    using G = BatchGeom<K, E_>;
    constexpr int Q = G::Q, L = G::L, S = G::S, E = G::E, SIGMA = G::SIGMA;
    __shared__ int sRpAll[8][G::CAP];
    const bool bz = betaZero != 0;
    const int lane = threadIdx.x & 31, slot = lane / L, kq = lane % L;
    int* sRp = sRpAll[threadIdx.x >> 5];
    const int W = numWarps;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= W) return;  // whole warps only
    const int tAll0 = __ldg(tileStart + mBegin);
    const int tAllEnd = __ldg(tileStart + mEnd);
    const int chunks = (tAllEnd - tAll0 + CH - 1) / CH;
    int ch = w;
    if (ch >= chunks) return;
    int t = tAll0 + ch * CH;
    int chEnd = min(t + CH, tAllEnd);

    // Matrix of the first tile: last m in [mBegin, mEnd) with tileStart[m] <= t.
    int m;
    {
        int lo = mBegin, hi = mEnd - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tileStart + mid) <= t) lo = mid;
            else hi = mid - 1;
        }
        m = lo;
    }
    // cur = the tile being computed, nxt = the one being loaded
    BatchDesc dCur = descs[m];
    int mCur = m, cur0 = __ldg(tileStart + m), curEnd = __ldg(tileStart + m + 1);
    int mNxt = mCur, nxt0 = cur0, nxtEnd = curEnd;
    BatchDesc dNxt = dCur;
    TileLoad<K, E> cur, nxt;
    tile_load<K, E>(cur, dCur, t, t - cur0, curEnd, tileRow, lane, slot);

    int cinRow = -1;  // row carried from this warp's previous tile (same matrix)
    float cin[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) cin[q] = 0.f;

    for (;;) {
        // the tile after this one: next in the chunk, else the warp's next chunk
        int tn = -1, chn = ch, chEndN = chEnd;
        if (t + 1 < chEnd) {
            tn = t + 1;
        } else if (ch + W < chunks) {
            chn = ch + W;
            tn = tAll0 + chn * CH;
            chEndN = min(tn + CH, tAllEnd);
        }
        if (tn >= 0) {
            while (tn >= nxtEnd) {
                ++mNxt;
                nxt0 = nxtEnd;
                nxtEnd = __ldg(tileStart + mNxt + 1);
            }
            if (mNxt != mCur) dNxt = descs[mNxt];
            tile_load<K, E>(nxt, dNxt, tn, tn - nxt0, nxtEnd, tileRow, lane, slot);
        }

        const int* __restrict__ rowPtr = dCur.rowPtr;
        float* __restrict__ y = dCur.y;
        const int tl = t - cur0;
        const int tStart = tl * SIGMA;
        const int tEnd = min(tStart + SIGMA, dCur.nnz);
        const int rFirst = cur.rFirst, rLast = cur.rLast;
        const bool staged = rLast - rFirst + 2 <= G::CAP;
        if (staged) {
#pragma unroll
            for (int k = 0; k < G::RPL; ++k) sRp[lane + 32 * k] = cur.rp[k];
        }
        __syncwarp();
        auto RP = [&](int r) { return (staged && r >= rFirst) ? sRp[r - rFirst] : __ldg(rowPtr + r); };
        const int colOff = kq * Q;

        // Empty rows of (rFirst, rLast] (from row 0 in a matrix's first tile).
        {
            const int lo = tl == 0 ? 0 : rFirst + 1;
            const float zero[Q] = {};
            for (int r = lo + slot; r <= rLast; r += S)
                if (RP(r) == RP(r + 1)) st_yq<Q>(y + (long long)r * K + colOff, zero, alpha, beta, bz);
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
            // Gathers first (independent of the row search), then the search.
            const float* __restrict__ xb = dCur.x + colOff;
            VQ<Q> xv[E];
#pragma unroll
            for (int e = 0; e < E; ++e) {
                if (j0 + e < laneEnd) {
                    xv[e] = ld_xq<Q>(xb + (long long)cur.c[e] * K);
                } else {
#pragma unroll
                    for (int q = 0; q < Q; ++q) xv[e].v[q] = 0.f;
                }
            }
            int lo = rFirst, hi = rLast;  // last row with rowPtr <= j0
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (RP(mid) <= j0) lo = mid;
                else hi = mid - 1;
            }
            key = startRow = lo;
            rowEnd = RP(lo + 1);
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int jj = j0 + e;
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
                            rowEnd = RP(key + 1);
                        } while (jj >= rowEnd);
#pragma unroll
                        for (int q = 0; q < Q; ++q) run[q] = 0.f;
                    }
#pragma unroll
                    for (int q = 0; q < Q; ++q) run[q] = fmaf(cur.v[e], xv[e].v[q], run[q]);
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
        __syncwarp();  // sRp is rewritten by the next tile

        if (tn < 0 || chn != ch) {  // chunk done: leave its carry
            if (slot == 0) {
                if (kq == 0) {
                    carryRow[ch] = cinRow;
                    carryMat[ch] = mCur;
                }
#pragma unroll
                for (int q = 0; q < Q; ++q) carryVal[(long long)ch * K + kq * Q + q] = cin[q];
            }
            cinRow = -1;
        }
        if (tn < 0) break;
        // advance: the loaded tile becomes the current one
        if (mNxt != mCur) cinRow = -1;
        t = tn;
        ch = chn;
        chEnd = chEndN;
        mCur = mNxt;
        dCur = dNxt;
        cur0 = nxt0;
        curEnd = nxtEnd;
        cur = nxt;
    }
}

// Adds the carries of chunks whose last tile ended inside a row, in chunk order
// (the chunks carrying one row are consecutive: only the first adds).
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

// k = 1, ordered tiles: the batch's CSR5 tiles of 32*E nonzeros (each
// matrix cut into its own tiles, concatenated) run one per warp exactly as a
// single-matrix plan runs them (csr5_ordered.cuh: loads and gathers in
// nonzero order, interior tiles as warp sums, row logic for the rest): no
// slot machinery, about 48 registers, up to 40 warps per SM.  tileMat[t]
// names the matrix of global tile t; the tile writes its carry at its
// global index.  Tiles [tBegin, tEnd) of the batch.
template <int E, int MINB>
__global__ void __launch_bounds__(128, MINB)
batch_ordered_kernel(const BatchDesc* __restrict__ descs, const int* __restrict__ tileStart,
                     const int* __restrict__ tileMat, const int* __restrict__ tileRow, int tBegin, int tEnd,
                     int* __restrict__ carryRow, float* __restrict__ carryVal, float alpha, float beta, int betaZero) {
    __shared__ int sRpAll[4][kOrderedRpCap];
    __shared__ __align__(16) float sPAll[4][ordered_slots<float, E>()];
    const int w = threadIdx.x >> 5;
    const long long t = tBegin + ((long long)blockIdx.x * 128 + threadIdx.x) / 32;
    if (t >= tEnd) return;  // whole warps
    const int m = __ldg(tileMat + t);
    const BatchDesc d = descs[m];
    const int ts = __ldg(tileStart + m);
    const long long tilesM = __ldg(tileStart + m + 1) - ts;
    csr5_ordered_tile<float, E>(t - ts, threadIdx.x & 31, d.numRows, d.nnz, d.rowPtr, d.colIdx, d.values, d.x, d.y,
                                alpha, beta, betaZero != 0, tileRow + ts, tilesM, carryRow + ts, carryVal + ts,
                                false, nullptr, sRpAll[w], sPAll[w], betaZero == kPlainAxpby);
}

// Adds the carries of rows split between ordered tiles: the thread at the
// first tile of a run of tiles of one matrix carrying one row sums the run in
// tile order (runs never cross matrices).
__global__ void batch_ordered_fixup_kernel(const BatchDesc* __restrict__ descs, const int* __restrict__ tileMat,
                                           int tBegin, int tEnd, const int* __restrict__ carryRow,
                                           const float* __restrict__ carryVal, float alpha) {
    const long long t = tBegin + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tEnd) return;
    const int r = carryRow[t];
    if (r < 0) return;
    const int m = tileMat[t];
    if (t > tBegin && carryRow[t - 1] == r && tileMat[t - 1] == m) return;
    float sum = 0.f;
    for (long long u = t; u < tEnd && carryRow[u] == r && tileMat[u] == m; ++u) sum += carryVal[u];
    descs[m].y[r] += alpha * sum;
}

}  // namespace mxs

using namespace mxs;

struct spmv_batch_s {
    int count = 0, k = 0, device = 0;
    spmv_batch_variant_t variant{};
    int sigma = 0;       // nonzeros per tile
    int chunkTiles = 0;  // tiles per chunk of the persistent launch
    long long nnzTotal = 0;
    int tiles = 0;
    int warps = 0;  // resident warps of a full-GPU launch
    int maxTiles = 0;  // tiles of the largest matrix
    std::vector<int> hTileStart;
    std::vector<BatchDesc> hDesc;
    BatchDesc* dDesc = nullptr;
    int* dTileStart = nullptr;
    int* dTileRow = nullptr;
    int* dCarryRow = nullptr;
    int* dCarryMat = nullptr;
    float* dCarryVal = nullptr;
    int* dTileMat = nullptr;  // ordered k = 1 batches: matrix of each tile
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

using BatchKernel = void (*)(const BatchDesc*, int, int, const int*, const int*, int*, int*, float*, float, float,
                             int, int, int);
using FixupKernel = void (*)(const BatchDesc*, int, const int*, const int*, const float*, float);

// (k, nonzeros per slot, blocks per SM) -> kernel; nullptr where not built.
BatchKernel batch_kernel_for(int k, int e, int minb) {
#define MXS_BK(K, E, B) \
    if (k == K && e == E && minb == B) return batch_tile_kernel<K, E, B>;
    MXS_BK(1, 8, 2) MXS_BK(1, 4, 2) MXS_BK(1, 4, 3)
    MXS_BK(2, 8, 2) MXS_BK(2, 4, 2) MXS_BK(2, 4, 3)
    MXS_BK(4, 8, 2) MXS_BK(4, 4, 2) MXS_BK(4, 4, 3)
    MXS_BK(8, 8, 2) MXS_BK(8, 4, 2) MXS_BK(8, 4, 3)
    MXS_BK(16, 8, 2) MXS_BK(16, 4, 2) MXS_BK(16, 4, 3)
#undef MXS_BK
    return nullptr;
}

FixupKernel fixup_kernel_for(int k) {
    switch (k) {
        case 1: return batch_fixup_kernel<1>;
        case 2: return batch_fixup_kernel<2>;
        case 4: return batch_fixup_kernel<4>;
        case 8: return batch_fixup_kernel<8>;
        default: return batch_fixup_kernel<16>;
    }
}

using OrderedKernel = void (*)(const BatchDesc*, const int*, const int*, const int*, int, int, int*, float*, float,
                               float, int);

OrderedKernel ordered_kernel_for(int e, int minb) {
    if (e == 16 && minb == 10) return batch_ordered_kernel<16, 10>;
    if (e == 16 && minb == 8) return batch_ordered_kernel<16, 8>;
    if (e == 8 && minb == 16) return batch_ordered_kernel<8, 16>;
    if (e == 8 && minb == 12) return batch_ordered_kernel<8, 12>;
    return nullptr;
}

// One launch pair (tile kernel + carry fix-up) over the tiles of matrices
// [mBegin, mEnd) of an ordered batch.
spmv_status_t launch_ordered_range(const spmv_batch_s* b, int mBegin, int mEnd, float alpha, float beta,
                                   cudaStream_t s) {
    const int t0 = b->hTileStart[mBegin], t1 = b->hTileStart[mEnd];
    if (t1 <= t0) return SPMV_SUCCESS;
    const int bz = beta == 0.f ? (alpha == 1.f ? kPlainAxpby : 1) : 0;
    ordered_kernel_for(b->variant.nnzPerSlot, b->variant.blocksPerSM)<<<grid_for((long long)(t1 - t0) * 32, 128), 128,
                                                                        0, s>>>(
        b->dDesc, b->dTileStart, b->dTileMat, b->dTileRow, t0, t1, b->dCarryRow, b->dCarryVal, alpha, beta, bz);
    MXS_LAUNCH_CHECK();
    batch_ordered_fixup_kernel<<<grid_for(t1 - t0, 256), 256, 0, s>>>(b->dDesc, b->dTileMat, t0, t1, b->dCarryRow,
                                                                        b->dCarryVal, alpha);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

// One launch pair over matrices [mBegin, mEnd) with chunks of chunkTiles tiles.
spmv_status_t launch_range(const spmv_batch_s* b, int mBegin, int mEnd, int chunkTiles, float alpha, float beta,
                           cudaStream_t s) {
    if (b->variant.ordered) return launch_ordered_range(b, mBegin, mEnd, alpha, beta, s);
    const int tiles = b->hTileStart[mEnd] - b->hTileStart[mBegin];
    const int chunks = (tiles + chunkTiles - 1) / chunkTiles;
    const int warps = chunks < b->warps ? chunks : b->warps;
    const int blocks = (warps + 7) / 8;
    const BatchKernel kern = batch_kernel_for(b->k, b->variant.nnzPerSlot, b->variant.blocksPerSM);
    kern<<<blocks, 256, 0, s>>>(b->dDesc, mBegin, mEnd, b->dTileStart, b->dTileRow, b->dCarryRow, b->dCarryMat,
                                b->dCarryVal, alpha, beta, beta == 0.f ? 1 : 0, warps, chunkTiles);
    MXS_LAUNCH_CHECK();
    fixup_kernel_for(b->k)<<<grid_for(chunks, 128), 128, 0, s>>>(b->dDesc, chunks, b->dCarryRow, b->dCarryMat,
                                                                  b->dCarryVal, alpha);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

// All launches of one execution: one persistent range, or one range per
// matrix (each spread over the whole GPU: chunks of ceil(tiles / warps) tiles).
spmv_status_t launch_all(const spmv_batch_s* b, bool loop, float alpha, float beta, cudaStream_t s) {
    if (!loop) return launch_range(b, 0, b->count, b->chunkTiles, alpha, beta, s);
    for (int i = 0; i < b->count; ++i) {
        const int t = b->hTileStart[i + 1] - b->hTileStart[i];
        int c = (t + b->warps - 1) / b->warps;
        c = c < 1 ? 1 : (c > b->chunkTiles ? b->chunkTiles : c);
        MXS_TRY(launch_range(b, i, i + 1, c, alpha, beta, s));
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
    dev_free(b->dDesc);
    dev_free(b->dTileStart);
    dev_free(b->dTileRow);
    dev_free(b->dCarryRow);
    dev_free(b->dTileMat);
    delete b;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_create_ex(spmv_handle_t* h, int count, const spmv_batch_matrix_t* mats, int k,
                                   const spmv_batch_variant_t* variant, spmv_batch_t* out) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    *out = nullptr;
    if (count <= 0 || !mats) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "count must be positive and mats non-NULL");
    if (k != 1 && k != 2 && k != 4 && k != 8 && k != 16)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "k must be 1, 2, 4, 8 or 16 (got %d)", k);
    spmv_batch_variant_t v = variant ? *variant : spmv_batch_variant_t{};
    int sigma = 0;
    if (v.ordered) {
        if (k != 1) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "ordered batch tiles need k = 1 (got %d)", k);
        if (!v.nnzPerSlot) v.nnzPerSlot = 16;
        if (!v.blocksPerSM) v.blocksPerSM = v.nnzPerSlot == 16 ? 10 : 16;
        if (!ordered_kernel_for(v.nnzPerSlot, v.blocksPerSM))
            MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT,
                     "no ordered batch kernel for %d nonzeros per lane, %d blocks per SM (16: 10 or 8; 8: 16 or 12)",
                     v.nnzPerSlot, v.blocksPerSM);
        sigma = 32 * v.nnzPerSlot;
        v.chunkNnz = sigma;  // one tile per warp
    } else {
        if (!v.nnzPerSlot) v.nnzPerSlot = 8;
        if (!v.blocksPerSM) v.blocksPerSM = 2;
        if (!v.chunkNnz) v.chunkNnz = 2048;
        if (!batch_kernel_for(k, v.nnzPerSlot, v.blocksPerSM))
            MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "no batch kernel for k=%d, %d nonzeros per slot, %d blocks per SM",
                     k, v.nnzPerSlot, v.blocksPerSM);
        sigma = batch_sigma(k, v.nnzPerSlot);
        if (v.chunkNnz < sigma || v.chunkNnz % sigma)
            MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "chunkNnz must be a positive multiple of the tile (%d)", sigma);
    }
    long long tiles = 0, nnzTotal = 0, maxTiles = 0;
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
        const long long mt = a.nnz > 0 ? ((long long)a.nnz + sigma - 1) / sigma : 1;
        tiles += mt;
        if (mt > maxTiles) maxTiles = mt;
        nnzTotal += a.nnz;
        if (tiles > 0x7fffffff - 1) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "batch has more than 2^31 tiles");
    }
    tileStart[count] = (int)tiles;

    spmv_batch_s* b = new (std::nothrow) spmv_batch_s();
    if (!b) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    b->count = count;
    b->k = k;
    b->variant = v;
    b->sigma = sigma;
    b->chunkTiles = v.chunkNnz / sigma;
    b->device = h->deviceId;
    b->tiles = (int)tiles;
    b->maxTiles = (int)maxTiles;
    b->nnzTotal = nnzTotal;
    b->hTileStart = tileStart;
    b->hDesc.resize(count);
    for (int i = 0; i < count; ++i)
        b->hDesc[i] = BatchDesc{mats[i].rowPtr, mats[i].colIdx, mats[i].values, nullptr, nullptr, mats[i].numRows,
                                mats[i].nnz};
    int perSM = 0;
    if (v.ordered) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, ordered_kernel_for(v.nnzPerSlot, v.blocksPerSM), 128, 0);
        b->warps = current_sm_count() * (perSM > 0 ? perSM : 1) * 4;
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, batch_kernel_for(k, v.nnzPerSlot, v.blocksPerSM), 256,
                                                      0);
        b->warps = current_sm_count() * (perSM > 0 ? perSM : 1) * 8;
    }

    const cudaStream_t s = h->stream;
    int* tileOff = nullptr;
    spmv_status_t st = SPMV_SUCCESS;
    cudaError_t e = dev_malloc(&b->dDesc, sizeof(BatchDesc) * count);
    if (e == cudaSuccess) e = dev_malloc(&b->dTileStart, sizeof(int) * (count + 1));
    if (e == cudaSuccess) e = dev_malloc(&b->dTileRow, sizeof(int) * tiles);
    if (e == cudaSuccess) e = dev_malloc(&tileOff, sizeof(int) * tiles);
    // carries: row, matrix, k values per chunk (ordered: per tile, plus the
    // matrix of each tile)
    // persistent chunks, or at most one full-GPU grid of chunks per matrix
    size_t nch = (size_t)((tiles + b->chunkTiles - 1) / b->chunkTiles);
    if (nch < (size_t)b->warps) nch = (size_t)b->warps;
    if (v.ordered) nch = (size_t)tiles;
    if (e == cudaSuccess && v.ordered) e = dev_malloc(&b->dTileMat, sizeof(int) * tiles);
    const size_t rowsBytes = (sizeof(int) * 2 * nch + 255) & ~size_t(255);
    const size_t cb = rowsBytes + sizeof(float) * k * nch;
    if (e == cudaSuccess) e = dev_malloc(&b->dCarryRow, cb);
    if (e != cudaSuccess) {
        dev_free(tileOff);
        spmv_batch_destroy(b);
        return cuda_fail(e, "batch allocation", __FILE__, __LINE__);
    }
    b->dCarryMat = b->dCarryRow + nch;
    b->dCarryVal = reinterpret_cast<float*>(reinterpret_cast<char*>(b->dCarryRow) + rowsBytes);
    e = cudaMemcpyAsync(b->dTileStart, tileStart.data(), sizeof(int) * (count + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dTileRow, 0, sizeof(int) * tiles, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->dDesc, b->hDesc.data(), sizeof(BatchDesc) * count,
                                              cudaMemcpyHostToDevice, s);
    std::vector<int> tileMat;
    if (v.ordered) {
        // tiles of matrices without nonzeros never write a carry: -1 (all bytes 0xff) from the start
        if (e == cudaSuccess) e = cudaMemsetAsync(b->dCarryRow, 0xff, sizeof(int) * tiles, s);
        tileMat.resize((size_t)tiles);
        for (int i = 0; i < count; ++i)
            for (int t = tileStart[i]; t < tileStart[i + 1]; ++t) tileMat[(size_t)t] = i;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->dTileMat, tileMat.data(), sizeof(int) * tiles, cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess) st = cuda_fail(e, "batch setup", __FILE__, __LINE__);
    for (int i = 0; i < count && st == SPMV_SUCCESS; ++i)
        if (mats[i].nnz > 0)
            st = csr5_tiles(mats[i].rowPtr, mats[i].numRows, mats[i].nnz, sigma, b->dTileRow + tileStart[i],
                            tileOff + tileStart[i], s);
    if (st == SPMV_SUCCESS) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "batch setup", __FILE__, __LINE__);
    }
    dev_free(tileOff);
    if (st != SPMV_SUCCESS) {
        spmv_batch_destroy(b);
        return st;
    }
    *out = b;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_create(spmv_handle_t* h, int count, const spmv_batch_matrix_t* mats, int k,
                                spmv_batch_t* out) {
    return spmv_batch_create_ex(h, count, mats, k, nullptr, out);
}

spmv_status_t spmv_batch_get_variant(spmv_batch_t b, spmv_batch_variant_t* v) {
    clear_error();
    if (!b || !v) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "NULL argument");
    *v = b->variant;
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

// ---------------------------------------------------------------------------
// Batch groups: matrices with their own k.  One batch per distinct k (its
// persistent kernel is compiled for that k); execution runs the batches back
// to back on the stream, and the graph modes capture all of them in one
// graph.
// ---------------------------------------------------------------------------
}  // extern "C"

struct spmv_batch_group_s {
    int count = 0;
    long long nnzTotal = 0;
    std::vector<int> ks;                    // distinct k, ascending
    std::vector<spmv_batch_t> batches;      // one per k
    std::vector<std::vector<int>> members;  // matrix indices of each batch
    spmv_batch_s::G graph[2];
    cudaStream_t capStream = nullptr;
};

namespace mxs {
namespace {
spmv_status_t group_launch(spmv_batch_group_t g, bool loop, float alpha, float beta, cudaStream_t s) {
    for (spmv_batch_t b : g->batches) MXS_TRY(launch_all(b, loop, alpha, beta, s));
    return SPMV_SUCCESS;
}
}  // namespace
}  // namespace mxs

extern "C" {

spmv_status_t spmv_batch_group_destroy(spmv_batch_group_t g) {
    clear_error();
    if (!g) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch group is NULL");
    for (auto& gr : g->graph)
        if (gr.exec) cudaGraphExecDestroy(gr.exec);
    if (g->capStream) cudaStreamDestroy(g->capStream);
    for (spmv_batch_t b : g->batches)
        if (b) spmv_batch_destroy(b);
    delete g;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_group_create(spmv_handle_t* h, int count, const spmv_batch_matrix_t* mats, const int* k,
                                      const spmv_batch_variant_t* variants, spmv_batch_group_t* out) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    *out = nullptr;
    if (count <= 0 || !mats || !k) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "count must be positive, mats and k non-NULL");
    static const int kAll[5] = {1, 2, 4, 8, 16};
    std::vector<std::vector<int>> byK(5);
    for (int i = 0; i < count; ++i) {
        int j = 0;
        while (j < 5 && kAll[j] != k[i]) ++j;
        if (j == 5) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "matrix %d: k must be 1, 2, 4, 8 or 16 (got %d)", i, k[i]);
        byK[j].push_back(i);
    }
    spmv_batch_group_s* g = new (std::nothrow) spmv_batch_group_s();
    if (!g) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    g->count = count;
    for (int j = 0; j < 5; ++j) {
        if (byK[j].empty()) continue;
        std::vector<spmv_batch_matrix_t> sub(byK[j].size());
        for (size_t t = 0; t < sub.size(); ++t) sub[t] = mats[byK[j][t]];
        spmv_batch_t b = nullptr;
        const spmv_status_t st = spmv_batch_create_ex(h, (int)sub.size(), sub.data(), kAll[j],
                                                      variants ? &variants[j] : nullptr, &b);
        if (st != SPMV_SUCCESS) {
            spmv_batch_group_destroy(g);
            return st;
        }
        g->ks.push_back(kAll[j]);
        g->batches.push_back(b);
        g->members.push_back(byK[j]);
        g->nnzTotal += b->nnzTotal;
    }
    *out = g;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_group_set_vectors_f32(spmv_batch_group_t g, const float* const* x, float* const* y) {
    clear_error();
    if (!g) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch group is NULL");
    if (!x || !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x/y pointer arrays are NULL");
    for (size_t j = 0; j < g->batches.size(); ++j) {
        std::vector<const float*> xs(g->members[j].size());
        std::vector<float*> ys(g->members[j].size());
        for (size_t t = 0; t < xs.size(); ++t) {
            xs[t] = x[g->members[j][t]];
            ys[t] = y[g->members[j][t]];
        }
        MXS_TRY(spmv_batch_set_vectors_f32(g->batches[j], xs.data(), ys.data()));
    }
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_group_exec_f32(spmv_handle_t* h, spmv_batch_group_t g, float alpha, float beta,
                                        spmv_batch_mode_t mode) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!g) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch group is NULL");
    for (spmv_batch_t b : g->batches)
        if (!b->vectorsSet) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "spmv_batch_group_set_vectors_f32 was not called");
    const cudaStream_t s = h->stream;
    switch (mode) {
        case SPMV_BATCH_PERSISTENT:
        case SPMV_BATCH_LOOP:
            MXS_TRY(group_launch(g, mode == SPMV_BATCH_LOOP, alpha, beta, s));
            break;
        case SPMV_BATCH_PERSISTENT_GRAPH:
        case SPMV_BATCH_LOOP_GRAPH: {
            const bool loop = mode == SPMV_BATCH_LOOP_GRAPH;
            auto& gr = g->graph[loop ? 1 : 0];
            if (gr.exec && (gr.alpha != alpha || gr.beta != beta)) {
                cudaGraphExecDestroy(gr.exec);
                gr.exec = nullptr;
            }
            if (!gr.exec) {
                if (!g->capStream) MXS_CUDA(cudaStreamCreateWithFlags(&g->capStream, cudaStreamNonBlocking));
                cudaGraph_t graph = nullptr;
                MXS_CUDA(cudaStreamBeginCapture(g->capStream, cudaStreamCaptureModeThreadLocal));
                const spmv_status_t st = group_launch(g, loop, alpha, beta, g->capStream);
                const cudaError_t e = cudaStreamEndCapture(g->capStream, &graph);
                if (st != SPMV_SUCCESS) {
                    if (graph) cudaGraphDestroy(graph);
                    return st;
                }
                if (e != cudaSuccess) return cuda_fail(e, "batch group graph capture", __FILE__, __LINE__);
                const cudaError_t e2 = cudaGraphInstantiate(&gr.exec, graph, 0);
                cudaGraphDestroy(graph);
                if (e2 != cudaSuccess) {
                    gr.exec = nullptr;
                    return cuda_fail(e2, "batch group graph instantiate", __FILE__, __LINE__);
                }
                gr.alpha = alpha;
                gr.beta = beta;
            }
            MXS_CUDA(cudaGraphLaunch(gr.exec, s));
            break;
        }
        default:
            MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "unknown batch mode %d", (int)mode);
    }
    if (h->opts.sync) MXS_CUDA(cudaStreamSynchronize(s));
    return SPMV_SUCCESS;
}

spmv_status_t spmv_batch_group_info(spmv_batch_group_t g, int* batches, long long* nnzTotal) {
    clear_error();
    if (!g) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "batch group is NULL");
    if (batches) *batches = (int)g->batches.size();
    if (nnzTotal) *nnzTotal = g->nnzTotal;
    return SPMV_SUCCESS;
}

}  // extern "C"
