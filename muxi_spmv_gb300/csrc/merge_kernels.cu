// Merge-path SpMV for sm_103a.
//
// The merge path of a CSR matrix interleaves its R row ends with its N nonzero
// indices (length L = R + N).  Cutting it into equal pieces balances rows and
// nonzeros at once, which is what power-law matrices need.  The reference
// (src/spmv/csr5/spmv_csr5.cu:497-626, 912-1014) cuts it into one piece per
// warp and lets each lane walk whole rows serially, adding split rows with
// atomics; its consumer double-counts the tail of a split row and drops the
// head.  This file keeps the reference's path coordinates (bit-exact through
// merge_partitions / merge_search) and replaces the consumer:
//
//   * one CTA per tile of BLOCK*IPT path items;
//   * the CTA stages its row ends and the products val[j]*x[col[j]] of its
//     nonzeros in shared memory with coalesced loads;
//   * each thread walks IPT consecutive path items (a merge search in shared
//     memory finds its start), emitting complete rows;
//   * a block-wide segmented scan joins rows split between threads;
//   * the partial sum of the row left open at the tile end goes to a carry
//     slot, and a second kernel adds the carries of each row in tile order.
// No floating-point atomics are used, so results are run-to-run identical.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"

namespace mxs {

// ---------------------------------------------------------------------------
// Reference-compatible partition positions and path search.
// ---------------------------------------------------------------------------
__global__ void partitions_kernel(long long L, int P, int* __restrict__ pos) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > P) return;
    const long long per = (L + P - 1) / P;
    const long long v = t * per;
    pos[t] = (int)(v < L ? v : L);
}

spmv_status_t merge_partitions(int numRows, int nnz, int P, int* pos, cudaStream_t s) {
    if (P < 1) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "numPartitions must be >= 1 (got %d)", P);
    if (!pos) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "pos is NULL");
    const long long L = (long long)numRows + nnz;
    if (L > 0x7fffffffLL) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "numRows+nnz exceeds int32 positions");
    partitions_kernel<<<grid_for((long long)P + 1, 256), 256, 0, s>>>(L, P, pos);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

__global__ void search_kernel(const int* __restrict__ rowPtr, int numRows, int nnz,
                              const int* __restrict__ diag, int count, int* __restrict__ rowIdx,
                              int* __restrict__ nnzIdx) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    long long k = diag[t];
    const long long L = (long long)numRows + nnz;
    if (k < 0) k = 0;
    if (k > L) k = L;
    const int r = merge_row_of_diag(rowPtr, numRows, nnz, k);
    rowIdx[t] = r;
    nnzIdx[t] = (int)(k - r);
}

spmv_status_t merge_search(const int* rowPtr, int numRows, int nnz, const int* diag, int count,
                           int* rowIdx, int* nnzIdx, cudaStream_t s) {
    if (count <= 0) return SPMV_SUCCESS;
    if (!rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (!diag || !rowIdx || !nnzIdx) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL search array");
    search_kernel<<<grid_for(count, 256), 256, 0, s>>>(rowPtr, numRows, nnz, diag, count, rowIdx, nnzIdx);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

// ---------------------------------------------------------------------------
// Tile geometry and coordinates.
// ---------------------------------------------------------------------------
bool merge_geom_supported(const MergeGeom& g) {
    if (g.block != 128 && g.block != 256) return false;
    if (g.vec) return g.vec == 4 && (g.ipt == 4 || g.ipt == 8 || g.ipt == 12 || g.ipt == 16);
    return g.ipt == 3 || g.ipt == 5 || g.ipt == 7 || g.ipt == 9 || g.ipt == 11;
}

MergeGeom merge_geom_of(const spmv_variant_t& v) {
    MergeGeom g;
    g.block = v.blockSize ? v.blockSize : 256;
    g.vec = v.vectorWidth == 4 ? 4 : 0;
    g.ipt = v.itemsPerThread ? v.itemsPerThread : (g.vec ? 8 : 7);
    return g;
}

long long merge_tile_count(int numRows, int nnz, const MergeGeom& g) {
    const long long L = (long long)numRows + nnz;
    const long long P = (L + g.tile() - 1) / g.tile();
    return P < 1 ? 1 : P;
}

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t merge_scratch_bytes(long long P, size_t vsize) {
    return 2 * align256(sizeof(int) * (P + 1)) + align256(sizeof(int) * P) + align256(vsize * P);
}

MergeScratch merge_carve(void* base, long long P, size_t vsize) {
    char* p = static_cast<char*>(base);
    MergeScratch s;
    s.tileRow = reinterpret_cast<int*>(p);
    p += align256(sizeof(int) * (P + 1));
    s.tileNnz = reinterpret_cast<int*>(p);
    p += align256(sizeof(int) * (P + 1));
    s.carryRow = reinterpret_cast<int*>(p);
    p += align256(sizeof(int) * P);
    s.carryVal = p;
    (void)vsize;
    return s;
}

__global__ void tile_coords_kernel(const int* __restrict__ rowPtr, int numRows, int nnz, long long tile,
                                   long long P, int* __restrict__ tileRow, int* __restrict__ tileNnz) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > P) return;
    const long long L = (long long)numRows + nnz;
    long long k = t * tile;
    if (k > L) k = L;
    const int r = merge_row_of_diag(rowPtr, numRows, nnz, k);
    tileRow[t] = r;
    tileNnz[t] = (int)(k - r);
}

spmv_status_t merge_tile_coords(const int* rowPtr, int numRows, int nnz, const MergeGeom& g,
                                long long P, int* tileRow, int* tileNnz, cudaStream_t s) {
    tile_coords_kernel<<<grid_for(P + 1, 256), 256, 0, s>>>(rowPtr, numRows, nnz, g.tile(), P, tileRow,
                                                            tileNnz);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

// ---------------------------------------------------------------------------
// Tile kernel.
// ---------------------------------------------------------------------------
template <typename T, int BLOCK, int IPT>
__global__ void __launch_bounds__(BLOCK)
merge_tile_kernel(int numRows, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                  const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha,
                  T beta, int betaZero, const int* __restrict__ tileRow,
                  const int* __restrict__ tileNnz, int* __restrict__ carryRow,
                  T* __restrict__ carryVal) {
    constexpr int TILE = BLOCK * IPT;
    constexpr int NW = BLOCK / 32;
    __shared__ int sEnd[TILE];     // row ends rowPtr[r0+1 .. r1]
    __shared__ T sProd[TILE];      // products of the tile's nonzeros
    __shared__ int sWarpKey[NW];
    __shared__ T sWarpVal[NW];
    __shared__ int sKey[BLOCK];
    __shared__ T sIncl[BLOCK];

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const long long t = blockIdx.x;
    const int r0 = tileRow[t], j0 = tileNnz[t];
    const int nr = tileRow[t + 1] - r0;  // row ends inside the tile
    const int nj = tileNnz[t + 1] - j0;  // nonzeros inside the tile
    const bool bz = betaZero != 0;

    // Stage row ends and products with coalesced loads.  All loads of a
    // thread are issued before the dependent gathers.
    int cl[IPT];
    T vl[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const int k = tid + u * BLOCK;
        if (k < nj) {
            cl[u] = ld_stream(colIdx + j0 + k);
            vl[u] = ld_stream(values + j0 + k);
        }
        if (k < nr) sEnd[k] = __ldg(rowPtr + r0 + 1 + k);
    }
    T g[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) g[u] = ld_x(x + (tid + u * BLOCK < nj ? cl[u] : 0));
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const int k = tid + u * BLOCK;
        if (k < nj) sProd[k] = vl[u] * g[u];
    }
    __syncthreads();

    // This thread's start on the tile's merge path: row-end index i, nnz jj.
    const int items = nr + nj;
    const int d = min(tid * IPT, items);
    int lo = max(0, d - nj), hi = min(d, nr);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sEnd[mid] <= j0 + d - 1 - mid) lo = mid + 1;
        else hi = mid;
    }
    const int startRow = lo;
    int i = lo, jj = d - lo;
    const int dEnd = min(d + IPT, items);

    T run = T(0), firstVal = T(0);
    int firstRow = -1;
#pragma unroll
    for (int s = 0; s < IPT; ++s) {
        if (d + s < dEnd) {
            if (i < nr && sEnd[i] <= j0 + jj) {
                // Row end: row r0+i is complete in this thread.
                if (firstRow < 0) {
                    firstRow = i;
                    firstVal = run;
                } else {
                    const int r = r0 + i;
                    y[r] = axpby(alpha, run, beta, bz, y + r);
                }
                run = T(0);
                ++i;
            } else {
                run += sProd[jj];
                ++jj;
            }
        }
    }

    // Block-wide inclusive segmented scan of (row, partial) over threads.  Row
    // indices are non-decreasing in tid, so equal keys at distance off imply
    // equal keys in between.
    int key = i;
    T v = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int k2 = __shfl_up_sync(kFull, key, off);
        const T v2 = __shfl_up_sync(kFull, v, off);
        if (lane >= off && k2 == key) v += v2;
    }
    if (lane == 31) {
        sWarpKey[warp] = key;
        sWarpVal[warp] = v;
    }
    __syncthreads();
    T pre = T(0);
    for (int w = warp - 1; w >= 0; --w) {
        if (sWarpKey[w] != key) break;
        pre += sWarpVal[w];
    }
    v += pre;
    sKey[tid] = key;
    sIncl[tid] = v;
    __syncthreads();

    // Partial sum of startRow accumulated by the threads before this one.
    const T cin = (tid > 0 && sKey[tid - 1] == startRow) ? sIncl[tid - 1] : T(0);
    if (firstRow >= 0) {
        const int r = r0 + firstRow;
        y[r] = axpby(alpha, firstVal + cin, beta, bz, y + r);
    }
    if (tid == BLOCK - 1) {
        carryRow[t] = r0 + key;  // == tileRow[t+1]
        carryVal[t] = v;
    }
}

// ---------------------------------------------------------------------------
// Tile kernel, nonzero-vectorised consumer.
//
// Same tiles, same carries, but the work is laid out by nonzero instead of by
// merge item: the CTA covers the 16-byte-aligned span [a0, a0 + BLOCK*EPT)
// with a0 = j0 rounded down to 4 elements, and thread t owns the EPT
// consecutive positions a0 + t*EPT.. (16-byte loads of colIdx and values,
// then EPT independent gathers of x).  Only positions in [j0, j1) count.  A
// thread finds the row of its first nonzero with one binary search in the
// tile's staged rowPtr slice, walks its nonzeros summing per row, writes the
// rows that end inside it, and the block scan joins rows that cross threads.
// Rows that end in this tile but own no nonzero in it (empty rows, or a row
// whose nonzeros all lie in earlier tiles) get y = beta*y here; the carry
// fix-up adds their earlier partial sums.
// ---------------------------------------------------------------------------
template <typename T, int EPT>
__device__ __forceinline__ void load_span(const int* __restrict__ colIdx, const T* __restrict__ values,
                                          const T* __restrict__ x, int nnz, int base, int lo, int hi, T (&p)[EPT]) {
    if (base + EPT <= nnz) {
#pragma unroll
        for (int q = 0; q < EPT; q += 4) {
            const int4 c = ld_stream4(colIdx + base + q);
            const Quad<T> v = ld_stream_quad(values + base + q);
            const int cc[4] = {c.x, c.y, c.z, c.w};
            T g[4];  // every quad column is a valid index (base + EPT <= nnz)
#pragma unroll
            for (int e = 0; e < 4; ++e) g[e] = ld_x(x + cc[e]);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int j = base + q + e;
                p[q + e] = (j >= lo && j < hi) ? v.v[e] * g[e] : T(0);
            }
        }
    } else {
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const int j = base + e;
            p[e] = (j >= lo && j < hi) ? ld_stream(values + j) * ld_x(x + ld_stream(colIdx + j)) : T(0);
        }
    }
}

template <typename T, int BLOCK, int EPT>
__global__ void __launch_bounds__(BLOCK)
merge_vec_kernel(int numRows, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                 const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                 int betaZero, const int* __restrict__ tileRow, const int* __restrict__ tileNnz,
                 int* __restrict__ carryRow, T* __restrict__ carryVal) {
    constexpr int SPAN = BLOCK * EPT;
    constexpr int NW = BLOCK / 32;
    __shared__ int sRp[SPAN];  // rowPtr[r0 .. r1+1]; a tile has at most SPAN-4 row ends
    __shared__ int sWarpKey[NW];
    __shared__ T sWarpVal[NW];
    __shared__ int sKey[BLOCK];
    __shared__ T sIncl[BLOCK];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long t = blockIdx.x;
    const int r0 = tileRow[t], j0 = tileNnz[t];
    const int r1 = tileRow[t + 1], j1 = tileNnz[t + 1];
    const int nr = r1 - r0;
    const bool bz = betaZero != 0;

    for (int k = tid; k < nr + 2; k += BLOCK) sRp[k] = __ldg(rowPtr + min(r0 + k, numRows));

    const int base = (j0 & ~3) + tid * EPT;
    const int lo = max(base, j0), hi = min(base + EPT, j1);
    const bool has = lo < hi;
    T p[EPT];
    if (has) load_span<T, EPT>(colIdx, values, x, nnz, base, lo, hi, p);
    __syncthreads();

    // Rows ending in this tile without a nonzero in it.
    for (int k = tid; k < nr; k += BLOCK) {
        const int first = k == 0 ? j0 : sRp[k];
        if (sRp[k + 1] <= first) y[r0 + k] = bz ? T(0) : beta * y[r0 + k];
    }

    int key = 0x7fffffff, startKey = -1, headRow = -1, rowEnd = 0;
    T run = T(0), headVal = T(0);
    if (has) {
        int l = 0, h = nr;  // last local row starting at or before lo
        while (l < h) {
            const int m = (l + h + 1) >> 1;
            if (sRp[m] <= lo) l = m;
            else h = m - 1;
        }
        key = startKey = l;
        rowEnd = sRp[l + 1];
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            const int q = base + e;
            if (q >= lo && q < hi) {
                if (q >= rowEnd) {
                    if (headRow < 0) {
                        headRow = key;
                        headVal = run;
                    } else {
                        y[r0 + key] = axpby(alpha, run, beta, bz, y + r0 + key);
                    }
                    do {
                        ++key;
                        rowEnd = sRp[key + 1];
                    } while (q >= rowEnd);
                    run = T(0);
                }
                run += p[e];
            }
        }
    }

    // Block-wide inclusive segmented scan of (tail row, partial).
    T v = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int k2 = __shfl_up_sync(kFull, key, off);
        const T v2 = __shfl_up_sync(kFull, v, off);
        if (lane >= off && k2 == key) v += v2;
    }
    if (lane == 31) {
        sWarpKey[warp] = key;
        sWarpVal[warp] = v;
    }
    __syncthreads();
    T pre = T(0);
    for (int w = warp - 1; w >= 0; --w) {
        if (sWarpKey[w] != key) break;
        pre += sWarpVal[w];
    }
    v += pre;
    sKey[tid] = key;
    sIncl[tid] = v;
    __syncthreads();

    if (has) {
        const T cin = (tid > 0 && sKey[tid - 1] == startKey) ? sIncl[tid - 1] : T(0);
        if (headRow >= 0) y[r0 + headRow] = axpby(alpha, headVal + cin, beta, bz, y + r0 + headRow);
        if (key < nr && rowEnd == hi) y[r0 + key] = axpby(alpha, v, beta, bz, y + r0 + key);
        if (hi == j1) {
            carryRow[t] = r1;
            carryVal[t] = key == nr ? v : T(0);
        }
    } else if (tid == 0 && j1 == j0) {
        carryRow[t] = r1;
        carryVal[t] = T(0);
    }
}

// Adds the carries of each split row, in tile order, once per row.
template <typename T>
__global__ void merge_fixup_kernel(long long P, int numRows, const int* __restrict__ carryRow,
                                   const T* __restrict__ carryVal, T* __restrict__ y, T alpha) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P) return;
    const int r = carryRow[t];
    if (r >= numRows) return;
    if (t > 0 && carryRow[t - 1] == r) return;
    T s = T(0);
    for (long long u = t; u < P && carryRow[u] == r; ++u) s += carryVal[u];
    y[r] += alpha * s;
}

template <typename T, int BLOCK, int IPT>
static void launch_merge(long long P, const MergeScratch& sc, const RowsArgs<T>& a, cudaStream_t s) {
    merge_tile_kernel<T, BLOCK, IPT><<<(unsigned)P, BLOCK, 0, s>>>(
        a.numRows, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha, a.beta, a.betaZero, sc.tileRow,
        sc.tileNnz, sc.carryRow, static_cast<T*>(sc.carryVal));
}

template <typename T, int BLOCK, int EPT>
static void launch_merge_vec(long long P, const MergeScratch& sc, const RowsArgs<T>& a, cudaStream_t s) {
    merge_vec_kernel<T, BLOCK, EPT><<<(unsigned)P, BLOCK, 0, s>>>(
        a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha, a.beta, a.betaZero, sc.tileRow,
        sc.tileNnz, sc.carryRow, static_cast<T*>(sc.carryVal));
}

template <typename T>
spmv_status_t run_merge(const MergeGeom& g, long long P, const MergeScratch& sc, const RowsArgs<T>& a,
                        cudaStream_t s, cudaEvent_t afterMain) {
    if (P > 0x7fffffffLL) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "too many merge tiles");
    bool ok = true;
    if (g.vec) {
        if (g.block == 256) {
            switch (g.ipt) {
                case 4: launch_merge_vec<T, 256, 4>(P, sc, a, s); break;
                case 8: launch_merge_vec<T, 256, 8>(P, sc, a, s); break;
                case 12: launch_merge_vec<T, 256, 12>(P, sc, a, s); break;
                case 16: launch_merge_vec<T, 256, 16>(P, sc, a, s); break;
                default: ok = false;
            }
        } else if (g.block == 128) {
            switch (g.ipt) {
                case 4: launch_merge_vec<T, 128, 4>(P, sc, a, s); break;
                case 8: launch_merge_vec<T, 128, 8>(P, sc, a, s); break;
                case 12: launch_merge_vec<T, 128, 12>(P, sc, a, s); break;
                case 16: launch_merge_vec<T, 128, 16>(P, sc, a, s); break;
                default: ok = false;
            }
        } else {
            ok = false;
        }
    } else if (g.block == 256) {
        switch (g.ipt) {
            case 3: launch_merge<T, 256, 3>(P, sc, a, s); break;
            case 5: launch_merge<T, 256, 5>(P, sc, a, s); break;
            case 7: launch_merge<T, 256, 7>(P, sc, a, s); break;
            case 9: launch_merge<T, 256, 9>(P, sc, a, s); break;
            case 11: launch_merge<T, 256, 11>(P, sc, a, s); break;
            default: ok = false;
        }
    } else if (g.block == 128) {
        switch (g.ipt) {
            case 3: launch_merge<T, 128, 3>(P, sc, a, s); break;
            case 5: launch_merge<T, 128, 5>(P, sc, a, s); break;
            case 7: launch_merge<T, 128, 7>(P, sc, a, s); break;
            case 9: launch_merge<T, 128, 9>(P, sc, a, s); break;
            case 11: launch_merge<T, 128, 11>(P, sc, a, s); break;
            default: ok = false;
        }
    } else {
        ok = false;
    }
    if (!ok) MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported merge shape block=%d ipt=%d", g.block, g.ipt);
    MXS_LAUNCH_CHECK();
    if (afterMain) MXS_CUDA(cudaEventRecord(afterMain, s));
    return run_merge_fixup<T>(P, sc, a, s);
}

template <typename T>
spmv_status_t run_merge_fixup(long long P, const MergeScratch& sc, const RowsArgs<T>& a, cudaStream_t s) {
    merge_fixup_kernel<T><<<grid_for(P, 256), 256, 0, s>>>(P, a.numRows, sc.carryRow,
                                                          static_cast<const T*>(sc.carryVal), a.y, a.alpha);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}
template spmv_status_t run_merge_fixup<float>(long long, const MergeScratch&, const RowsArgs<float>&, cudaStream_t);
template spmv_status_t run_merge_fixup<double>(long long, const MergeScratch&, const RowsArgs<double>&,
                                               cudaStream_t);

template spmv_status_t run_merge<float>(const MergeGeom&, long long, const MergeScratch&,
                                        const RowsArgs<float>&, cudaStream_t, cudaEvent_t);
template spmv_status_t run_merge<double>(const MergeGeom&, long long, const MergeScratch&,
                                         const RowsArgs<double>&, cudaStream_t, cudaEvent_t);

}  // namespace mxs
