// One CSR5 tile of 32*E consecutive nonzeros, processed by one warp.
// Shared by csr5_tile_kernel (format_kernels.cu) and the windowed persistent
// kernel (band_kernels.cu); the x gather is a template parameter.
//
// Lane l owns nonzeros [t*32E + l*E, +E): one or two 16-byte loads each of
// colIdx and values (the start is a multiple of 4 elements).  Its first row
// is searched inside [tile_row_ptr[t], tile_row_ptr[t+1]]; it sums per row,
// writes rows that end inside it, and a segmented warp scan joins rows that
// cross lanes.  The row still open at the tile end leaves a carry
// (carryRow[t] = row, or -1).  Empty rows whose position falls in this tile's
// row range get y = beta*y from this tile.
#pragma once

#include "device.cuh"

namespace mxs {

// rowPtr entries staged per warp: rows rFirst..rLast+1 of a tile.  A tile
// without empty rows spans at most 32E+1 rows (32E+2 entries); tiles that
// need more fall back to reading rowPtr from global memory.
template <int E> constexpr int csr5_rp_per_lane() { return E + 1; }
template <int E> constexpr int csr5_rp_cap() { return 32 * csr5_rp_per_lane<E>(); }

template <typename T, int E>
struct Csr5Load {
    int rFirst, rLast;
    int c[E];
    T v[E];
    int rp[csr5_rp_per_lane<E>()];  // this lane's share of the rowPtr slice
};

template <typename T, int E>
__device__ __forceinline__ void csr5_load(Csr5Load<T, E>& L, long long t, int lane, int nnz, long long tiles,
                                          int numRows, const int* __restrict__ tileRow, const int* __restrict__ rowPtr,
                                          const int* __restrict__ colIdx, const T* __restrict__ values) {
    L.rFirst = __ldg(tileRow + t);
    L.rLast = t + 1 < tiles ? __ldg(tileRow + t + 1) : numRows - 1;
    const int nRp = L.rLast - L.rFirst + 2;
#pragma unroll
    for (int k = 0; k < csr5_rp_per_lane<E>(); ++k) {
        const int i = lane + 32 * k;
        L.rp[k] = (nRp <= csr5_rp_cap<E>() && i < nRp) ? __ldg(rowPtr + L.rFirst + i) : 0;
    }
    const int j0 = (int)t * (32 * E) + lane * E;
    if (j0 + E <= nnz) {
#pragma unroll
        for (int q = 0; q < E; q += 4) {
            const int4 c = ld_stream4(colIdx + j0 + q);
            const Quad<T> v = ld_stream_quad(values + j0 + q);
            L.c[q] = c.x;
            L.c[q + 1] = c.y;
            L.c[q + 2] = c.z;
            L.c[q + 3] = c.w;
#pragma unroll
            for (int e = 0; e < 4; ++e) L.v[q + e] = v.v[e];
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const bool in = j0 + e < nnz;
            L.c[e] = in ? ld_stream(colIdx + j0 + e) : 0;
            L.v[e] = in ? ld_stream(values + j0 + e) : T(0);
        }
    }
}

// The row logic of a tile over this lane's E nonzeros: acc(run, e) adds the
// lane's e-th term a_j * x[col_j] to the running row sum (called only for
// positions before the tile end); RP(r): rowPtr[r] for r in [0, rLast+1].
// noEmpty: the caller knows every row holds a nonzero (no empty-row pass).
// plain: alpha = 1 and beta = 0 (y takes the sums as they are).
template <typename T, int E, typename Acc, typename RowPtrAt>
__device__ __forceinline__ void csr5_tile_rows(Acc acc, int rFirst, int rLast, long long t, int lane, int nnz,
                                               T* __restrict__ y, T alpha, T beta, bool bz,
                                               int* __restrict__ carryRow, T* __restrict__ carryVal, RowPtrAt RP,
                                               bool noEmpty = false, bool plain = false) {
    // 32-bit positions: the plans that run these tiles require
    // nnz <= INT_MAX - 32*E*32, so no position below overflows.
    constexpr int SIGMA = 32 * E;
    const int tStart = (int)t * SIGMA;
    const int tEnd = min(tStart + SIGMA, nnz);

    // Empty rows of this tile's range: (rFirst, rLast], plus leading rows for tile 0.
    if (!noEmpty) {
        const int lo = t == 0 ? 0 : rFirst + 1;
        for (int r = lo + lane; r <= rLast; r += 32)
            if (RP(r) == RP(r + 1)) y[r] = bz ? T(0) : beta * y[r];
    }

    const int j0 = tStart + lane * E;
    const int laneEnd = min(j0 + E, tEnd);
    const bool has = j0 < tEnd;

    int key = 0x7fffffff;  // lanes without elements sort last in the scan
    T run = T(0), headVal = T(0);
    int headRow = -1, startRow = -1;
    int rowEnd = 0;
    if (has) {
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
            const int j = j0 + e;
            if (j < laneEnd) {
                if (j >= rowEnd) {
                    // `key` is complete; rows skipped on the way are empty.
                    if (headRow < 0) {
                        headRow = key;
                        headVal = run;
                    } else {
                        y[key] = axpbyp(plain, alpha, run, beta, bz, y + key);
                    }
                    do {
                        ++key;
                        rowEnd = RP(key + 1);
                    } while (j >= rowEnd);
                    run = T(0);
                }
                run = acc(run, e);
            }
        }
    }

    T incl = run;
    // FP64: stop at the longest run of lanes sharing a key (keys rise with the lane)
    const int span = sizeof(T) == 8 ? key_run_length(key, lane) : 32;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        if (off >= span) break;  // warp-uniform
        const int k2 = __shfl_up_sync(kFull, key, off);
        const T v2 = __shfl_up_sync(kFull, incl, off);
        if (lane >= off && k2 == key) incl += v2;
    }
    const int prevKey = __shfl_up_sync(kFull, key, 1);
    const T prevIncl = __shfl_up_sync(kFull, incl, 1);
    if (!has) return;
    const T cin = (lane > 0 && prevKey == startRow) ? prevIncl : T(0);
    if (headRow >= 0) y[headRow] = axpbyp(plain, alpha, headVal + cin, beta, bz, y + headRow);
    if (rowEnd == laneEnd) y[key] = axpbyp(plain, alpha, incl, beta, bz, y + key);  // tail row ends in this lane
    if (laneEnd == tEnd) {  // the lane holding the tile's last nonzero
        carryRow[t] = rowEnd > laneEnd ? key : -1;
        carryVal[t] = incl;
    }
}

// The tile logic with the products formed here.  c/v: this lane's E column
// indices and values; gather(c): x[c].
template <typename T, int E, typename RowPtrAt, typename Gather>
__device__ __forceinline__ void csr5_tile_core(const int (&cIdx)[E], const T (&vals)[E], int rFirst, int rLast,
                                               long long t, int lane, int nnz, T* __restrict__ y, T alpha, T beta,
                                               bool bz, int* __restrict__ carryRow, T* __restrict__ carryVal,
                                               RowPtrAt RP, Gather gather) {
    constexpr int SIGMA = 32 * E;
    const int j0 = (int)t * SIGMA + lane * E;
    const int laneEnd = min(j0 + E, min((int)t * SIGMA + SIGMA, nnz));
    T p[E];
#pragma unroll
    for (int e = 0; e < E; ++e) p[e] = j0 + e < laneEnd ? vals[e] * gather(cIdx[e]) : T(0);
    csr5_tile_rows<T, E>([&](T r, int e) { return r + p[e]; }, rFirst, rLast, t, lane, nnz, y, alpha, beta, bz,
                         carryRow, carryVal, RP);
}

// Tile with register-loaded data (csr5_load): stages the rowPtr slice in this
// warp's shared-memory region sRp (csr5_rp_cap<E>() ints) and runs the core.
template <typename T, int E, typename Gather>
__device__ __forceinline__ void csr5_compute(const Csr5Load<T, E>& L, long long t, int lane, int numRows, int nnz,
                                             const int* __restrict__ rowPtr, T* __restrict__ y, T alpha, T beta,
                                             bool bz, int* __restrict__ carryRow, T* __restrict__ carryVal,
                                             int* sRp, Gather gather) {
    const int rFirst = L.rFirst;
    const bool staged = L.rLast - rFirst + 2 <= csr5_rp_cap<E>();
    if (staged) {
#pragma unroll
        for (int k = 0; k < csr5_rp_per_lane<E>(); ++k) sRp[lane + 32 * k] = L.rp[k];
    }
    __syncwarp();
    csr5_tile_core<T, E>(L.c, L.v, rFirst, L.rLast, t, lane, nnz, y, alpha, beta, bz, carryRow, carryVal,
                         [&](int r) { return (staged && r >= rFirst) ? sRp[r - rFirst] : __ldg(rowPtr + r); },
                         gather);
    (void)numRows;
}

}  // namespace mxs
