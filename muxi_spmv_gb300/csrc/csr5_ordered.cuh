// Ordered CSR5 tiles: one warp per tile of 32*E consecutive nonzeros, with
// loads and x gathers issued in nonzero order (lane l holds nonzeros
// t*32E + l + 32e, so each load instruction covers 32 consecutive nonzeros
// and gathers of neighbouring columns share sectors).  Shared by the
// one-tile-per-warp and block-range kernels (format_kernels.cu) and the
// x-window kernel (band_kernels.cu); the x gather is a functor, so the
// window kernel serves columns inside its shared-memory window from there.
#pragma once

#include "device.cuh"
#include "csr5_tile.cuh"

namespace mxs {
// CSR5 tiles with the gathers issued in nonzero order: lane l loads nonzeros
// t*32E + l + 32e (every load instruction covers 32 consecutive nonzeros, so
// x gathers of consecutive columns share sectors).
//   * A tile strictly inside one row (tile_row_ptr[t] == tile_row_ptr[t+1]:
//     no row starts in it, the row runs on past its end) -- most tiles of
//     long rows -- needs no row logic: a warp sum of its products becomes the
//     tile's carry.
//   * Any other tile hands each lane its E consecutive products through
//     shared memory and runs the CSR5 row logic.
// Row logic of a tile from its row-start mask, for matrices without empty
// rows.  The mask holds E 32-bit words for the tile's 32E positions: bit k is
// set when a row starts at position k (k >= 1); bit 0 of word 0 instead says
// the tile's last row ends exactly at the tile end.  A lane's first row is
// rFirst plus the set bits up to its first position (a popcount prefix over
// the words); a set bit inside the lane closes the current row.  Same
// results as csr5_tile_rows, without reading rowPtr.
// sY (nullptr: each lane stores its rows into y): a warp region of at least
// 32*E values.  The rows a tile completes are consecutive from rFirst (one
// per row start inside the tile, plus the last row when it ends at the tile
// end); their sums are staged at sY[r - rFirst] and stored to y by one
// coalesced pass instead of one scattered store per row.
template <typename T, int E, typename Acc>
__device__ __forceinline__ void csr5_tile_rows_bits(Acc acc, unsigned word, int rFirst, long long t, int lane,
                                                    int nnz, T* __restrict__ y, T alpha, T beta, bool bz,
                                                    int* __restrict__ carryRow, T* __restrict__ carryVal,
                                                    bool plain, T* sY) {
    constexpr int SIGMA = 32 * E;
    const int tStart = (int)t * SIGMA;
    const int tEnd = min(tStart + SIGMA, nnz);
    // lanes l and l+E, l+2E, ... hold word l % E
    const bool endsAtTileEnd = (__shfl_sync(kFull, word, 0) & 1u) != 0;
    const unsigned clean = (lane % E == 0) ? (word & ~1u) : word;
    const int pc = __popc(clean);
    int incl = pc;
#pragma unroll
    for (int off = 1; off < E; off <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, off, E);
        if (lane % E >= off) incl += v;
    }
    const int w = (E * lane) >> 5, o = (E * lane) & 31;
    const unsigned wordW = __shfl_sync(kFull, clean, w);
    const int exclW = __shfl_sync(kFull, incl - pc, w);
    const unsigned upTo = (o + 1 >= 32) ? 0xffffffffu : ((1u << (o + 1)) - 1u);
    const int startRow = rFirst + exclW + __popc(wordW & upTo);
    const unsigned myBits = (wordW >> o) & (E >= 32 ? 0xffffffffu : ((1u << E) - 1u));
    const unsigned nextFirst = __shfl_down_sync(kFull, myBits & 1u, 1);

    auto put = [&](int r, T s) {
        if (sY) sY[r - rFirst] = s;
        else y[r] = axpbyp(plain, alpha, s, beta, bz, y + r);
    };
    const int j0 = tStart + lane * E;
    const int laneEnd = min(j0 + E, tEnd);
    const bool has = j0 < tEnd;
    int key = has ? startRow : 0x7fffffff;  // lanes without elements sort last in the scan
    int headRow = -1;
    T run = T(0), headVal = T(0);
    if (has) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            if (j0 + e < laneEnd) {
                if (e > 0 && ((myBits >> e) & 1u)) {  // a row starts here: the current one is complete
                    if (headRow < 0) {
                        headRow = key;
                        headVal = run;
                    } else {
                        put(key, run);
                    }
                    ++key;
                    run = T(0);
                }
                run = acc(run, e);
            }
        }
    }
    // does the lane's last row end at its last element?
    const bool endsHere = laneEnd == tEnd ? endsAtTileEnd : (lane < 31 && nextFirst != 0u);

    T incl2 = run;
    // FP64: stop at the longest run of lanes sharing a key (keys rise with the lane)
    const int span = sizeof(T) == 8 ? key_run_length(key, lane) : 32;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        if (off >= span) break;  // warp-uniform
        const int k2 = __shfl_up_sync(kFull, key, off);
        const T v2 = __shfl_up_sync(kFull, incl2, off);
        if (lane >= off && k2 == key) incl2 += v2;
    }
    const int prevKey = __shfl_up_sync(kFull, key, 1);
    const T prevIncl = __shfl_up_sync(kFull, incl2, 1);
    if (has) {
        const T cin = (lane > 0 && prevKey == startRow) ? prevIncl : T(0);
        if (headRow >= 0) put(headRow, headVal + cin);
        if (endsHere) put(key, incl2);
        if (laneEnd == tEnd) {  // the lane holding the tile's last nonzero
            carryRow[t] = endsHere ? -1 : key;
            carryVal[t] = incl2;
        }
    }
    if (sY) {
        // row starts at positions 1..SIGMA-1 (lane E-1 holds the sum over the words)
        const int n = __shfl_sync(kFull, incl, E - 1) + (endsAtTileEnd ? 1 : 0);
        __syncwarp();
        for (int i = lane; i < n; i += 32) y[rFirst + i] = axpbyp(plain, alpha, sY[i], beta, bz, y + rFirst + i);
    }
}


// Products go through shared memory from nonzero order (lane l holds
// nonzeros l + 32e) to lane-contiguous order (lane l takes l*E .. l*E+E-1).
// 8-byte values: for E >= 8 nonzero j sits at slot j + j/16 (served sixteen
// lanes at a time): the writes (fixed e, consecutive lanes) and the reads
// (fixed e, lanes E apart; the pad spreads them over every bank) are both
// free of bank conflicts.
// 4-byte values: a lane reads its E products back as E/4 16-byte words (a
// quarter of the shared-memory instructions of one read per product).
// Product j lies in word f = j/4, component j%4, and word f is stored at
// f ^ ((f >> 3) & 7).  A write instruction (fixed e: 32 consecutive
// products, words 8e..8e+7) and each eight-lane phase of a 16-byte read
// (words 4l+q, 2l+q or l for E = 16, 8, 4) touch eight words whose stored
// positions differ modulo 8, i.e. every bank once: no conflicts either way.
template <typename T, int E>
__device__ __forceinline__ int ordered_slot(int j) {
    return E < 8 ? j : j + (j >> 4);  // 8-byte values
}
__device__ __forceinline__ int swizzled_word(int f) { return f ^ ((f >> 3) & 7); }
template <typename T, int E>
constexpr int ordered_slots() {
    return sizeof(T) == 4 ? 32 * E : (E < 8 ? 32 * E : 34 * E);
}

// sRp / sP: this warp's shared regions (kOrderedRpCap ints, ordered_slots values).
// The rowPtr slice holds up to kOrderedRpCap entries (tiles spanning up to
// 62 rows, nine in ten of the general tiles of a power-law matrix); a tile
// over more rows reads rowPtr from global memory.  Small slices leave the
// SM's L1 to the x gathers.
constexpr int kOrderedRpCap = 64;
template <typename T, int E>
struct OrderedLoad {
    int rFirst, rLast;
    unsigned bits;  // word (lane % E) of the tile's row-start mask (when the plan has masks)
    int c[E];
    T v[E];
};

// VEC (FP32, E a multiple of 4, 16-byte aligned colIdx and values): each
// 128-nonzero chunk of the tile is loaded with one 16-byte load per lane,
// lane l taking nonzeros 4l .. 4l+3 of the chunk, so element e of lane l is
// nonzero 128 * (e / 4) + 4l + e % 4 of the tile (a quarter of the load
// instructions).
template <int E, bool VEC>
__device__ __forceinline__ int ordered_pos(int lane, int e) {
    return VEC ? 128 * (e >> 2) + 4 * lane + (e & 3) : lane + 32 * e;
}

template <typename T, int E, bool VEC = false>
__device__ __forceinline__ void csr5_ordered_load(OrderedLoad<T, E>& L, long long t, int lane, int numRows, int nnz,
                                                  const int* __restrict__ colIdx, const T* __restrict__ values,
                                                  const int* __restrict__ tileRow, long long tiles,
                                                  const unsigned* __restrict__ tileBits) {
    constexpr int SIGMA = 32 * E;
    const int tStart = (int)t * SIGMA;
    L.bits = tileBits ? __ldg(tileBits + t * E + (lane % E)) : 0u;
    if constexpr (VEC) {
        static_assert(sizeof(T) == 4 && E % 4 == 0, "16-byte tile loads: FP32, E a multiple of 4");
        if (tStart + SIGMA <= nnz) {
#pragma unroll
            for (int k = 0; k < E / 4; ++k) {
                const int o = tStart + 128 * k + 4 * lane;
                const int4 c4 = ld_stream4(colIdx + o);
                const float4 v4 = ld_stream4(reinterpret_cast<const float*>(values) + o);
                L.c[4 * k] = c4.x;
                L.c[4 * k + 1] = c4.y;
                L.c[4 * k + 2] = c4.z;
                L.c[4 * k + 3] = c4.w;
                L.v[4 * k] = v4.x;
                L.v[4 * k + 1] = v4.y;
                L.v[4 * k + 2] = v4.z;
                L.v[4 * k + 3] = v4.w;
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int j = tStart + ordered_pos<E, true>(lane, e);
                L.c[e] = j < nnz ? ld_stream(colIdx + j) : 0;
                L.v[e] = j < nnz ? ld_stream(values + j) : T(0);
            }
        }
        L.rFirst = __ldg(tileRow + t);
        L.rLast = t + 1 < tiles ? __ldg(tileRow + t + 1) : numRows - 1;
        return;
    }
    if (tStart + SIGMA <= nnz) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            L.c[e] = ld_stream(colIdx + tStart + lane + 32 * e);
            L.v[e] = ld_stream(values + tStart + lane + 32 * e);
        }
    } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int j = tStart + lane + 32 * e;
            L.c[e] = j < nnz ? ld_stream(colIdx + j) : 0;
            L.v[e] = j < nnz ? ld_stream(values + j) : T(0);
        }
    }
    L.rFirst = __ldg(tileRow + t);
    L.rLast = t + 1 < tiles ? __ldg(tileRow + t + 1) : numRows - 1;
}

// Hands this lane's E consecutive terms to the row logic `rows(acc, sY)`;
// sY is the region once free for staging row sums (FP32) or nullptr (FP64,
// whose terms still read it).  FP32:
// the products go through shared memory (one round trip).  FP64: the values,
// then the gathered x, go through the same region and each term is one FMA
// -- on GB300 the FP64 pipe, not memory, bounds an FP64 SpMV, and a product
// plus an add cost it two instructions per nonzero where the FMA costs one.
template <typename T, int E, bool VEC, typename Rows>
__device__ __forceinline__ void ordered_handoff(const T (&v)[E], const T (&g)[E], int lane, T* sP, Rows rows) {
    if constexpr (sizeof(T) == 8) {
        T a[E];
#pragma unroll
        for (int e = 0; e < E; ++e) sP[ordered_slot<T, E>(lane + 32 * e)] = v[e];
        __syncwarp();
#pragma unroll
        for (int e = 0; e < E; ++e) a[e] = sP[ordered_slot<T, E>(lane * E + e)];
        __syncwarp();
#pragma unroll
        for (int e = 0; e < E; ++e) sP[ordered_slot<T, E>(lane + 32 * e)] = g[e];
        __syncwarp();
        rows([&](T r, int e) { return fma(a[e], sP[ordered_slot<T, E>(lane * E + e)], r); }, nullptr);
    } else {
        if constexpr (VEC) {
            // lane l's elements 4k .. 4k+3 are nonzeros 4(32k + l) .. +3: one
            // 16-byte word, 32 consecutive words per store (conflict-free
            // under the swizzle: eight words of an aligned group per phase)
            float4* w4 = reinterpret_cast<float4*>(sP);
#pragma unroll
            for (int k = 0; k < E / 4; ++k)
                w4[swizzled_word(32 * k + lane)] = make_float4(v[4 * k] * g[4 * k], v[4 * k + 1] * g[4 * k + 1],
                                                               v[4 * k + 2] * g[4 * k + 2], v[4 * k + 3] * g[4 * k + 3]);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int j = lane + 32 * e;
                sP[swizzled_word(j >> 2) * 4 + (j & 3)] = v[e] * g[e];
            }
        }
        __syncwarp();
        T p[E];
        const float4* w4 = reinterpret_cast<const float4*>(sP);
#pragma unroll
        for (int q = 0; q < E / 4; ++q) {
            const float4 w = w4[swizzled_word(lane * (E / 4) + q)];
            p[4 * q] = w.x;
            p[4 * q + 1] = w.y;
            p[4 * q + 2] = w.z;
            p[4 * q + 3] = w.w;
        }
        __syncwarp();  // the region is free again: the row logic may stage row sums in it
        rows([&](T r, int e) { return r + p[e]; }, sP);
    }
}

// betaZero value of the ordered kernels when alpha = 1 and beta = 0 (1: beta
// = 0 only), so that no thread tests alpha in FP64.
constexpr int kPlainAxpby = 3;

// x gather straight from global memory (read-only path, L1 allocating).
template <typename T>
struct GlobalGather {
    const T* __restrict__ x;
    __device__ __forceinline__ T operator()(int c) const { return ld_x(x + c); }
};

// REUSE: the warp runs further tiles on the same shared regions afterwards.
// gather(c): x[c].
template <typename T, int E, bool REUSE, bool VEC = false, typename Gather>
__device__ __forceinline__ void csr5_ordered_compute(const OrderedLoad<T, E>& L, long long t, int lane, int nnz,
                                                     const int* __restrict__ rowPtr, Gather gather,
                                                     T* __restrict__ y, T alpha, T beta, bool bz, long long tiles,
                                                     int* __restrict__ carryRow, T* __restrict__ carryVal,
                                                     bool noEmpty, int* sRp, T* sP, bool useBits, bool plain) {
    const int rFirst = L.rFirst, rLast = L.rLast;
    T g[E];
#pragma unroll
    for (int e = 0; e < E; ++e) g[e] = gather(L.c[e]);  // past nnz: c = 0, v = 0, unused

    // Interior tile of one row.  Tile 0 takes it only when no empty rows
    // precede its row: the row logic writes those leading rows.
    if (rFirst == rLast && t + 1 < tiles && (t > 0 || rFirst == 0)) {
        T sum = T(0);
#pragma unroll
        for (int e = 0; e < E; ++e) sum += L.v[e] * g[e];
        sum = warp_sum_exact(sum);  // FP32: the shuffle butterfly
        if (lane == 0) {
            carryRow[t] = rFirst;
            carryVal[t] = sum;
        }
        return;
    }

    if (useBits) {
        ordered_handoff<T, E, VEC>(L.v, g, lane, sP, [&](auto acc, T* sY) {
            csr5_tile_rows_bits<T, E>(acc, L.bits, rFirst, t, lane, nnz, y, alpha, beta, bz, carryRow, carryVal,
                                      plain, sY);
        });
        if (REUSE) __syncwarp();
        return;
    }
    const int nRp = rLast - rFirst + 2;
    const bool staged = nRp <= kOrderedRpCap;
    if (staged) {
#pragma unroll
        for (int k = 0; k < kOrderedRpCap / 32; ++k) {
            const int i = lane + 32 * k;
            if (i < nRp) sRp[i] = __ldg(rowPtr + rFirst + i);
        }
    }
    ordered_handoff<T, E, VEC>(L.v, g, lane, sP, [&](auto acc, T*) {
        csr5_tile_rows<T, E>(acc, rFirst, rLast, t, lane, nnz, y, alpha, beta, bz, carryRow, carryVal,
                             [&](int r) { return (staged && r >= rFirst) ? sRp[r - rFirst] : __ldg(rowPtr + r); },
                             noEmpty, plain);
    });
    if (REUSE) __syncwarp();  // the regions are reused by this warp's next tile
}

template <typename T, int E>
__device__ __forceinline__ void csr5_ordered_tile(long long t, int lane, int numRows, int nnz,
                                                  const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                                                  const T* __restrict__ values, const T* __restrict__ x,
                                                  T* __restrict__ y, T alpha, T beta, bool bz,
                                                  const int* __restrict__ tileRow, long long tiles,
                                                  int* __restrict__ carryRow, T* __restrict__ carryVal, bool noEmpty,
                                                  const unsigned* __restrict__ tileBits, int* sRp, T* sP,
                                                  bool plain) {
    OrderedLoad<T, E> L;
    csr5_ordered_load<T, E>(L, t, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
    csr5_ordered_compute<T, E, false>(L, t, lane, nnz, rowPtr, GlobalGather<T>{x}, y, alpha, beta, bz, tiles,
                                      carryRow, carryVal, noEmpty, sRp, sP, tileBits != nullptr, plain);
}

}  // namespace mxs
