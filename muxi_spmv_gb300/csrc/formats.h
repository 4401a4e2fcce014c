// CSR5 and ELL SpMV launchers (format_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include "kernels.h"

namespace mxs {

// Carry chains of a CSR5 tiling, built once per matrix: chain c covers tiles
// start[c]..end[c], all ending inside row row[c], which ends in tile end[c]+1.
// They depend only on rowPtr and sigma, so a plan precomputes them and its
// fix-up adds each chain with independent loads.
struct Csr5Chains {
    long long n = -1;  // -1: no table (the fix-up walks carryRow instead)
    const int* start = nullptr;
    const int* end = nullptr;
    const int* row = nullptr;
};

// Builds the chain table for tiles of `sigma` nonzeros.  *buf receives one
// device allocation (cudaMalloc; the caller frees it) holding the three arrays.
spmv_status_t csr5_chains(const int* rowPtr, int numRows, int nnz, int sigma, const int* tileRow, long long tiles,
                          void** buf, Csr5Chains* out, cudaStream_t s);

// Tile kernel then carry fix-up; carryRow/carryVal hold `tiles` entries.
// ordered: gathers issued in nonzero order (csr5_ordered_kernel); with
// chunk > 0 each block of `block` threads owns chunk * block/32 consecutive
// tiles that its warps take one at a time (csr5_ordered_range_kernel).
template <typename T>
spmv_status_t run_csr5(int sigma, const int* tileRow, long long tiles, int* carryRow, T* carryVal,
                       const RowsArgs<T>& a, cudaStream_t s, cudaEvent_t afterMain = nullptr, bool ordered = false,
                       int block = 256, int chunk = 0, const Csr5Chains* chains = nullptr,
                       const unsigned* tileBits = nullptr, bool prefetch = false);

// The carry fix-up behind a CSR5-tiled kernel: with a chain table, one
// thread (or warp) per chain; without one, runs of carryRow walked in tile
// order.  `programmatic`: the tile kernel triggers a programmatic launch, so
// the fix-up is scheduled behind its last wave -- unless an event
// (`afterMain`, recorded here first) sits between them.
template <typename T>
spmv_status_t run_csr5_fixups(long long tiles, const int* carryRow, const T* carryVal, const RowsArgs<T>& a,
                              cudaStream_t s, cudaEvent_t afterMain, const Csr5Chains* chains, bool programmatic);

// Ordered CSR5 tiles over a shared-memory x window per CTA (band_kernels.cu).
// E = nonzeros per lane (8, 16), block = threads per CTA (256, 512, 1024);
// tilesPerWarp: target tiles per warp of a CTA's block range (0: 8); winK:
// window capacity in units of 1,024 elements (0: the largest the shape
// fits).  tileRow / carries / chains / tileBits as run_csr5.  errFlag: device
// int raised (code 2) when a window wait gave up.
struct BandTest {
    long long waitLimit = 0;  // SM clocks of the window wait (0: the default, about two seconds)
    bool inject = false;      // hold back one arrival of the window barrier (the wait runs out)
};
bool band_shape_supported(int block, int E);
template <typename T>
spmv_status_t run_band(int block, int E, int tilesPerWarp, int winK, const int* tileRow, long long tiles,
                       int* carryRow, T* carryVal, int* errFlag, const RowsArgs<T>& a, int numCols, cudaStream_t s,
                       cudaEvent_t afterMain, const Csr5Chains* chains, const unsigned* tileBits,
                       const BandTest& test);

// Ordered CSR5 tiles fed by bulk copies into per-warp shared-memory rings of
// `stages` tiles (stream_kernels.cu), one CTA of `block` threads per SM over
// a contiguous tile range.  FP32: E = 16 with block 512 (3 stages) or 768 (2),
// E = 8 with block 1024 (2 or 3); FP64: E = 8 with block 512 (3) or 1024 (2).
// Arrays that are not 16-byte aligned run the register-prefetching block
// ranges instead.  errFlag: raised (code 3) when a slot wait gave up.
bool stream_shape_supported(int block, int E, int stages, bool dbl);
template <typename T>
spmv_status_t run_stream(int block, int E, int stages, const int* tileRow, long long tiles, int* carryRow,
                         T* carryVal, int* errFlag, const RowsArgs<T>& a, cudaStream_t s, cudaEvent_t afterMain,
                         const Csr5Chains* chains, const unsigned* tileBits, const BandTest& test);

// Row-start masks of a CSR5 tiling for an ordered plan (matrices without
// empty rows): sigma/32 words per tile, one cudaMalloc'd buffer in *buf.
spmv_status_t csr5_tile_bits(const int* rowPtr, int numRows, int sigma, long long tiles, void** buf, cudaStream_t s);

// Adds the carries of rows split between CSR5 tiles, in tile order.
template <typename T>
spmv_status_t run_csr5_fixup(long long tiles, const int* carryRow, const T* carryVal, const RowsArgs<T>& a,
                             cudaStream_t s);

template <typename T>
spmv_status_t run_ell(int numRows, int width, const int* ellCol, const T* ellVal, const T* x, T* y, T alpha, T beta,
                      cudaStream_t s);

}  // namespace mxs
