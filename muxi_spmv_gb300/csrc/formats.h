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
                       const unsigned* tileBits = nullptr);

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
