// Device scan / stable radix sort used by the preprocessing kernels.
#pragma once

#include <cuda_runtime.h>
#include "muxi_spmv.h"

namespace mxs {

// out[i] = sum_{k<i} in[k] (uint32); *total (device, optional) = sum of all.
spmv_status_t scan_exclusive_u32(const unsigned* in, unsigned* out, long long n, unsigned* total,
                                 cudaStream_t s);
// Stable ascending sort of (keys, vals) by the low keyBits bits of keys.
// Results replace the inputs.  Scratch comes from the stream-ordered pool.
spmv_status_t radix_sort_pairs(unsigned* keys, unsigned* vals, long long n, int keyBits, cudaStream_t s);
// Number of bits needed to represent maxKey (at least 1).
int bits_for(unsigned long long maxKey);

}  // namespace mxs
