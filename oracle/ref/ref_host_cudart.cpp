// Host stand-ins for the two CUDA runtime calls that csr_to_ellpack
// (src/spmv/ellpack/spmv_ellpack.cu:58-63) makes after converting on the
// host: allocation and host-to-device copy land in host memory, so the
// reference's conversion output can be read on a machine without a GPU.
// Linked into oracle/_ref/libmuxi_ref.so with -Bsymbolic so that the
// reference code in that library binds to these definitions.
#include <cstdlib>
#include <cstring>
#include <cuda_runtime_api.h>

extern "C" cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::malloc(n ? n : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

extern "C" cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
    std::memcpy(dst, src, n);
    return cudaSuccess;
}
