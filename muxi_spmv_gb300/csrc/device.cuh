// Device-side helpers shared by the SpMV kernels: cache-hinted loads,
// vector types and segmented warp reductions.  Everything here is written for
// sm_103a (warp 32).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace mxs {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Streaming loads for matrix data (read once per SpMV): no L1 allocation, so
// the L1 keeps the x lines that neighbouring rows re-gather.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ld_stream(const int* p) {
    int r;
    asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ float ld_stream(const float* p) {
    float r;
    asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ double ld_stream(const double* p) {
    double r;
    asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ int4 ld_stream4(const int* p) {
    int4 r;
    asm("ld.global.nc.L1::no_allocate.v4.s32 {%0,%1,%2,%3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ float4 ld_stream4(const float* p) {
    float4 r;
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
        : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ double2 ld_stream2(const double* p) {
    double2 r;
    asm("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];"
        : "=d"(r.x), "=d"(r.y) : "l"(p));
    return r;
}

// Gather of x: read-only path, L1 allocating.
template <typename T>
__device__ __forceinline__ T ld_x(const T* p) { return __ldg(p); }

// Programmatic dependent launch: a kernel calls pdl_trigger() to let the
// next kernel of its stream (launched with programmatic stream
// serialization) be scheduled early; that kernel's pdl_wait() returns once
// the triggering grid has completed and its writes are visible.  Without the
// launch attribute both are no-ops.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Four consecutive values as an array (float: one 16-byte load; double: two).
template <typename T> struct Quad { T v[4]; };
__device__ __forceinline__ Quad<float> ld_stream_quad(const float* p) {
    float4 a = ld_stream4(p);
    return Quad<float>{{a.x, a.y, a.z, a.w}};
}
__device__ __forceinline__ Quad<double> ld_stream_quad(const double* p) {
    double2 a = ld_stream2(p), b = ld_stream2(p + 2);
    return Quad<double>{{a.x, a.y, b.x, b.y}};
}

// y epilogue: y = alpha*s + beta*y, without reading y when beta == 0.
template <typename T>
__device__ __forceinline__ T axpby(T alpha, T s, T beta, bool beta_zero, const T* yp) {
    return beta_zero ? alpha * s : alpha * s + beta * (*yp);
}

// Sum over aligned groups of G lanes (G a power of two <= 32).
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy (TMA) helpers, CTA scope.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Makes barrier initialisation visible to the async (bulk-copy) proxy.
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with the given parity to complete; gives up after
// about two seconds and returns false (the caller records the failure).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long start = clock64();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - start > 4000000000LL) return false;
        __nanosleep(64);
    }
}
// Global -> shared bulk copy completing on `bar` (16-byte aligned, size a
// multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Largest i in [lo, hi] with rowPtr[i] + i <= k: the row of merge-path
// diagonal k.  The merge path of CSR row ends and nnz indices passes through
// (i, k-i) for exactly one i with rowPtr[i] <= k-i <= rowPtr[i+1]; that i is
// the largest one whose row start lies on or before the diagonal.
__device__ __forceinline__ int merge_row_of_diag(const int* __restrict__ rowPtr, int numRows,
                                                 int nnz, long long k) {
    long long lo = k - nnz > 0 ? k - nnz : 0;
    long long hi = k < numRows ? k : numRows;
    while (lo < hi) {
        long long mid = (lo + hi + 1) >> 1;  // upper middle: lo always satisfies
        if ((long long)rowPtr[mid] + mid <= k) lo = mid;
        else hi = mid - 1;
    }
    return (int)lo;
}

// Largest r in [0, numRows-1] with rowPtr[r] <= idx (the row owning nnz idx
// when idx < nnz); -1 when numRows == 0.
__device__ __forceinline__ int row_of_nnz(const int* __restrict__ rowPtr, int numRows, long long idx) {
    int lo = 0, hi = numRows;  // answer + 1 lies in [lo, hi]
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((long long)rowPtr[mid] <= idx) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

}  // namespace mxs
