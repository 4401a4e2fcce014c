// Device-side helpers shared by the SpMV kernels: cache-hinted loads,
// vector types and segmented warp reductions.  Everything here is written for
// sm_103a (warp 32).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace mxs {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// L2 residency of x.  The matrix streams through L2 once per SpMV while x is
// gathered over and over.  With MXS_L2_HINTS=1 every x gather carries an L2
// evict_last policy and every matrix load an evict_first one (an access
// window per instruction, no device-wide L2 set-aside).  Measured on GB300,
// x stays in L2 without it (DRAM bytes of a power-law SpMV equal the
// algorithmic bytes) and the hinted loads run 0.2-1.2% slower, so the
// default is plain loads.
// ---------------------------------------------------------------------------
#ifndef MXS_L2_HINTS
#define MXS_L2_HINTS 0
#endif
#if MXS_L2_HINTS
#define MXS_STREAM_LD(TY, EXTRA) "ld.global.nc.L1::no_allocate.L2::cache_hint" TY " " EXTRA
#define MXS_X_LD(TY) "ld.global.nc.L2::cache_hint" TY " %0, [%1], %2;"
#else
#define MXS_STREAM_LD(TY, EXTRA) "ld.global.nc.L1::no_allocate" TY " " EXTRA
#define MXS_X_LD(TY) "ld.global.nc" TY " %0, [%1];"
#endif
__device__ __forceinline__ unsigned long long l2_evict_first() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long l2_evict_last() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// ---------------------------------------------------------------------------
// Streaming loads for matrix data (read once per SpMV): no L1 allocation, so
// the L1 keeps the x lines that neighbouring rows re-gather.
// ---------------------------------------------------------------------------
#if MXS_L2_HINTS
#define MXS_POL , "l"(l2_evict_first())
#define MXS_XPOL , "l"(l2_evict_last())
#define MXS_P1 ", %2"
#define MXS_P5 ", %5"
#define MXS_P3 ", %3"
#else
#define MXS_POL
#define MXS_XPOL
#define MXS_P1 ""
#define MXS_P5 ""
#define MXS_P3 ""
#endif
__device__ __forceinline__ int ld_stream(const int* p) {
    int r;
    asm(MXS_STREAM_LD(".s32", "%0, [%1]" MXS_P1 ";") : "=r"(r) : "l"(p) MXS_POL);
    return r;
}
__device__ __forceinline__ float ld_stream(const float* p) {
    float r;
    asm(MXS_STREAM_LD(".f32", "%0, [%1]" MXS_P1 ";") : "=f"(r) : "l"(p) MXS_POL);
    return r;
}
__device__ __forceinline__ double ld_stream(const double* p) {
    double r;
    asm(MXS_STREAM_LD(".f64", "%0, [%1]" MXS_P1 ";") : "=d"(r) : "l"(p) MXS_POL);
    return r;
}
__device__ __forceinline__ int4 ld_stream4(const int* p) {
    int4 r;
    asm(MXS_STREAM_LD(".v4.s32", "{%0,%1,%2,%3}, [%4]" MXS_P5 ";")
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p) MXS_POL);
    return r;
}
__device__ __forceinline__ float4 ld_stream4(const float* p) {
    float4 r;
    asm(MXS_STREAM_LD(".v4.f32", "{%0,%1,%2,%3}, [%4]" MXS_P5 ";")
        : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p) MXS_POL);
    return r;
}
__device__ __forceinline__ double2 ld_stream2(const double* p) {
    double2 r;
    asm(MXS_STREAM_LD(".v2.f64", "{%0,%1}, [%2]" MXS_P3 ";") : "=d"(r.x), "=d"(r.y) : "l"(p) MXS_POL);
    return r;
}

// Gather of x: read-only path, L1 allocating.
__device__ __forceinline__ float ld_x(const float* p) {
    float r;
    asm(MXS_X_LD(".f32") : "=f"(r) : "l"(p) MXS_XPOL);
    return r;
}
__device__ __forceinline__ double ld_x(const double* p) {
    double r;
    asm(MXS_X_LD(".f64") : "=d"(r) : "l"(p) MXS_XPOL);
    return r;
}

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

// axpby that stores s itself when `plain` (alpha = 1 and beta = 0, decided on
// the host: 1*s == s exactly).  GB300 runs FP64 arithmetic at about 1.25
// TFLOP/s per GPU, a small fraction of its FP32 rate, so the FP64 kernels keep
// such instructions -- the alpha == 1 test included -- off the plain y = A x
// path.
template <typename T>
__device__ __forceinline__ T axpbyp(bool plain, T alpha, T s, T beta, bool beta_zero, const T* yp) {
    return plain ? s : axpby(alpha, s, beta, beta_zero, yp);
}

// Longest run of lanes sharing `key`, for keys non-decreasing over the lanes:
// a segmented inclusive scan over such keys is complete after the steps
// with offsets below this length (integer work only; the FP64 adds of the
// skipped steps are what the FP64 kernels save).
__device__ __forceinline__ int key_run_length(int key, int lane) {
    const unsigned same = __match_any_sync(kFull, key);
    return __reduce_max_sync(kFull, (unsigned)(lane - (__ffs(same) - 1) + 1));
}

// Sum over aligned groups of G lanes (G a power of two <= 32).
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}

// Full-warp sum of one double per lane, returned to every lane, computed with
// integer reductions instead of FP64 adds (GB300 runs FP64 arithmetic at
// about two lanes per clock per SM, so five FP64 adds per warp sum cost as
// much as five of a tile's eight FMAs).  Every lane's value is truncated to
// a multiple of 2^(emax - 1079), emax the largest biased exponent in the
// warp, so |V| < 2^57 and the 32-lane sum fits an int64; V is split into
// three fields of 21 unsigned, 21 unsigned and 15 signed bits, each summed
// exactly by redux.sync.  The result is that fixed-point sum rounded once to
// the nearest double (ties to even).  Error: under 32 units of 2^(emax -
// 1079), i.e. below 2^-51 of the largest lane's magnitude, which is no more
// than the sum of the lanes' magnitudes.  Infinities, NaNs and exponents
// near the ends of the range (emax < 64 or > 2040) take the FP64 butterfly.
__device__ __forceinline__ double fixed_to_double(long long t, unsigned emax) {
    if (t == 0) return 0.0;
    const unsigned long long sign = t < 0 ? (1ull << 63) : 0ull;
    unsigned long long m = t < 0 ? 0ull - (unsigned long long)t : (unsigned long long)t;
    const int lz = __clzll((long long)m);  // m < 2^62: lz >= 2
    m <<= lz;                              // leading one at bit 63
    unsigned long long mant = m >> 11;     // 53 bits, leading one at bit 52
    const unsigned long long rest = m & 0x7ffull;
    if (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) ++mant;
    long long be = (long long)emax + 7 - lz;  // value = (m / 2^63) * 2^(63 - lz) * 2^(emax - 1079)
    if (mant >> 53) {
        mant >>= 1;
        ++be;
    }
    return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | (mant & 0xfffffffffffffull)));
}

__device__ __forceinline__ double warp_sum_exact(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    const unsigned emax = __reduce_max_sync(kFull, e);
    if (emax == 0x7ffu || emax < 64u || emax > 2040u) return group_sum<32>(v);  // warp-uniform
    const unsigned long long m = (b & 0xfffffffffffffull) | (e ? (1ull << 52) : 0ull);
    const unsigned d = emax - (e ? e : 1u);
    long long V = d >= 57u ? 0ll : (long long)((m << 4) >> d);
    if (b >> 63) V = -V;
    const unsigned lo = __reduce_add_sync(kFull, (unsigned)V & 0x1fffffu);
    const unsigned mid = __reduce_add_sync(kFull, (unsigned)(V >> 21) & 0x1fffffu);
    const int hi = (int)__reduce_add_sync(kFull, (unsigned)(int)(V >> 42));
    return fixed_to_double(((long long)hi << 42) + ((long long)mid << 21) + (long long)lo, emax);
}
__device__ __forceinline__ float warp_sum_exact(float v) { return group_sum<32>(v); }

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
// Default limit of a bounded wait: about two seconds of SM clock.
constexpr long long kWaitLimitCycles = 4000000000LL;

// Waits for the phase with the given parity to complete; gives up after
// `limit` SM clocks and returns false (the caller records the failure).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  long long limit = kWaitLimitCycles) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long start = clock64();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (clock64() - start > limit) return false;
        __nanosleep(64);
    }
}
// Orders this thread's earlier generic-proxy accesses to shared memory before
// later async-proxy (bulk-copy) writes to the same bytes.
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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
