// Ordered CSR5 tiles with a shared-memory window of x per CTA (the BAND
// kernel family).
//
// CSR5 tiles (reference: spmv_csr5_warp32_kernel,
// src/spmv/csr5/spmv_csr5.cu:148-219) are processed exactly as the ordered
// kernels do (csr5_ordered.cuh: loads and gathers in nonzero order, interior
// tiles as warp sums, row logic for the rest, carries fixed up in tile order),
// but each CTA owns a block range of consecutive tiles and first copies the
// slice of x around its rows into shared memory with one bulk copy
// (cp.async.bulk completing on an mbarrier).  A gather whose column lies in
// the window reads shared memory; every other gather reads x from global
// memory, so the window changes only speed, never results.
//
// Why: random gathers of 32 lanes ran at about 330 G/s from L2-resident x,
// 880 G/s from L1-resident x and 2,130 G/s from shared memory on GB300 (one
// CTA of 1,024 threads per SM, 8 independent gathers per thread): a global
// gather costs the L1 about one tag lookup per lane, a shared one a few bank
// wavefronts per instruction.  On matrices whose columns cluster near the
// diagonal (the 70% near share of the power-law workload, stencils, banded
// matrices) the window turns most gathers into shared-memory reads; the x
// slice crosses from L2 once per CTA (one bulk copy of W elements for
// perBlock * sigma nonzeros), and only the far gathers still go to the L1.
// The window and the hand-off regions come out of the same on-chip memory as
// the L1, where the far gathers and the matrix stream's loads in flight
// land, so the launch asks for no more shared memory than it uses (the
// carve-out below) and windows of 14-20K elements beat larger ones.
//
// Window placement: the CTA's rows [R0, R1] map to columns by the aspect
// ratio C/R; the window of `winCap` elements is centred there and clamped to
// [0, C), with its start a multiple of 16 bytes.  When x is not 16-byte
// aligned the host passes winCap = 0 and every gather reads global memory
// (the dynamic shared memory is then one 16-byte unit).
//
// Waits: each thread waits once on the window's mbarrier, with an iteration
// limit.  A thread that gives up raises *errFlag (code 2), then waits again,
// bounded, so that the copy into its CTA's shared memory has landed before the
// CTA can leave, and returns without computing.  The host reads the flag with
// spmv_plan_device_error.  For tests, `inject` initialises the barrier with
// one arrival that nobody makes until a thread has given up (so the first wait
// always runs out) and `waitLimit` shortens that wait; thread 0 then makes the
// missing arrival, which lets every thread's draining wait complete.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "formats.h"
#include "csr5_ordered.cuh"

namespace mxs {

// Gather through the CTA's window: columns in [lo, lo + span) from shared
// memory, all others from global memory.  With a window each lane executes
// exactly one of two complementary predicated loads (ld.shared for window
// columns, ld.global.nc for the rest): a shared-memory gather of 32 lanes
// costs a few bank wavefronts where a global one costs about one L1 tag
// lookup per lane, and only the lanes outside the window reach the L1.
// Without one (span = 0: x not 16-byte aligned) it is the plain read-only
// load.  The test on span also changes how the compiled code schedules the
// gathers, and measured faster than the same loads without it (4,550 against
// 4,450 GB/s on the 8M-row power law).  What keeps the shared
// loads after the wait for the window's bulk copy is their input `span`,
// which passes through a volatile move placed after that wait.
template <typename T>
struct WindowGather {
    const T* __restrict__ x;
    unsigned win;  // shared-window address of the window
    int lo, span;
    __device__ __forceinline__ T operator()(int c) const {
        if (span == 0) return ld_x(x + c);
        const unsigned o = (unsigned)(c - lo);
        T r;
        if constexpr (sizeof(T) == 4)
            asm("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %1, %2;\n\t@p ld.shared.f32 %0, [%3];\n\t"
                "@!p ld.global.nc.f32 %0, [%4];\n\t}"
                : "=f"(r)
                : "r"(o), "r"((unsigned)span), "r"(win + 4u * o), "l"(x + c));
        else
            asm("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %1, %2;\n\t@p ld.shared.f64 %0, [%3];\n\t"
                "@!p ld.global.nc.f64 %0, [%4];\n\t}"
                : "=d"(r)
                : "r"(o), "r"((unsigned)span), "r"(win + 8u * o), "l"(x + c));
        return r;
    }
};

// Window [lo, lo + span) for rows [R0, R1]: centred on the rows' diagonal
// position (scaled by C/R), clamped to the 16-byte units of x, start a
// multiple of 16 bytes.  span = 0 when no window is used.
template <typename T>
__device__ __forceinline__ void window_bounds(int R0, int R1, int numRows, int numCols, int cap, int& lo,
                                              int& span) {
    constexpr long long A = 16 / sizeof(T);  // elements per 16-byte unit
    const long long cols = (long long)numCols / A * A;
    lo = 0;
    span = 0;
    if (cap <= 0 || cols <= 0) return;
    long long mid = ((long long)R0 + R1) / 2;
    if (numRows != numCols && numRows > 0) mid = mid * numCols / numRows;
    long long l = mid - cap / 2;
    if (l > cols - cap) l = cols - cap;
    if (l < 0) l = 0;
    l = l / A * A;
    const long long h = l + cap < cols ? l + cap : cols;
    lo = (int)l;
    span = (int)(h - l);
}

// Waits for the window; false when the wait gave up (after draining the copy).
__device__ __forceinline__ bool window_wait(unsigned long long* bar, long long limit, int inject,
                                            int* __restrict__ errFlag) {
    if (mbar_wait_bounded(bar, 0, limit)) return true;
    atomicExch(errFlag, 2);
    if (inject && threadIdx.x == 0) mbar_arrive(bar);  // the arrival held back by the test
    mbar_wait_bounded(bar, 0, kWaitLimitCycles);        // the bulk copy lands before the CTA leaves
    return false;
}

// One CTA per block range of `perBlock` tiles; its warps draw the range's
// tiles one at a time from a shared counter (neighbouring rows in flight
// together, no block waits on one long tile).  Dynamic shared memory: the
// window, winCap elements.
template <typename T, int E, int BLOCK, int MINB, bool PF = false, bool VEC = false>
__global__ void __launch_bounds__(BLOCK, MINB)
csr5_window_kernel(int numRows, int numCols, int nnz, const int* __restrict__ rowPtr,
                   const int* __restrict__ colIdx, const T* __restrict__ values, const T* __restrict__ x,
                   T* __restrict__ y, T alpha, T beta, int betaZero, const int* __restrict__ tileRow, long long tiles,
                   int* __restrict__ carryRow, T* __restrict__ carryVal, int noEmptyRows, int perBlock,
                   const unsigned* __restrict__ tileBits, int winCap, int* __restrict__ errFlag, long long waitLimit,
                   int inject) {
    constexpr int WARPS = BLOCK / 32;
    extern __shared__ __align__(128) unsigned char smemDyn[];
    T* win = reinterpret_cast<T*>(smemDyn);
    __shared__ int sRpAll[WARPS][kOrderedRpCap];
    __shared__ __align__(16) T sPAll[WARPS][ordered_slots<T, E>()];
    __shared__ int sNext;
    __shared__ __align__(8) unsigned long long bar;
    pdl_trigger();  // the carry fix-up may be scheduled behind the last wave
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Tile counts fit in int: plans cap nnz below 2^31.
    const int tb = blockIdx.x * perBlock;
    const int te = min(tb + perBlock, (int)tiles);
    int lo, span;
    window_bounds<T>(__ldg(tileRow + tb), te < tiles ? __ldg(tileRow + te) : numRows - 1, numRows, numCols, winCap,
                     lo, span);
    if (threadIdx.x == 0) {
        sNext = tb + WARPS;
        if (span > 0) {
            mbar_init(&bar, inject ? 2 : 1);
            fence_barrier_init();
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && span > 0) {
        mbar_arrive_expect_tx(&bar, (unsigned)(span * sizeof(T)));
        bulk_g2s(win, x + lo, (unsigned)(span * sizeof(T)), &bar);
    }

    const bool bz = betaZero != 0, plain = betaZero == kPlainAxpby;
    const bool useBits = tileBits != nullptr, noEmpty = noEmptyRows != 0;

    int t = tb + w;
    OrderedLoad<T, E> L;
    if (t < te) csr5_ordered_load<T, E, VEC>(L, t, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
    // every thread waits (also warps without a tile: the CTA stays until the copy has landed)
    if (span > 0 && !window_wait(&bar, waitLimit, inject, errFlag)) return;
    int spanAfterWait = span;
    asm volatile("mov.b32 %0, %0;" : "+r"(spanAfterWait));  // orders every window read after the wait
    const WindowGather<T> gather{x, smem_u32(win), lo, spanAfterWait};
    if constexpr (PF) {  // the next tile's loads in flight during this tile's gathers and row logic
        OrderedLoad<T, E> nxt;
        while (t < te) {
            int next = 0;
            if (lane == 0) next = atomicAdd(&sNext, 1);
            next = __shfl_sync(kFull, next, 0);
            if (next < te)
                csr5_ordered_load<T, E, VEC>(nxt, next, lane, numRows, nnz, colIdx, values, tileRow, tiles,
                                             tileBits);
            csr5_ordered_compute<T, E, true, VEC>(L, t, lane, nnz, rowPtr, gather, y, alpha, beta, bz, tiles,
                                                  carryRow, carryVal, noEmpty, sRpAll[w], sPAll[w], useBits, plain);
            L = nxt;
            t = next;
        }
        return;
    }
    while (t < te) {
        int next = 0;  // drawn before the compute so its latency hides under the gathers
        if (lane == 0) next = atomicAdd(&sNext, 1);
        csr5_ordered_compute<T, E, true>(L, t, lane, nnz, rowPtr, gather, y, alpha, beta, bz, tiles, carryRow,
                                         carryVal, noEmpty, sRpAll[w], sPAll[w], useBits, plain);
        t = __shfl_sync(kFull, next, 0);
        if (t < te) csr5_ordered_load<T, E>(L, t, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
    }
}

bool band_shape_supported(int block, int E) {
    return (block == 256 || block == 512 || block == 1024) && (E == 8 || E == 16);
}

// Largest window (elements) of a shape: the largest multiple of 1,024
// elements that keeps MINB CTAs per SM within the SM's shared memory (228 KB,
// 1 KB of it reserved per CTA), capped at 40,960.  Windows default to 16,384
// elements (or this, if smaller): larger ones take L1 from the far gathers.
template <typename T, int E, int BLOCK, int MINB>
static int max_window(const DeviceProps& dp) {
    constexpr size_t staticBytes = (BLOCK / 32) * (kOrderedRpCap * sizeof(int) + ordered_slots<T, E>() * sizeof(T)) + 64;
    const size_t smPerSm = dp.smem_per_sm ? dp.smem_per_sm : 233472;
    const size_t perCta = smPerSm / MINB - 1024;
    size_t room = perCta > staticBytes ? perCta - staticBytes : 0;
    if (dp.smem_optin && room + staticBytes > dp.smem_optin) room = dp.smem_optin - staticBytes;
    long long elems = (long long)(room / sizeof(T)) / 1024 * 1024;
    if (elems > 40960) elems = 40960;
    return (int)(elems < 0 ? 0 : elems);
}

template <typename T, int E, int BLOCK, int MINB, bool PF = false, bool VEC = false>
static spmv_status_t launch_window(const int* tileRow, long long tiles, int* carryRow, T* carryVal, int* errFlag,
                                   const RowsArgs<T>& a, int numCols, int tilesPerWarp, int winK,
                                   const unsigned* bits, const BandTest& test, cudaStream_t s) {
    auto kern = csr5_window_kernel<T, E, BLOCK, MINB, PF, VEC>;
    int dev = 0;
    MXS_CUDA(cudaGetDevice(&dev));
    const DeviceProps& dp = device_props(dev);
    const int maxWin = max_window<T, E, BLOCK, MINB>(dp);
    int cap = winK > 0 ? winK * 1024 : 16384;
    if (cap > maxWin) cap = maxWin;
    const bool aligned = (reinterpret_cast<uintptr_t>(a.x) & 15) == 0;
    if (!aligned) cap = 0;
    static bool attrSet[64] = {false};
    static size_t staticSmem = 0;
    if (dev >= 64 || !attrSet[dev]) {
        MXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(sizeof(T) * (size_t)maxWin > 16 ? sizeof(T) * (size_t)maxWin : 16)));
        cudaFuncAttributes fa{};
        MXS_CUDA(cudaFuncGetAttributes(&fa, kern));
        staticSmem = fa.sharedSizeBytes;
        if (dev < 64) attrSet[dev] = true;
    }
    // at least one 16-byte unit, also when no window is used
    const size_t smem = sizeof(T) * (size_t)cap > 16 ? sizeof(T) * (size_t)cap : 16;
    // Shared-memory carve-out: what MINB CTAs of this launch take (static +
    // window + the 1 KB the system reserves per CTA), the rest stays L1,
    // where the gathers outside the window and the matrix stream's loads in
    // flight land.
    {
        const size_t smPerSm = dp.smem_per_sm ? dp.smem_per_sm : 233472;
        const size_t need = (size_t)MINB * (staticSmem + smem + 1024);
        int pct = (int)((need * 100 + smPerSm - 1) / smPerSm);
        if (pct > 100) pct = 100;
        MXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
    }
    // Whole waves: CTAs hold equal nonzero counts, so the range length is
    // picked to make the CTA count a multiple of the CTAs resident at once.
    int perSm = 0;
    MXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, BLOCK, smem));
    if (perSm < 1) MXS_FAIL(SPMV_ERROR_INTERNAL, "window kernel does not fit an SM (window %d elements)", cap);
    const long long resident = (long long)perSm * dp.sm_count;
    const long long per = fitted_range(tiles, (long long)(tilesPerWarp > 0 ? tilesPerWarp : 8) * (BLOCK / 32),
                                       resident, BLOCK / 32);
    if (per > 0x7fffffffLL) MXS_FAIL(SPMV_ERROR_INTERNAL, "block range too large");
    const long long grid = (tiles + per - 1) / per;
    const int bzFlags = a.betaZero ? (a.alpha == T(1) ? kPlainAxpby : 1) : 0;
    kern<<<(unsigned)grid, BLOCK, smem, s>>>(a.numRows, numCols, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y,
                                             a.alpha, a.beta, bzFlags, tileRow, tiles, carryRow, carryVal,
                                             a.noEmptyRows, (int)per, bits, cap, errFlag,
                                             test.waitLimit > 0 ? test.waitLimit : kWaitLimitCycles,
                                             test.inject ? 1 : 0);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t run_band(int block, int E, int tilesPerWarp, int winK, const int* tileRow, long long tiles,
                       int* carryRow, T* carryVal, int* errFlag, const RowsArgs<T>& a, int numCols, cudaStream_t s,
                       cudaEvent_t afterMain, const Csr5Chains* chains, const unsigned* tileBits,
                       const BandTest& test) {
    if (tiles <= 0) return SPMV_SUCCESS;
    constexpr bool wide = sizeof(T) == 8;
    spmv_status_t st;
#define MXS_WIN(B, EE, M)                                                                                 \
    st = launch_window<T, EE, B, M>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols, tilesPerWarp, \
                                    winK, tileBits, test, s)
    if (block == 512 && E == 16) MXS_WIN(512, 16, 2);
    else if (block == 512 && E == 8) MXS_WIN(512, 8, 2);
    else if (block == 1024 && E == 16) MXS_WIN(1024, 16, 1);
    else if (block == 1024 && E == 8) {
        if constexpr (!wide) {
            // one CTA per SM, the next tile's loads in flight; with 16-byte
            // aligned colIdx / values each lane loads four consecutive
            // nonzeros per instruction (a quarter of the load instructions
            // and of the hand-off stores: this kernel is bound by issue)
            const bool vec = (reinterpret_cast<uintptr_t>(a.colIdx) & 15) == 0 &&
                             (reinterpret_cast<uintptr_t>(a.values) & 15) == 0;
            if (vec)
                st = launch_window<T, 8, 1024, 1, true, true>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols,
                                                              tilesPerWarp, winK, tileBits, test, s);
            else
                st = launch_window<T, 8, 1024, 1, true>(tileRow, tiles, carryRow, carryVal, errFlag, a, numCols,
                                                        tilesPerWarp, winK, tileBits, test, s);
        } else {
            MXS_WIN(1024, 8, 1);
        }
    }
    else if (block == 256 && E == 16) MXS_WIN(256, 16, wide ? 3 : 4);
    else if (block == 256 && E == 8) MXS_WIN(256, 8, 4);
    else MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported band shape block=%d ept=%d", block, E);
#undef MXS_WIN
    MXS_TRY(st);
    return run_csr5_fixups<T>(tiles, carryRow, carryVal, a, s, afterMain, chains, true);
}

template spmv_status_t run_band<float>(int, int, int, int, const int*, long long, int*, float*, int*,
                                       const RowsArgs<float>&, int, cudaStream_t, cudaEvent_t, const Csr5Chains*,
                                       const unsigned*, const BandTest&);
template spmv_status_t run_band<double>(int, int, int, int, const int*, long long, int*, double*, int*,
                                        const RowsArgs<double>&, int, cudaStream_t, cudaEvent_t, const Csr5Chains*,
                                        const unsigned*, const BandTest&);

}  // namespace mxs
