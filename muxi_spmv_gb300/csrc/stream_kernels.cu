// Ordered CSR5 tiles fed by bulk copies into shared memory (the STREAM
// kernel family).
//
// CSR5 tiles (reference: spmv_csr5_warp32_kernel,
// src/spmv/csr5/spmv_csr5.cu:148-219) are processed exactly as the ordered
// kernels do (csr5_ordered.cuh: gathers in nonzero order, interior tiles as
// warp sums, row logic for the rest, carries fixed up in tile order), but a
// tile's column indices and values do not pass through registers while they
// are in flight.  Each warp owns a ring of S slots in shared memory; lane 0
// requests its next tiles with cp.async.bulk (TMA) copies that complete on
// one mbarrier per slot, S - 1 tiles ahead of the tile being computed.  The
// matrix stream -- two thirds of the bytes of a power-law SpMV -- therefore
// stays in flight while the warp gathers x and runs the row logic, without
// the registers that holding a prefetched tile would take.
//
// Work split: one CTA per SM over a contiguous range of tiles (the range's
// near-diagonal x stays in that SM's L1); warp w of the CTA takes the
// range's tiles w, w + W, w + 2W, ... so its next tiles are known ahead.
// A consumed slot doubles as the warp's product hand-off region before it
// is refilled.  Only tiles whose 32*E nonzeros all exist are copied (the
// copies are whole 16-byte units); the one partial last tile of a matrix is
// loaded with ordinary loads.
//
// Waits: every wait on a slot is bounded.  A warp whose wait gives up raises
// *errFlag (code 3), waits again -- bounded -- for each copy it still has in
// flight, so none lands in shared memory after its CTA left, and returns.
// For tests `inject` initialises every slot barrier with one arrival held
// back, so the first wait runs out; the draining warp then makes the held
// arrivals itself.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "formats.h"
#include "csr5_ordered.cuh"

namespace mxs {

template <typename T, int E>
struct StreamSlot {
    static constexpr int SIGMA = 32 * E;
    static constexpr int COL_BYTES = SIGMA * 4;
    static constexpr int BYTES = SIGMA * (4 + (int)sizeof(T));  // column indices, then values
};

template <typename T, int E, int W, int S>
__global__ void __launch_bounds__(W * 32, 1)
csr5_stream_kernel(int numRows, int nnz, const int* __restrict__ rowPtr, const int* __restrict__ colIdx,
                   const T* __restrict__ values, const T* __restrict__ x, T* __restrict__ y, T alpha, T beta,
                   int betaZero, const int* __restrict__ tileRow, long long tiles, int* __restrict__ carryRow,
                   T* __restrict__ carryVal, int noEmptyRows, int perBlock, const unsigned* __restrict__ tileBits,
                   int* __restrict__ errFlag, long long waitLimit, int inject) {
    using Slot = StreamSlot<T, E>;
    constexpr int SIGMA = Slot::SIGMA;
    static_assert(ordered_slots<T, E>() * (int)sizeof(T) <= Slot::BYTES, "a slot must hold the hand-off region");
    extern __shared__ __align__(128) unsigned char smemDyn[];
    __shared__ int sRpAll[W][kOrderedRpCap];
    __shared__ __align__(8) unsigned long long bars[W][S];
    pdl_trigger();  // the carry fix-up may be scheduled behind the last wave
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* ring = smemDyn + (size_t)w * S * Slot::BYTES;
    // Tile counts fit in int: plans cap nnz below 2^31.
    const int tb = blockIdx.x * perBlock;
    const int te = min(tb + perBlock, (int)tiles);
    const int fullTiles = nnz / SIGMA;  // tiles whose nonzeros all exist
    auto armed = [&](int t) { return t < te && t < fullTiles; };
    auto issue = [&](int t, int s) {  // lane 0: request tile t into slot s
        unsigned char* slot = ring + s * Slot::BYTES;
        mbar_arrive_expect_tx(&bars[w][s], (unsigned)Slot::BYTES);
        bulk_g2s(slot, colIdx + (size_t)t * SIGMA, (unsigned)Slot::COL_BYTES, &bars[w][s]);
        bulk_g2s(slot + Slot::COL_BYTES, values + (size_t)t * SIGMA, (unsigned)(SIGMA * sizeof(T)), &bars[w][s]);
    };
    // The warp's k-th tile is tb + w + k*W and sits in slot k % S, whose
    // barrier completes its phase (k / S) for it.
    auto drain = [&](int k0) {  // after a wait gave up: let every copy in flight land
        atomicExch(errFlag, 3);
        for (int j = 0; j < S; ++j) {
            const int k = k0 + j;
            if (!armed(tb + w + k * W)) continue;
            if (inject && lane == 0) mbar_arrive(&bars[w][k % S]);  // the arrival held back by the test
            mbar_wait_bounded(&bars[w][k % S], (unsigned)((k / S) & 1), kWaitLimitCycles);
        }
    };

    if (lane == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&bars[w][s], inject ? 2 : 1);
        fence_barrier_init();
        for (int s = 0; s < S; ++s)
            if (armed(tb + w + s * W)) issue(tb + w + s * W, s);
    }
    __syncwarp();
    const bool bz = betaZero != 0, plain = betaZero == kPlainAxpby;
    const bool useBits = tileBits != nullptr, noEmpty = noEmptyRows != 0;
    for (int k = 0;; ++k) {
        const int t = tb + w + k * W;
        if (t >= te) break;
        const int s = k % S;
        unsigned char* slot = ring + s * Slot::BYTES;
        OrderedLoad<T, E> L;
        if (armed(t)) {
            if (!mbar_wait_bounded(&bars[w][s], (unsigned)((k / S) & 1), waitLimit)) {
                drain(k);
                return;
            }
            const int* sc = reinterpret_cast<const int*>(slot);
            const T* sv = reinterpret_cast<const T*>(slot + Slot::COL_BYTES);
#pragma unroll
            for (int e = 0; e < E; ++e) {
                L.c[e] = sc[lane + 32 * e];
                L.v[e] = sv[lane + 32 * e];
            }
            L.bits = useBits ? __ldg(tileBits + (long long)t * E + (lane % E)) : 0u;
            L.rFirst = __ldg(tileRow + t);
            L.rLast = t + 1 < tiles ? __ldg(tileRow + t + 1) : numRows - 1;
        } else {
            csr5_ordered_load<T, E>(L, t, lane, numRows, nnz, colIdx, values, tileRow, tiles, tileBits);
        }
        __syncwarp();  // every lane holds its tile: the slot becomes the hand-off region
        csr5_ordered_compute<T, E, true>(L, t, lane, nnz, rowPtr, GlobalGather<T>{x}, y, alpha, beta, bz, tiles,
                                         carryRow, carryVal, noEmpty, sRpAll[w], reinterpret_cast<T*>(slot),
                                         useBits, plain);
        __syncwarp();  // the hand-off is done with the slot
        if (lane == 0 && armed(t + S * W)) {
            fence_proxy_async_shared();  // this warp's generic accesses to the slot precede the copy into it
            issue(t + S * W, s);
        }
    }
}

bool stream_shape_supported(int block, int E, int stages, bool dbl) {
    if (dbl) return E == 8 && ((block == 512 && stages == 3) || (block == 1024 && stages == 2));
    return (E == 16 && ((block == 512 && stages == 3) || (block == 768 && stages == 2))) ||
           (E == 8 && block == 1024 && (stages == 2 || stages == 3));
}

template <typename T, int E, int W, int S>
static spmv_status_t launch_stream(const int* tileRow, long long tiles, int* carryRow, T* carryVal, int* errFlag,
                                   const RowsArgs<T>& a, const unsigned* bits, const BandTest& test,
                                   cudaStream_t s) {
    auto kern = csr5_stream_kernel<T, E, W, S>;
    constexpr size_t smem = (size_t)W * S * StreamSlot<T, E>::BYTES;
    int dev = 0;
    MXS_CUDA(cudaGetDevice(&dev));
    static bool attrSet[64] = {false};
    if (dev >= 64 || !attrSet[dev]) {
        MXS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (dev < 64) attrSet[dev] = true;
    }
    int perSm = 0;
    MXS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, W * 32, smem));
    if (perSm < 1) MXS_FAIL(SPMV_ERROR_INTERNAL, "stream kernel does not fit an SM (%zu bytes of rings)", smem);
    const long long resident = (long long)perSm * device_props(dev).sm_count;
    const long long per = fitted_range(tiles, (tiles + resident - 1) / resident, resident, W);
    if (per > 0x7fffffffLL) MXS_FAIL(SPMV_ERROR_INTERNAL, "tile range too large");
    const int bzFlags = a.betaZero ? (a.alpha == T(1) ? kPlainAxpby : 1) : 0;
    kern<<<grid_for(tiles, (int)per), W * 32, smem, s>>>(
        a.numRows, a.nnz, a.rowPtr, a.colIdx, a.values, a.x, a.y, a.alpha, a.beta, bzFlags, tileRow, tiles, carryRow,
        carryVal, a.noEmptyRows, (int)per, bits, errFlag, test.waitLimit > 0 ? test.waitLimit : kWaitLimitCycles,
        test.inject ? 1 : 0);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t run_stream(int block, int E, int stages, const int* tileRow, long long tiles, int* carryRow,
                         T* carryVal, int* errFlag, const RowsArgs<T>& a, cudaStream_t s, cudaEvent_t afterMain,
                         const Csr5Chains* chains, const unsigned* tileBits, const BandTest& test) {
    if (tiles <= 0) return SPMV_SUCCESS;
    // Bulk copies start on 16-byte boundaries: other arrays take the
    // register-prefetching block ranges (same tiles, same results).
    if (!(aligned16(a.colIdx) && aligned16(a.values)))
        return run_csr5<T>(32 * E, tileRow, tiles, carryRow, carryVal, a, s, afterMain, true, 1024, 1 << 20, chains,
                           tileBits, true);
    spmv_status_t st;
    if constexpr (sizeof(T) == 8) {
        if (E == 8 && block == 512 && stages == 3) st = launch_stream<T, 8, 16, 3>(tileRow, tiles, carryRow, carryVal, errFlag, a, tileBits, test, s);
        else if (E == 8 && block == 1024 && stages == 2) st = launch_stream<T, 8, 32, 2>(tileRow, tiles, carryRow, carryVal, errFlag, a, tileBits, test, s);
        else MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported FP64 stream shape block=%d ept=%d stages=%d", block, E, stages);
    } else {
        if (E == 16 && block == 512 && stages == 3) st = launch_stream<T, 16, 16, 3>(tileRow, tiles, carryRow, carryVal, errFlag, a, tileBits, test, s);
        else if (E == 16 && block == 768 && stages == 2) st = launch_stream<T, 16, 24, 2>(tileRow, tiles, carryRow, carryVal, errFlag, a, tileBits, test, s);
        else if (E == 8 && block == 1024 && stages == 3) st = launch_stream<T, 8, 32, 3>(tileRow, tiles, carryRow, carryVal, errFlag, a, tileBits, test, s);
        else if (E == 8 && block == 1024 && stages == 2) st = launch_stream<T, 8, 32, 2>(tileRow, tiles, carryRow, carryVal, errFlag, a, tileBits, test, s);
        else MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported stream shape block=%d ept=%d stages=%d", block, E, stages);
    }
    MXS_TRY(st);
    return run_csr5_fixups<T>(tiles, carryRow, carryVal, a, s, afterMain, chains, true);
}

template spmv_status_t run_stream<float>(int, int, int, const int*, long long, int*, float*, int*,
                                         const RowsArgs<float>&, cudaStream_t, cudaEvent_t, const Csr5Chains*,
                                         const unsigned*, const BandTest&);
template spmv_status_t run_stream<double>(int, int, int, const int*, long long, int*, double*, int*,
                                          const RowsArgs<double>&, cudaStream_t, cudaEvent_t, const Csr5Chains*,
                                          const unsigned*, const BandTest&);

}  // namespace mxs
