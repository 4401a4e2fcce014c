// Device-wide exclusive scan and stable LSD radix sort of (uint32 key,
// uint32 value) pairs.  The reorders that must be bit-exact with the
// reference (row-length stable_sort, column sorts with ties by column id,
// the stable column transpose behind the centre-of-mass keys) are all stable
// sorts; LSD radix with a stable scatter gives exactly std::stable_sort's
// order.
//
// Scatter ranking: a 4096-element tile is processed in 16 rounds of 256
// consecutive elements; inside a round, lanes with equal digits are ranked
// with __match_any_sync, warps by per-digit counts in shared memory, and rounds
// by a running per-digit count -- so equal digits keep their input order.
#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "sort.h"

namespace mxs {

constexpr int kScanBlock = 256;
constexpr int kScanIpt = 16;
constexpr int kScanTile = kScanBlock * kScanIpt;

// ---------------------------------------------------------------------------
// Exclusive scan (uint32, wrap-around arithmetic; callers keep totals < 2^32)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* sWarp, unsigned* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned n = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += n;
    }
    if (lane == 31) sWarp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < kScanBlock / 32 ? sWarp[lane] : 0u;
        unsigned wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned n = __shfl_up_sync(kFull, wi, off);
            if (lane >= off) wi += n;
        }
        if (lane < kScanBlock / 32) sWarp[lane] = wi - w;
        if (lane == kScanBlock / 32 - 1) *total = wi;
    }
    __syncthreads();
    const unsigned r = incl - v + sWarp[warp];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanBlock)
scan_tiles_kernel(const unsigned* __restrict__ in, unsigned* __restrict__ out, long long n,
                  unsigned* __restrict__ tileSums) {
    __shared__ unsigned sWarp[kScanBlock / 32];
    __shared__ unsigned sTotal;
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanIpt;
    unsigned v[kScanIpt];
    unsigned s = 0;
#pragma unroll
    for (int u = 0; u < kScanIpt; ++u) {
        v[u] = base + u < n ? in[base + u] : 0u;
        s += v[u];
    }
    unsigned run = block_exclusive_scan(s, sWarp, &sTotal);
#pragma unroll
    for (int u = 0; u < kScanIpt; ++u) {
        if (base + u < n) out[base + u] = run;
        run += v[u];
    }
    if (threadIdx.x == 0 && tileSums) tileSums[blockIdx.x] = sTotal;
}

__global__ void scan_add_kernel(unsigned* __restrict__ out, long long n, const unsigned* __restrict__ tileOffsets) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tileOffsets[i / kScanTile];
}

__global__ void total_kernel(const unsigned* __restrict__ in, const unsigned* __restrict__ out, long long n,
                             unsigned* __restrict__ total) {
    *total = n > 0 ? out[n - 1] + in[n - 1] : 0u;
}

spmv_status_t scan_exclusive_u32(const unsigned* in, unsigned* out, long long n, unsigned* total,
                                 cudaStream_t s) {
    if (n <= 0) {
        if (total) MXS_CUDA(cudaMemsetAsync(total, 0, sizeof(unsigned), s));
        return SPMV_SUCCESS;
    }
    const long long tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 1) {
        scan_tiles_kernel<<<1, kScanBlock, 0, s>>>(in, out, n, nullptr);
        MXS_LAUNCH_CHECK();
    } else {
        void* buf = nullptr;
        MXS_TRY(scratch_alloc(&buf, sizeof(unsigned) * 2 * tiles, s));
        unsigned* sums = static_cast<unsigned*>(buf);
        unsigned* offs = sums + tiles;
        scan_tiles_kernel<<<(unsigned)tiles, kScanBlock, 0, s>>>(in, out, n, sums);
        spmv_status_t st = SPMV_SUCCESS;
        if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
        if (st == SPMV_SUCCESS) st = scan_exclusive_u32(sums, offs, tiles, nullptr, s);
        if (st == SPMV_SUCCESS) {
            scan_add_kernel<<<grid_for(n, 256), 256, 0, s>>>(out, n, offs);
            if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
        }
        scratch_free(buf, s);
        if (st != SPMV_SUCCESS) MXS_FAIL(st, "scan launch failed");
    }
    if (total) {
        total_kernel<<<1, 1, 0, s>>>(in, out, n, total);
        MXS_LAUNCH_CHECK();
    }
    return SPMV_SUCCESS;
}

// ---------------------------------------------------------------------------
// Radix sort
// ---------------------------------------------------------------------------
constexpr int kRsBlock = 256;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsBlock * kRsRounds;
constexpr int kRadix = 256;
constexpr int kRsWarps = kRsBlock / 32;

__global__ void __launch_bounds__(kRsBlock)
radix_hist_kernel(const unsigned* __restrict__ keys, long long n, int shift, unsigned* __restrict__ counts,
                  long long tiles) {
    __shared__ unsigned hist[kRadix];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * kRsTile;
#pragma unroll 4
    for (int r = 0; r < kRsRounds; ++r) {
        const long long i = base + r * kRsBlock + threadIdx.x;
        if (i < n) atomicAdd(&hist[(keys[i] >> shift) & 0xff], 1u);
    }
    __syncthreads();
    counts[(long long)threadIdx.x * tiles + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(kRsBlock)
radix_scatter_kernel(const unsigned* __restrict__ kin, const unsigned* __restrict__ vin,
                     unsigned* __restrict__ kout, unsigned* __restrict__ vout, long long n, int shift,
                     const unsigned* __restrict__ offsets, long long tiles) {
    __shared__ unsigned sBase[kRadix];
    __shared__ unsigned sRun[kRadix];
    __shared__ unsigned sWarp[kRsWarps][kRadix];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    sBase[tid] = offsets[(long long)tid * tiles + blockIdx.x];
    sRun[tid] = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) sWarp[w][tid] = 0;
    __syncthreads();
    const unsigned lowerMask = (1u << lane) - 1u;
    const long long base = (long long)blockIdx.x * kRsTile;
    for (int r = 0; r < kRsRounds; ++r) {
        const long long i = base + r * kRsBlock + tid;
        const bool valid = i < n;
        unsigned key = 0, val = 0;
        if (valid) {
            key = kin[i];
            val = vin[i];
        }
        const unsigned d = (key >> shift) & 0xff;
        const unsigned tag = valid ? d : 0x100u + lane;  // invalid lanes match nobody
        const unsigned peers = __match_any_sync(kFull, tag);
        const unsigned below = __popc(peers & lowerMask);
        if (valid && below == 0) sWarp[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned before = 0;
            for (int w = 0; w < warp; ++w) before += sWarp[w][d];
            const unsigned pos = sBase[d] + sRun[d] + before + below;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        unsigned add = 0;
#pragma unroll
        for (int w = 0; w < kRsWarps; ++w) {
            add += sWarp[w][tid];
            sWarp[w][tid] = 0;
        }
        sRun[tid] += add;
        __syncthreads();
    }
}

spmv_status_t radix_sort_pairs(unsigned* keys, unsigned* vals, long long n, int keyBits, cudaStream_t s) {
    if (n <= 1) return SPMV_SUCCESS;
    if (n > 0xffffffffLL) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "sort size exceeds 2^32");
    if (keyBits < 1) keyBits = 1;
    if (keyBits > 32) keyBits = 32;
    const long long tiles = (n + kRsTile - 1) / kRsTile;
    const long long ncount = tiles * kRadix;
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(unsigned) * (2 * n + 2 * ncount), s));
    unsigned* k2 = static_cast<unsigned*>(buf);
    unsigned* v2 = k2 + n;
    unsigned* counts = v2 + n;
    unsigned* offs = counts + ncount;
    unsigned *ka = keys, *va = vals, *kb = k2, *vb = v2;
    spmv_status_t st = SPMV_SUCCESS;
    int passes = 0;
    for (int shift = 0; shift < keyBits && st == SPMV_SUCCESS; shift += 8, ++passes) {
        radix_hist_kernel<<<(unsigned)tiles, kRsBlock, 0, s>>>(ka, n, shift, counts, tiles);
        if (cudaGetLastError() != cudaSuccess) {
            st = SPMV_ERROR_DEVICE;
            break;
        }
        st = scan_exclusive_u32(counts, offs, ncount, nullptr, s);
        if (st != SPMV_SUCCESS) break;
        radix_scatter_kernel<<<(unsigned)tiles, kRsBlock, 0, s>>>(ka, va, kb, vb, n, shift, offs, tiles);
        if (cudaGetLastError() != cudaSuccess) st = SPMV_ERROR_DEVICE;
        unsigned* t = ka;
        ka = kb;
        kb = t;
        t = va;
        va = vb;
        vb = t;
    }
    if (st == SPMV_SUCCESS && (passes & 1)) {
        cudaError_t e = cudaMemcpyAsync(keys, ka, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(vals, va, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) st = SPMV_ERROR_DEVICE;
    }
    scratch_free(buf, s);
    if (st != SPMV_SUCCESS) MXS_FAIL(st, "radix sort failed: %s", cudaGetErrorString(cudaGetLastError()));
    return SPMV_SUCCESS;
}

int bits_for(unsigned long long maxKey) {
    int b = 0;
    while (b < 64 && (maxKey >> b) != 0) ++b;
    return b < 1 ? 1 : b;
}

}  // namespace mxs
