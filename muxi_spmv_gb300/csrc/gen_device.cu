// Device-side synthetic generators for large corpora and batches.
//
// Same length laws as the host generators (generators.cpp builds the
// inverse-CDF table; the device draws from it), but drawn on the GPU, so the
// values differ from the host generator's.  Columns of a row are drawn
// already sorted by exponential spacings: for k columns in [lo, lo+range),
// with E_0..E_k ~ Exp(1) and S = sum E, column i = lo + floor(range *
// (E_0+..+E_i) / S).  Columns may repeat when a row is dense in its range
// (CSR with repeated columns is well defined: the entries add).  Values are
// N(0,1) (Box-Muller); x vectors U[lo,hi].  Stencil laws build the grid
// operators directly.  Each draw is a counter-based hash
// of (seed, row, element), so results do not depend on the launch shape.
#include <vector>

#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "sort.h"

namespace mxs {

bool gen_length_table(const spmv_gen_params_t& p, std::vector<double>& cdf, int& first);

__device__ __forceinline__ unsigned long long dmix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
// Uniform in (0, 1) from (seed, a, b, purpose).
__device__ __forceinline__ double dunif(unsigned long long seed, unsigned long long a, unsigned long long b,
                                        unsigned purpose) {
    const unsigned long long h =
        dmix64(seed * 0x9e3779b97f4a7c15ULL + dmix64(a * 0x632be59bd9b4e019ULL + b * 8 + purpose + 1));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

struct DevLaw {
    int kind, numRows, numCols;
    double p0, p1, p2, p3;
    unsigned long long seed;
};

__device__ __forceinline__ void row_span(const DevLaw& L, int r, int& lo, int& range) {
    switch (L.kind) {
        case SPMV_GEN_BANDED: {
            const int w = max(1, (int)L.p1);
            long long l = (long long)r - w / 2;
            l = l > (long long)L.numCols - w ? (long long)L.numCols - w : l;
            l = l < 0 ? 0 : l;
            lo = (int)l;
            range = (int)min((long long)w, (long long)L.numCols - l);
            return;
        }
        case SPMV_GEN_BLOCKDIAG: {
            const long long nb = max(1LL, (long long)L.p0);
            const long long b = (long long)r * nb / L.numRows;
            lo = (int)(b * L.numCols / nb);
            range = (int)((b + 1) * L.numCols / nb) - lo;
            return;
        }
        default:
            lo = 0;
            range = L.numCols;
    }
}

__global__ void dgen_lengths_kernel(DevLaw L, const double* __restrict__ cdf, int ncdf, int first,
                                    unsigned* __restrict__ len) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= L.numRows) return;
    const double u = dunif(L.seed, r, 0, 0);
    int a = 0, b = ncdf - 1;  // first cdf entry > u
    while (a < b) {
        const int m = (a + b) >> 1;
        if (cdf[m] > u) b = m;
        else a = m + 1;
    }
    int k = first + a;
    int lo, range;
    row_span(L, (int)r, lo, range);
    if (k > range) k = range;
    if (k < 0) k = 0;
    len[r] = (unsigned)k;
}

// Warp per row: two passes over the row's exponential spacings (total, then
// prefix) give sorted columns without a sort.
template <typename T>
__global__ void dgen_fill_kernel(DevLaw L, const int* __restrict__ rowPtr, int* __restrict__ colIdx,
                                 T* __restrict__ values) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= L.numRows) return;
    const int r = (int)w;
    const int s = rowPtr[r], k = rowPtr[r + 1] - s;
    if (k == 0) return;
    int lo, range;
    row_span(L, r, lo, range);
    double total = 0.0;
    for (int i = lane; i <= k; i += 32) total += -log(dunif(L.seed, r, i, 1));
    for (int off = 16; off > 0; off >>= 1) total += __shfl_xor_sync(kFull, total, off);
    double carry = 0.0;
    for (int base = 0; base < k; base += 32) {
        const int i = base + lane;
        double e = i < k ? -log(dunif(L.seed, r, i, 1)) : 0.0;
        double incl = e;
        for (int off = 1; off < 32; off <<= 1) {
            const double v = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += v;
        }
        if (i < k) {
            long long c = lo + (long long)((double)range * ((carry + incl) / total));
            if (c >= (long long)lo + range) c = (long long)lo + range - 1;
            colIdx[s + i] = (int)c;
            const double u1 = dunif(L.seed, r, i, 2), u2 = dunif(L.seed, r, i, 3);
            values[s + i] = (T)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
        }
        carry += __shfl_sync(kFull, incl, 31);
    }
}

// Stencils (no length law): the 5-point Laplacian on an nx x ny grid (4 on
// the diagonal, -1 off it) and the 27-point stencil on n0 x n1 x n2 (N(0,1)
// values), columns ascending -- the host generator's matrices (the 3D values
// come from this file's hash, so they differ from the host's).
__device__ __forceinline__ bool dstencil(const DevLaw& L) {
    return L.kind == SPMV_GEN_STENCIL2D || L.kind == SPMV_GEN_STENCIL3D;
}
__device__ __forceinline__ int dstencil_len(const DevLaw& L, long long r) {
    if (L.kind == SPMV_GEN_STENCIL2D) {
        const long long nx = (long long)L.p0, ny = (long long)L.p1, i = r / ny, j = r % ny;
        return 1 + (i > 0) + (i < nx - 1) + (j > 0) + (j < ny - 1);
    }
    const long long n0 = (long long)L.p0, n1 = (long long)L.p1, n2 = (long long)L.p2;
    const long long k = r / (n1 * n2), rem = r % (n1 * n2), j = rem / n2, i = rem % n2;
    return (1 + (k > 0) + (k < n0 - 1)) * (1 + (j > 0) + (j < n1 - 1)) * (1 + (i > 0) + (i < n2 - 1));
}

__global__ void dgen_stencil_lengths_kernel(DevLaw L, unsigned* __restrict__ len) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < L.numRows) len[r] = (unsigned)dstencil_len(L, r);
}

template <typename T>
__global__ void dgen_stencil_fill_kernel(DevLaw L, const int* __restrict__ rowPtr, int* __restrict__ colIdx,
                                         T* __restrict__ values) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= L.numRows) return;
    int n = rowPtr[r];
    if (L.kind == SPMV_GEN_STENCIL2D) {
        const long long nx = (long long)L.p0, ny = (long long)L.p1, i = r / ny, j = r % ny;
        if (i > 0) { colIdx[n] = (int)(r - ny); values[n++] = T(-1); }
        if (j > 0) { colIdx[n] = (int)(r - 1); values[n++] = T(-1); }
        colIdx[n] = (int)r;
        values[n++] = T(4);
        if (j < ny - 1) { colIdx[n] = (int)(r + 1); values[n++] = T(-1); }
        if (i < nx - 1) { colIdx[n] = (int)(r + ny); values[n++] = T(-1); }
        return;
    }
    const long long n0 = (long long)L.p0, n1 = (long long)L.p1, n2 = (long long)L.p2;
    const long long k = r / (n1 * n2), rem = r % (n1 * n2), j = rem / n2, i = rem % n2;
    int e = 0;
    for (int dk = -1; dk <= 1; ++dk)
        for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di, ++e) {
                const long long kk = k + dk, jj = j + dj, ii = i + di;
                if (kk < 0 || kk >= n0 || jj < 0 || jj >= n1 || ii < 0 || ii >= n2) continue;
                colIdx[n] = (int)((kk * n1 + jj) * n2 + ii);
                const double u1 = dunif(L.seed, r, e, 2), u2 = dunif(L.seed, r, e, 3);
                values[n++] = (T)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
            }
}

__global__ void sum64_kernel(long long n, const unsigned* __restrict__ v, unsigned long long* __restrict__ out) {
    unsigned long long s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += v[i];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

template <typename T>
__global__ void dgen_vector_kernel(long long n, unsigned long long seed, double lo, double hi, T* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (T)(lo + (hi - lo) * dunif(seed, i, 0, 5));
}

static bool device_law_ok(const spmv_gen_params_t* p) {
    if (!p || p->numRows < 0 || p->numCols <= 0) return false;
    if (p->kind == SPMV_GEN_STENCIL2D)
        return p->p0 >= 1 && p->p1 >= 1 && (long long)p->p0 * (long long)p->p1 == p->numRows &&
               p->numRows == p->numCols;
    if (p->kind == SPMV_GEN_STENCIL3D)
        return p->p0 >= 1 && p->p1 >= 1 && p->p2 >= 1 &&
               (long long)p->p0 * (long long)p->p1 * (long long)p->p2 == p->numRows && p->numRows == p->numCols;
    return p->kind == SPMV_GEN_POISSON_UNIFORM || p->kind == SPMV_GEN_ZIPF_UNIFORM || p->kind == SPMV_GEN_BANDED ||
           p->kind == SPMV_GEN_BLOCKDIAG;
}
static bool is_stencil(const spmv_gen_params_t* p) {
    return p->kind == SPMV_GEN_STENCIL2D || p->kind == SPMV_GEN_STENCIL3D;
}

static DevLaw law_of(const spmv_gen_params_t* p) {
    return DevLaw{(int)p->kind, p->numRows, p->numCols, p->p0, p->p1, p->p2, p->p3, p->seed};
}

}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_gen_device_row_ptr(const spmv_gen_params_t* p, int* rowPtr, long long* nnz, cudaStream_t stream) {
    clear_error();
    if (!device_law_ok(p)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "law not available on the device generator");
    if (!rowPtr || !nnz) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL output");
    std::vector<double> cdf;
    int first = 0;
    if (is_stencil(p))
        cdf.assign(1, 1.0);  // unused
    else if (!gen_length_table(*p, cdf, first))
        MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "no length table for this law");
    const long long R = p->numRows;
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(double) * cdf.size() + sizeof(unsigned long long) + sizeof(unsigned) * (R + 2),
                          stream));
    double* dcdf = static_cast<double*>(buf);
    unsigned long long* sum = reinterpret_cast<unsigned long long*>(dcdf + cdf.size());
    unsigned* len = reinterpret_cast<unsigned*>(sum + 1);
    unsigned* total = len + R;
    spmv_status_t st = SPMV_SUCCESS;
    unsigned long long hsum = 0;
    cudaError_t e = cudaMemcpyAsync(dcdf, cdf.data(), sizeof(double) * cdf.size(), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(sum, 0, sizeof(*sum), stream);
    if (e == cudaSuccess && R > 0) {
        if (is_stencil(p))
            dgen_stencil_lengths_kernel<<<grid_for(R, 256), 256, 0, stream>>>(law_of(p), len);
        else
            dgen_lengths_kernel<<<grid_for(R, 256), 256, 0, stream>>>(law_of(p), dcdf, (int)cdf.size(), first, len);
        const unsigned g = grid_for(R, 256);
        sum64_kernel<<<g < 4096u ? g : 4096u, 256, 0, stream>>>(R, len, sum);
        e = cudaGetLastError();
    }
    // nnz must stay below 2^31: check the exact 64-bit sum before the scan.
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hsum, sum, sizeof(hsum), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) st = cuda_fail(e, "device generator", __FILE__, __LINE__);
    if (st == SPMV_SUCCESS && hsum > 0x7fffffffULL) {
        set_error(__FILE__, __LINE__, "generated matrix has %llu nonzeros (limit 2^31-1)", hsum);
        st = SPMV_ERROR_INVALID_MATRIX;
    }
    if (st == SPMV_SUCCESS) st = scan_exclusive_u32(len, reinterpret_cast<unsigned*>(rowPtr), R, total, stream);
    if (st == SPMV_SUCCESS) {
        e = cudaMemcpyAsync(rowPtr + R, total, sizeof(unsigned), cudaMemcpyDeviceToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) st = cuda_fail(e, "device generator", __FILE__, __LINE__);
    }
    scratch_free(buf, stream);
    MXS_TRY(st);
    *nnz = (long long)hsum;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_gen_device_fill_f32(const spmv_gen_params_t* p, const int* rowPtr, int* colIdx, float* values,
                                       cudaStream_t stream) {
    clear_error();
    if (!device_law_ok(p)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "law not available on the device generator");
    if (p->numRows == 0) return SPMV_SUCCESS;
    if (!rowPtr || !colIdx || !values) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL array");
    if (is_stencil(p))
        dgen_stencil_fill_kernel<float><<<grid_for(p->numRows, 256), 256, 0, stream>>>(law_of(p), rowPtr, colIdx,
                                                                                       values);
    else
        dgen_fill_kernel<float><<<grid_for((long long)p->numRows * 32, 256), 256, 0, stream>>>(law_of(p), rowPtr,
                                                                                              colIdx, values);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

spmv_status_t spmv_gen_device_vector_f32(long long n, unsigned long long seed, double lo, double hi, float* out,
                                         cudaStream_t stream) {
    clear_error();
    if (n <= 0) return SPMV_SUCCESS;
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL output");
    const unsigned g = grid_for(n, 256);
    dgen_vector_kernel<float><<<g < 65535u * 4 ? g : 65535u * 4, 256, 0, stream>>>(n, seed, lo, hi, out);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

}  // extern "C"
