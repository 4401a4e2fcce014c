// C ABI: handle, error reporting, stateless CSR execution, merge-path entry
// points and plans.  Reference surface: src/api/spmv_api.{h,cu},
// src/spmv/csr/spmv_csr.cu:52-249, src/spmv/csr5/spmv_csr5.cu:930-1014.
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.h"
#include "preprocess.h"
#include "kernels.h"
#include "plan.h"

namespace mxs {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = {0};

void set_error(const char* file, int line, const char* fmt, ...) {
    char msg[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    const char* base = strrchr(file, '/');
    snprintf(g_err, sizeof g_err, "%s (%s:%d)", msg, base ? base + 1 : file, line);
}

void clear_error() { g_err[0] = 0; }

spmv_status_t cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    set_error(file, line, "CUDA error in %s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SPMV_ERROR_MEMORY_ALLOC : SPMV_ERROR_DEVICE;
}

// ---------------------------------------------------------------------------
// Device properties
// ---------------------------------------------------------------------------
static std::mutex g_props_mu;
static std::vector<DeviceProps> g_props;

const DeviceProps& device_props(int dev) {
    std::lock_guard<std::mutex> lk(g_props_mu);
    if ((int)g_props.size() <= dev) g_props.resize(dev + 1);
    DeviceProps& p = g_props[dev];
    if (p.sm_count == 0) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
            p.sm_count = prop.multiProcessorCount;
            p.l2_bytes = prop.l2CacheSize;
            p.smem_optin = prop.sharedMemPerBlockOptin;
            p.smem_per_sm = prop.sharedMemPerMultiprocessor;
            p.cc_major = prop.major;
            p.cc_minor = prop.minor;
        }
    }
    return p;
}

int current_sm_count() {
    int dev = 0;
    cudaGetDevice(&dev);
    const int n = device_props(dev).sm_count;
    return n > 0 ? n : 1;
}

// ---------------------------------------------------------------------------
// Stream-ordered scratch: one memory pool per device that keeps its memory
// between calls (release threshold = unlimited), so repeated stateless calls
// do not return memory to the CUDA driver and re-map it.
// ---------------------------------------------------------------------------
static std::mutex g_pool_mu;
static std::vector<cudaMemPool_t> g_pools;

static spmv_status_t pool_for_current(cudaMemPool_t* out) {
    int dev = 0;
    MXS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if ((int)g_pools.size() <= dev) g_pools.resize(dev + 1, nullptr);
    if (!g_pools[dev]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        MXS_CUDA(cudaMemPoolCreate(&pool, &props));
        unsigned long long thr = ~0ull;
        MXS_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return SPMV_SUCCESS;
}

spmv_status_t scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
    cudaMemPool_t pool;
    MXS_TRY(pool_for_current(&pool));
    if (bytes == 0) bytes = 256;
    cudaError_t e = dev_malloc_pool_async(p, bytes, pool, s);
    if (e != cudaSuccess) {
        set_error(__FILE__, __LINE__, "scratch allocation of %zu bytes failed: %s", bytes,
                  cudaGetErrorString(e));
        return SPMV_ERROR_MEMORY_ALLOC;
    }
    return SPMV_SUCCESS;
}

spmv_status_t scratch_free(void* p, cudaStream_t s) {
    if (!p) return SPMV_SUCCESS;
    MXS_CUDA(dev_free_async(p, s));
    return SPMV_SUCCESS;
}

// ---------------------------------------------------------------------------
// Shared execution helpers
// ---------------------------------------------------------------------------
template <typename T>
static spmv_status_t check_csr_args(int R, int C, int N, const int* rowPtr, const int* colIdx,
                                    const T* values, const T* x, const T* y) {
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension (R=%d C=%d nnz=%d)", R, C, N);
    if (R > 0 && !rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (N > 0 && (!colIdx || !values)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx/values is NULL");
    if (R > 0 && !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y is NULL");
    if (N > 0 && !x) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x is NULL");
    return SPMV_SUCCESS;
}

const MergeGeom kDefaultMerge = {256, 8, 4};

template <typename T>
spmv_status_t merge_stateless(const MergeGeom& g, const RowsArgs<T>& a, cudaStream_t s) {
    const long long P = merge_tile_count(a.numRows, a.nnz, g);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, merge_scratch_bytes(P, sizeof(T)), s));
    MergeScratch sc = merge_carve(buf, P, sizeof(T));
    spmv_status_t st = merge_tile_coords(a.rowPtr, a.numRows, a.nnz, g, P, sc.tileRow, sc.tileNnz, s);
    if (st == SPMV_SUCCESS) st = run_merge<T>(g, P, sc, a, s);
    spmv_status_t st2 = scratch_free(buf, s);
    return st != SPMV_SUCCESS ? st : st2;
}

// The default stateless SpMV: CSR5 tiles of 256 nonzeros found for this call
// (one binary search per tile), the ordered tile kernel (128-thread blocks)
// and the tile-walking carry fix-up, all in stream-ordered scratch.  (A call
// has no row-start masks, without which 256-nonzero tiles beat 512.)
template <typename T>
spmv_status_t csr5_stateless(const RowsArgs<T>& a, cudaStream_t s) {
    constexpr int kSigma = 256;
    const long long tiles = ((long long)a.nnz + kSigma - 1) / kSigma;
    const size_t a4 = ((sizeof(int) * tiles) + 255) & ~size_t(255);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, 2 * a4 + sizeof(T) * tiles, s));
    int* tileRow = static_cast<int*>(buf);
    int* carryRow = reinterpret_cast<int*>(static_cast<char*>(buf) + a4);
    T* carryVal = reinterpret_cast<T*>(static_cast<char*>(buf) + 2 * a4);
    spmv_status_t st = csr5_tiles(a.rowPtr, a.numRows, a.nnz, kSigma, tileRow, nullptr, s);
    if (st == SPMV_SUCCESS)
        st = run_csr5<T>(kSigma, tileRow, tiles, carryRow, carryVal, a, s, nullptr, true, 128, 0, nullptr, nullptr);
    const spmv_status_t st2 = scratch_free(buf, s);
    return st != SPMV_SUCCESS ? st : st2;
}

template <typename T>
static spmv_status_t finish(const spmv_opts_t* opts, cudaStream_t s) {
    if (opts && opts->sync) MXS_CUDA(cudaStreamSynchronize(s));
    return SPMV_SUCCESS;
}

template <typename T>
static spmv_status_t csr_exec(const spmv_variant_t* v, int R, int C, int N, const int* rowPtr,
                              const int* colIdx, const T* values, const T* x, T* y, T alpha, T beta,
                              const spmv_opts_t* opts);

// y = alpha*A^T*x + beta*y (x has R entries, y has C): the transpose is built
// in stream-ordered scratch (csr_transpose) and run as a normal CSR SpMV, so
// the result is deterministic (the reference scattered with float atomics,
// spmv_csr.cuh:105-107).
template <typename T>
static spmv_status_t csr_exec_transpose(const spmv_variant_t* v, int R, int C, int N, const int* rowPtr,
                                        const int* colIdx, const T* values, const T* x, T* y, T alpha, T beta,
                                        const spmv_opts_t* opts) {
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension (R=%d C=%d nnz=%d)", R, C, N);
    if (R > 0 && !rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (N > 0 && (!colIdx || !values)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx/values is NULL");
    if (C > 0 && !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y (numCols entries) is NULL");
    if (N > 0 && !x) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x (numRows entries) is NULL");
    const cudaStream_t s = opts_stream(opts);
    if (C == 0) return SPMV_SUCCESS;
    const size_t a = (sizeof(int) * ((size_t)C + 1) + 255) & ~size_t(255);
    const size_t b = (sizeof(int) * (size_t)(N > 0 ? N : 1) + 255) & ~size_t(255);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, a + b + sizeof(T) * (size_t)(N > 0 ? N : 1), s));
    int* tRp = static_cast<int*>(buf);
    int* tCi = reinterpret_cast<int*>(static_cast<char*>(buf) + a);
    T* tVa = reinterpret_cast<T*>(static_cast<char*>(buf) + a + b);
    spmv_status_t st = csr_transpose<T>(R, C, N, rowPtr, colIdx, values, tRp, tCi, tVa, s);
    if (st == SPMV_SUCCESS) {
        spmv_opts_t o = opts ? *opts : spmv_default_opts();
        o.operation = SPMV_OP_NORMAL;
        st = csr_exec<T>(v, C, R, N, tRp, tCi, tVa, x, y, alpha, beta, &o);
    }
    scratch_free(buf, s);
    return st;
}

template <typename T>
static spmv_status_t csr_exec(const spmv_variant_t* v, int R, int C, int N, const int* rowPtr,
                              const int* colIdx, const T* values, const T* x, T* y, T alpha, T beta,
                              const spmv_opts_t* opts) {
    clear_error();
    if (opts && opts->operation == SPMV_OP_TRANSPOSE)
        return csr_exec_transpose<T>(v, R, C, N, rowPtr, colIdx, values, x, y, alpha, beta, opts);
    if (opts && opts->operation != SPMV_OP_NORMAL)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "SPMV_OP_CONJUGATE is not supported (real types only)");
    MXS_TRY(check_csr_args<T>(R, C, N, rowPtr, colIdx, values, x, y));
    const cudaStream_t s = opts_stream(opts);
    if (R == 0) return SPMV_SUCCESS;
    if (N == 0) {
        MXS_TRY(run_scale<T>(R, y, beta, s));
        return finish<T>(opts, s);
    }
    RowsArgs<T> a{R, N, rowPtr, colIdx, values, x, y, alpha, beta, beta == T(0)};
    if ((!v || v->kernel == SPMV_KERNEL_AUTO) && N <= 0x7fffffff - 32768) {
        MXS_TRY(csr5_stateless<T>(a, s));
        return finish<T>(opts, s);
    }
    spmv_variant_t def{SPMV_KERNEL_MERGE, 256, 0, 8, 4};
    if (!v) v = &def;
    switch (v->kernel) {
        case SPMV_KERNEL_SCALAR:
            MXS_TRY(run_rows<T>(v->blockSize ? v->blockSize : 256, 1, 1, a, s));
            break;
        case SPMV_KERNEL_VECTOR:
            MXS_TRY(run_rows<T>(v->blockSize ? v->blockSize : 256, v->threadsPerRow ? v->threadsPerRow : 32,
                                v->vectorWidth == 4 ? 4 : 1, a, s));
            break;
        case SPMV_KERNEL_MERGE:
        case SPMV_KERNEL_AUTO: {
            MergeGeom g = v->kernel == SPMV_KERNEL_AUTO ? kDefaultMerge : merge_geom_of(*v);
            if (g.vec && !(aligned16(colIdx) && aligned16(values))) g = merge_unaligned_geom(g);
            if (!merge_geom_supported(g))
                MXS_FAIL(SPMV_ERROR_INTERNAL, "unsupported merge shape block=%d ipt=%d", g.block, g.ipt);
            MXS_TRY(merge_stateless<T>(g, a, s));
            break;
        }
        default:
            MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "kernel %d needs a plan (CSR5/ELL metadata)", (int)v->kernel);
    }
    return finish<T>(opts, s);
}

// COO SpMV: the matrix is converted to CSR in stream-ordered scratch
// (coo_to_csr), then runs as the stateless CSR call.
template <typename T>
static spmv_status_t coo_exec(int R, int C, int N, const int* rowIdx, const int* colIdx, const T* values, const T* x,
                              T* y, T alpha, T beta, const spmv_opts_t* opts) {
    clear_error();
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (opts && opts->operation != SPMV_OP_NORMAL)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "COO SpMV supports SPMV_OP_NORMAL only");
    const cudaStream_t s = opts_stream(opts);
    const size_t ar = (sizeof(int) * ((size_t)R + 1) + 255) & ~size_t(255);
    const size_t ac = (sizeof(int) * (size_t)N + 255) & ~size_t(255);
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, ar + ac + sizeof(T) * (size_t)N + 16, s));
    int* rp = static_cast<int*>(buf);
    int* ci = reinterpret_cast<int*>(static_cast<char*>(buf) + ar);
    T* va = reinterpret_cast<T*>(static_cast<char*>(buf) + ar + ac);
    spmv_status_t st = coo_to_csr<T>(R, C, N, rowIdx, colIdx, values, rp, ci, va, s);
    if (st == SPMV_SUCCESS) {
        spmv_opts_t o = opts ? *opts : spmv_default_opts();
        o.sync = 0;
        st = csr_exec<T>(nullptr, R, C, N, rp, ci, va, x, y, alpha, beta, &o);
    }
    const spmv_status_t st2 = scratch_free(buf, s);
    MXS_TRY(st);
    MXS_TRY(st2);
    if (opts && opts->sync) MXS_CUDA(cudaStreamSynchronize(s));
    return SPMV_SUCCESS;
}

}  // namespace mxs

using namespace mxs;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

spmv_opts_t spmv_default_opts(void) {
    spmv_opts_t o;
    o.operation = SPMV_OP_NORMAL;
    o.sync = 0;
    o.check_inputs = 0;
    o.use_tensor_core = 0;
    o.use_streaming = 0;
    o.stream_id = 0;
    o.stream = nullptr;
    return o;
}

const char* spmv_last_error(void) { return g_err; }
int spmv_abi_version(void) { return MUXI_SPMV_ABI_VERSION; }

spmv_status_t spmv_create_handle(spmv_handle_t** handle) {
    clear_error();
    if (!handle) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle pointer is NULL");
    *handle = nullptr;
    int dev = 0;
    MXS_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    MXS_CUDA(cudaGetDeviceProperties(&prop, dev));
    spmv_handle_t* h = new (std::nothrow) spmv_handle_t();
    if (!h) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    h->deviceId = dev;
    h->stream = nullptr;
    h->opts = spmv_default_opts();
    h->warpSize = prop.warpSize;
    h->smCount = prop.multiProcessorCount;
    h->maxThreadsPerBlock = prop.maxThreadsPerBlock;
    h->sharedMemPerSM = prop.sharedMemPerMultiprocessor;
    h->l2CacheBytes = prop.l2CacheSize;
    h->sharedMemPerBlockOptin = prop.sharedMemPerBlockOptin;
    h->ccMajor = prop.major;
    h->ccMinor = prop.minor;
    h->internal = new (std::nothrow) HandleState{dev};
    *handle = h;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_destroy_handle(spmv_handle_t* handle) {
    clear_error();
    if (!handle) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    delete static_cast<HandleState*>(handle->internal);
    delete handle;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_set_stream(spmv_handle_t* handle, cudaStream_t stream) {
    clear_error();
    if (!handle) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    handle->stream = stream;
    handle->opts.stream = reinterpret_cast<void*>(stream);
    return SPMV_SUCCESS;
}

spmv_status_t spmv_csr_f32(int R, int C, int N, const int* rowPtr, const int* colIdx, const float* values,
                           const float* x, float* y, float alpha, float beta, const spmv_opts_t* opts) {
    return csr_exec<float>(nullptr, R, C, N, rowPtr, colIdx, values, x, y, alpha, beta, opts);
}
spmv_status_t spmv_csr_f64(int R, int C, int N, const int* rowPtr, const int* colIdx, const double* values,
                           const double* x, double* y, double alpha, double beta, const spmv_opts_t* opts) {
    return csr_exec<double>(nullptr, R, C, N, rowPtr, colIdx, values, x, y, alpha, beta, opts);
}

spmv_status_t spmv_csr_variant_f32(const spmv_variant_t* v, int R, int C, int N, const int* rowPtr,
                                   const int* colIdx, const float* values, const float* x, float* y,
                                   float alpha, float beta, const spmv_opts_t* opts) {
    if (!v) {
        set_error(__FILE__, __LINE__, "variant is NULL");
        return SPMV_ERROR_INTERNAL;
    }
    return csr_exec<float>(v, R, C, N, rowPtr, colIdx, values, x, y, alpha, beta, opts);
}
spmv_status_t spmv_csr_variant_f64(const spmv_variant_t* v, int R, int C, int N, const int* rowPtr,
                                   const int* colIdx, const double* values, const double* x, double* y,
                                   double alpha, double beta, const spmv_opts_t* opts) {
    if (!v) {
        set_error(__FILE__, __LINE__, "variant is NULL");
        return SPMV_ERROR_INTERNAL;
    }
    return csr_exec<double>(v, R, C, N, rowPtr, colIdx, values, x, y, alpha, beta, opts);
}

int spmv_merge_default_partitions(int numRows, int nnz) {
    // spmv_csr5.cu:941-972 for warp 32: elementsPerPartition 32, 128 SMs,
    // 8 warps per 256-thread block, multiplier 8.
    const long long L = (long long)numRows + nnz;
    const long long target = L / 32;
    const long long maxP = 128LL * 8 * 8;
    long long p = target < maxP ? target : maxP;
    return (int)(p < 1 ? 1 : p);
}

spmv_status_t spmv_merge_partitions(int numRows, int nnz, int P, int* pos, cudaStream_t stream) {
    clear_error();
    if (numRows < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    return merge_partitions(numRows, nnz, P, pos, stream);
}

spmv_status_t spmv_merge_path_search(const int* rowPtr, int numRows, int nnz, const int* diag, int count,
                                     int* rowIdx, int* nnzIdx, cudaStream_t stream) {
    clear_error();
    if (numRows < 0 || nnz < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    return merge_search(rowPtr, numRows, nnz, diag, count, rowIdx, nnzIdx, stream);
}

spmv_status_t spmv_coo_f32(int R, int C, int N, const int* rowIdx, const int* colIdx, const float* values,
                           const float* x, float* y, float alpha, float beta, const spmv_opts_t* opts) {
    return coo_exec<float>(R, C, N, rowIdx, colIdx, values, x, y, alpha, beta, opts);
}
spmv_status_t spmv_coo_f64(int R, int C, int N, const int* rowIdx, const int* colIdx, const double* values,
                           const double* x, double* y, double alpha, double beta, const spmv_opts_t* opts) {
    return coo_exec<double>(R, C, N, rowIdx, colIdx, values, x, y, alpha, beta, opts);
}

spmv_status_t spmv_merge_based_f32(int R, int C, int N, const int* rowPtr, const int* colIdx, const float* values,
                                   const float* x, float* y, cudaStream_t stream) {
    spmv_variant_t v{SPMV_KERNEL_MERGE, 256, 0, 8, 4};
    spmv_opts_t o = spmv_default_opts();
    o.stream = reinterpret_cast<void*>(stream);
    return csr_exec<float>(&v, R, C, N, rowPtr, colIdx, values, x, y, 1.0f, 0.0f, &o);
}
spmv_status_t spmv_merge_based_f64(int R, int C, int N, const int* rowPtr, const int* colIdx,
                                   const double* values, const double* x, double* y, cudaStream_t stream) {
    spmv_variant_t v{SPMV_KERNEL_MERGE, 256, 0, 8, 4};
    spmv_opts_t o = spmv_default_opts();
    o.stream = reinterpret_cast<void*>(stream);
    return csr_exec<double>(&v, R, C, N, rowPtr, colIdx, values, x, y, 1.0, 0.0, &o);
}

spmv_status_t spmv_count_distinct_columns(int numCols, int nnz, const int* colIdx, long long* distinct,
                                          cudaStream_t stream) {
    clear_error();
    return count_distinct_columns(numCols, nnz, colIdx, distinct, stream);
}

spmv_status_t spmv_validate_csr(int numRows, int numCols, int nnz, const int* rowPtr, const int* colIdx,
                                long long* bad, cudaStream_t stream) {
    clear_error();
    return validate_csr(numRows, numCols, nnz, rowPtr, colIdx, bad, stream);
}

}  // extern "C"
