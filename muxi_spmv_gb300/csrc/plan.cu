// Plans: precomputed per-matrix state so repeated SpMVs launch only the hot
// kernels.  This is the definition of the reference's declared-but-undefined
// spmv_exec<T>(handle, format, matrix, x, y, alpha, beta)
// (src/api/spmv_api.h:57-65) in a form a C caller can hold on to.
#include "internal.h"
#include "kernels.h"
#include "plan.h"
#include "formats.h"
#include "preprocess.h"

namespace mxs {

spmv_variant_t auto_variant(spmv_type_t type, int nnz) {
    // Without a selector model (FP64: always): CSR5 tiles with gathers in nonzero order,
    // 128-thread blocks (nnz-balanced, warp-local, the fastest measured
    // variant on irregular matrices) -- 512-nonzero tiles for FP32 (256 when
    // the matrix has empty rows, plan_variant), 256 for FP64; merge-path
    // tiles when the nonzero count is beyond CSR5's range.
    if (nnz > 0x7fffffff - 32768) return spmv_variant_t{SPMV_KERNEL_MERGE, 256, 0, 8, 4};
    return spmv_variant_t{SPMV_KERNEL_CSR5, 128, 0, type == SPMV_TYPE_DOUBLE ? 8 : 16, 32};
}

spmv_status_t matrix_features(int R, int C, int N, const int* rowPtr, const int* colIdx, size_t vsize, float* dOut,
                              cudaStream_t s, long long* maxLenOut);

// Share of the sampled nonzeros within 4,096 columns of the diagonal (the
// selector's feature 24: up to 4,096 sampled rows, their first 1,024
// nonzeros each).  Synchronises the stream.
static spmv_status_t near_diagonal_share(int R, int C, int N, const int* rowPtr, const int* colIdx, cudaStream_t s,
                                         float* share) {
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(float) * SPMV_NUM_FEATURES, s));
    float f[SPMV_NUM_FEATURES] = {};
    spmv_status_t st = matrix_features(R, C, N, rowPtr, colIdx, 8, static_cast<float*>(buf), s, nullptr);
    cudaError_t e = cudaSuccess;
    if (st == SPMV_SUCCESS) e = cudaMemcpyAsync(f, buf, sizeof(f), cudaMemcpyDeviceToHost, s);
    if (st == SPMV_SUCCESS && e == cudaSuccess) e = cudaStreamSynchronize(s);
    scratch_free(buf, s);
    MXS_TRY(st);
    if (e != cudaSuccess) return cuda_fail(e, "near-diagonal share", __FILE__, __LINE__);
    *share = f[24];
    return SPMV_SUCCESS;
}

spmv_variant_t heuristic_variant(int numRows, int nnz) {
    const int avg = nnz / (numRows > 1 ? numRows : 1);
    spmv_variant_t v{};
    v.blockSize = 256;
    v.vectorWidth = 1;
    if (avg < 32) {
        v.kernel = SPMV_KERNEL_SCALAR;
        v.threadsPerRow = 1;
    } else {
        v.kernel = SPMV_KERNEL_VECTOR;
        v.threadsPerRow = 32;
    }
    return v;
}

static spmv_variant_t resolve(const spmv_variant_t* req, spmv_type_t type, int R, int N) {
    spmv_variant_t v{};
    if (req) v = *req;
    if (v.kernel == SPMV_KERNEL_HEURISTIC) return heuristic_variant(R, N);
    if (v.kernel == SPMV_KERNEL_AUTO) return auto_variant(type, N);
    if (!v.blockSize) v.blockSize = (v.kernel == SPMV_KERNEL_BAND || v.kernel == SPMV_KERNEL_STREAM) ? 512 : 256;
    if (v.kernel == SPMV_KERNEL_SCALAR) v.threadsPerRow = 1;
    if (v.kernel == SPMV_KERNEL_VECTOR && !v.threadsPerRow) v.threadsPerRow = 32;
    if (v.kernel == SPMV_KERNEL_MERGE && !v.itemsPerThread) v.itemsPerThread = v.vectorWidth == 4 ? 8 : 7;
    if (v.kernel == SPMV_KERNEL_BAND && !v.itemsPerThread) v.itemsPerThread = type == SPMV_TYPE_DOUBLE ? 8 : 16;
    if (v.kernel == SPMV_KERNEL_STREAM) {
        if (!v.itemsPerThread) v.itemsPerThread = (type == SPMV_TYPE_DOUBLE || v.blockSize == 1024) ? 8 : 16;
        if (!v.threadsPerRow) v.threadsPerRow = v.blockSize == 512 ? 3 : 2;
    }
    if (v.kernel == SPMV_KERNEL_CSR5 && !v.itemsPerThread) v.itemsPerThread = 4;  // sigma 128
    if (!v.vectorWidth && v.kernel != SPMV_KERNEL_BAND && v.kernel != SPMV_KERNEL_STREAM)
        v.vectorWidth = 1;  // BAND: 0 = largest window; STREAM: unused
    return v;
}

template <typename T>
spmv_status_t plan_exec_stream(spmv_plan_t p, T alpha, const T* x, T beta, T* y, cudaStream_t s) {
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan is NULL");
    const spmv_type_t want = sizeof(T) == 4 ? SPMV_TYPE_FLOAT : SPMV_TYPE_DOUBLE;
    if (p->type != want) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "plan value type does not match the call");
    if (p->numRows > 0 && !y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "y is NULL");
    if (p->nnz > 0 && !x) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "x is NULL");
    if (p->numRows == 0) return SPMV_SUCCESS;
    if (p->nnz == 0) return run_scale<T>(p->numRows, y, beta, s);
    RowsArgs<T> a{p->numRows, p->nnz, p->rowPtr, p->colIdx, static_cast<const T*>(p->values), x, y,
                  alpha, beta, beta == T(0)};
    a.noEmptyRows = p->noEmptyRows ? 1 : 0;
    const spmv_variant_t& v = p->variant;
    cudaEvent_t evStart = nullptr, evEnd = nullptr;
    if (p->profiling) {
        if (p->eventsUsed == p->events.size()) {
            cudaEvent_t e0, e1;
            MXS_CUDA(cudaEventCreate(&e0));
            MXS_CUDA(cudaEventCreate(&e1));
            p->events.emplace_back(e0, e1);
        }
        evStart = p->events[p->eventsUsed].first;
        evEnd = p->events[p->eventsUsed].second;
        ++p->eventsUsed;
        MXS_CUDA(cudaEventRecord(evStart, s));
    }
    switch (v.kernel) {
        case SPMV_KERNEL_SCALAR:
        case SPMV_KERNEL_VECTOR:
            MXS_TRY(run_rows<T>(v.blockSize, v.threadsPerRow, v.vectorWidth, a, s));
            if (evEnd) MXS_CUDA(cudaEventRecord(evEnd, s));
            break;
        case SPMV_KERNEL_MERGE:
            MXS_TRY(run_merge<T>(merge_geom_of(v), p->mergeTiles, p->merge, a, s, evEnd));
            break;
        case SPMV_KERNEL_BAND:
            MXS_TRY(run_band<T>(v.blockSize, v.itemsPerThread, v.threadsPerRow, v.vectorWidth, p->csr5TileRow,
                                p->csr5Tiles, p->csr5CarryRow, static_cast<T*>(p->csr5CarryVal), p->errFlag, a,
                                p->numCols, s, evEnd, &p->chains, static_cast<const unsigned*>(p->tileBits),
                                p->bandTest));
            break;
        case SPMV_KERNEL_CSR5:
            MXS_TRY(run_csr5<T>(32 * v.itemsPerThread, p->csr5TileRow, p->csr5Tiles, p->csr5CarryRow,
                                static_cast<T*>(p->csr5CarryVal), a, s, evEnd, v.vectorWidth >= 32, v.blockSize,
                                v.vectorWidth >= 32 ? v.threadsPerRow : 0, &p->chains,
                                static_cast<const unsigned*>(p->tileBits), v.vectorWidth == 64));
            break;
        case SPMV_KERNEL_STREAM:
            MXS_TRY(run_stream<T>(v.blockSize, v.itemsPerThread, v.threadsPerRow, p->csr5TileRow, p->csr5Tiles,
                                  p->csr5CarryRow, static_cast<T*>(p->csr5CarryVal), p->errFlag, a, s, evEnd,
                                  &p->chains, static_cast<const unsigned*>(p->tileBits), p->bandTest));
            break;
        case SPMV_KERNEL_ELL:
            MXS_TRY(run_ell<T>(p->numRows, p->ellWidth, p->ellCol, static_cast<const T*>(p->ellVal), x, y, alpha, beta,
                               s));
            if (evEnd) MXS_CUDA(cudaEventRecord(evEnd, s));
            break;
        default:
            MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "plan kernel %d not available", (int)v.kernel);
    }
    return SPMV_SUCCESS;
}
template spmv_status_t plan_exec_stream<float>(spmv_plan_t, float, const float*, float, float*, cudaStream_t);
template spmv_status_t plan_exec_stream<double>(spmv_plan_t, double, const double*, double, double*,
                                                cudaStream_t);

template <typename T>
static spmv_status_t plan_exec(spmv_handle_t* h, spmv_plan_t p, T alpha, const T* x, T beta, T* y) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    MXS_TRY(plan_exec_stream<T>(p, alpha, x, beta, y, h->stream));
    if (h->opts.sync) MXS_CUDA(cudaStreamSynchronize(h->stream));
    return SPMV_SUCCESS;
}

spmv_status_t plan_variant(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                           const int* colIdx, const void* values, const spmv_variant_t* variant,
                           spmv_variant_t* out) {
    *out = resolve(variant, type, R, N);
    const HandleState* hs = static_cast<const HandleState*>(h->internal);
    const bool autoPick = !variant || variant->kernel == SPMV_KERNEL_AUTO;
    if (autoPick && !(hs && hs->selector && type == SPMV_TYPE_FLOAT) && out->kernel == SPMV_KERNEL_CSR5 &&
        out->itemsPerThread == 16 && R > 0) {
        // 512-nonzero tiles pay with plan-time row-start masks, which need a
        // matrix without empty rows; otherwise the tile's row search reads
        // rowPtr slices that 512-nonzero tiles overflow: take 256.
        long long empties = 0;
        MXS_TRY(count_empty_rows(rowPtr, R, &empties, h->stream));
        if (empties > 0) out->itemsPerThread = 8;
    }
    // The model is trained on FP32 timings; FP64 AUTO plans keep the FP64
    // default (one FMA per nonzero), which beat the model's FP32 picks on
    // FP64 matrices by 15-28%, with one rule: one range of tiles per resident
    // block when every warp of those ranges gets at least 8 tiles and at
    // least half of the sampled nonzeros lie within 4,096 columns of the
    // diagonal, so an SM's L1 holds the x its neighbouring tiles gather
    // (FP64: power law +12%, mean-8 power law +29%, 2D stencil +0.4%; the
    // 27-point stencil, 33% near, lost 6.6% and small matrices a third).
    if (autoPick && type == SPMV_TYPE_DOUBLE && out->kernel == SPMV_KERNEL_CSR5 && R > 0 && N > 0) {
        const long long tiles = ((long long)N + 255) / 256;
        if (tiles >= (long long)current_sm_count() * 32 * 8) {
            float near = 0.f;
            MXS_TRY(near_diagonal_share(R, C, N, rowPtr, colIdx, h->stream, &near));
            if (near >= 0.5f)
                *out = spmv_variant_t{SPMV_KERNEL_CSR5, 1024, SPMV_RANGE_PER_RESIDENT_BLOCK, 8, SPMV_CSR5_ORDERED};
        }
    }
    const bool useModel = hs && hs->selector && type == SPMV_TYPE_FLOAT;
    if (autoPick && useModel && R > 0 && N > 0 && hs->selectorMode == SPMV_SELECT_LEARNED_FALLBACK) {
        spmv_variant_t pick{};
        MXS_TRY(spmv_select(h, SPMV_SELECT_LEARNED_FALLBACK, hs->selector, 0, type, R, C, N, rowPtr, colIdx, values,
                            &pick, nullptr));
        *out = resolve(&pick, type, R, N);
        return SPMV_SUCCESS;
    }
    if (autoPick && useModel && R > 0 && N > 0) {
        std::vector<int> order;
        MXS_TRY(learned_rank(hs->selector, type, R, C, N, rowPtr, colIdx, h->stream, order));
        std::vector<spmv_variant_t> space(spmv_variant_space(nullptr, 0));
        spmv_variant_space(space.data(), (int)space.size());
        *out = resolve(&space[order[0]], type, R, N);
    }
    return SPMV_SUCCESS;
}

}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_plan_create(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                               const int* colIdx, const void* values, const spmv_variant_t* variant,
                               spmv_plan_t* out) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan pointer is NULL");
    *out = nullptr;
    if (type != SPMV_TYPE_FLOAT && type != SPMV_TYPE_DOUBLE)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "only SPMV_TYPE_FLOAT and SPMV_TYPE_DOUBLE are supported");
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (R > 0 && !rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (N > 0 && (!colIdx || !values)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx/values is NULL");

    spmv_plan_s* p = new (std::nothrow) spmv_plan_s();
    if (!p) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    p->type = type;
    p->numRows = R;
    p->numCols = C;
    p->nnz = N;
    p->rowPtr = rowPtr;
    p->colIdx = colIdx;
    p->values = values;
    p->device = h->deviceId;
    {
        const spmv_status_t sst = plan_variant(h, type, R, C, N, rowPtr, colIdx, values, variant, &p->variant);
        if (sst != SPMV_SUCCESS) {
            delete p;
            return sst;
        }
    }
    const size_t vs = type == SPMV_TYPE_FLOAT ? 4 : 8;

    spmv_status_t st = SPMV_SUCCESS;
    const spmv_variant_t& v = p->variant;
    if (v.kernel == SPMV_KERNEL_MERGE) {
        MergeGeom g = merge_geom_of(v);
        if (g.vec && N > 0 && !(aligned16(colIdx) && aligned16(values))) {
            g = merge_unaligned_geom(g);
            p->variant = spmv_variant_t{SPMV_KERNEL_MERGE, g.block, 0, g.ipt, 1};
        }
        if (!merge_geom_supported(g)) {
            set_error(__FILE__, __LINE__, "unsupported merge shape block=%d ipt=%d", g.block, g.ipt);
            st = SPMV_ERROR_INTERNAL;
        } else if (R > 0 && N > 0) {
            p->mergeTiles = merge_tile_count(R, N, g);
            const size_t bytes = merge_scratch_bytes(p->mergeTiles, vs);
            cudaError_t e = dev_malloc(&p->mergeBuf, bytes);
            if (e != cudaSuccess) {
                set_error(__FILE__, __LINE__, "plan allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
                st = SPMV_ERROR_MEMORY_ALLOC;
            } else {
                p->workspaceBytes = bytes;
                p->merge = merge_carve(p->mergeBuf, p->mergeTiles, vs);
                st = merge_tile_coords(rowPtr, R, N, g, p->mergeTiles, p->merge.tileRow, p->merge.tileNnz,
                                       h->stream);
                if (st == SPMV_SUCCESS) {
                    e = cudaStreamSynchronize(h->stream);
                    if (e != cudaSuccess) st = cuda_fail(e, "plan build", __FILE__, __LINE__);
                }
            }
        }
    } else if (v.kernel == SPMV_KERNEL_CSR5 || v.kernel == SPMV_KERNEL_BAND || v.kernel == SPMV_KERNEL_STREAM) {
        const int sigma = 32 * v.itemsPerThread;
        if (v.kernel == SPMV_KERNEL_CSR5 && v.vectorWidth == 32 &&
            (v.threadsPerRow > 0 ? (v.blockSize != 256 && v.blockSize != 384 && v.blockSize != 512 &&
                                    v.blockSize != 640 && v.blockSize != 1024)
                                 : (v.blockSize != 128 && v.blockSize != 256 && v.blockSize != 512 &&
                                    v.blockSize != 1024))) {
            set_error(__FILE__, __LINE__,
                      "ordered CSR5 needs blockSize 128/256/512/1024 (block ranges 256/384/512/640/1024), got %d",
                      v.blockSize);
            st = SPMV_ERROR_INTERNAL;
        } else if (v.kernel == SPMV_KERNEL_BAND &&
                   (!band_shape_supported(v.blockSize, v.itemsPerThread) || v.threadsPerRow < 0 ||
                    v.vectorWidth < 0)) {
            set_error(__FILE__, __LINE__, "unsupported band shape block=%d ept=%d tiles/warp=%d window=%dK",
                      v.blockSize, v.itemsPerThread, v.threadsPerRow, v.vectorWidth);
            st = SPMV_ERROR_INTERNAL;
        } else if (v.kernel == SPMV_KERNEL_CSR5 && v.vectorWidth >= 32 && v.vectorWidth != 32 &&
                   (v.vectorWidth != 64 || v.threadsPerRow <= 0 ||
                    (v.blockSize != 512 && v.blockSize != 768 && v.blockSize != 1024))) {
            set_error(__FILE__, __LINE__,
                      "ordered CSR5 takes vectorWidth 32, or 64 (prefetching block ranges: threadsPerRow > 0, "
                      "512, 768 or 1024 threads)");
            st = SPMV_ERROR_INTERNAL;
        } else if (v.kernel == SPMV_KERNEL_STREAM &&
                   !stream_shape_supported(v.blockSize, v.itemsPerThread, v.threadsPerRow, type == SPMV_TYPE_DOUBLE)) {
            set_error(__FILE__, __LINE__, "unsupported stream shape block=%d ept=%d stages=%d", v.blockSize,
                      v.itemsPerThread, v.threadsPerRow);
            st = SPMV_ERROR_INTERNAL;
        } else if (sigma != 128 && sigma != 256 && sigma != 512) {
            set_error(__FILE__, __LINE__, "CSR5 needs itemsPerThread 4, 8 or 16 (sigma 128, 256 or 512)");
            st = SPMV_ERROR_INTERNAL;
        } else if (N > 0x7fffffff - 32768) {
            set_error(__FILE__, __LINE__, "CSR5 tiles need nnz <= 2^31 - 32769 (got %d)", N);
            st = SPMV_ERROR_INVALID_MATRIX;
        } else if (R > 0 && N > 0) {
            const long long T = ((long long)N + sigma - 1) / sigma;
            const size_t a4 = ((sizeof(int) * T) + 255) & ~size_t(255);
            const size_t av = ((vs * T) + 255) & ~size_t(255);
            const size_t bytes = 3 * a4 + av + 256;  // + the device error word
            cudaError_t e = dev_malloc(&p->csr5Buf, bytes);
            if (e != cudaSuccess) {
                set_error(__FILE__, __LINE__, "plan allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
                st = SPMV_ERROR_MEMORY_ALLOC;
            } else {
                char* b = static_cast<char*>(p->csr5Buf);
                p->csr5Tiles = T;
                p->csr5TileRow = reinterpret_cast<int*>(b);
                p->csr5TileOff = reinterpret_cast<int*>(b + a4);
                p->csr5CarryRow = reinterpret_cast<int*>(b + 2 * a4);
                p->csr5CarryVal = b + 3 * a4;
                p->errFlag = reinterpret_cast<int*>(b + 3 * a4 + av);
                p->workspaceBytes = bytes;
                e = cudaMemsetAsync(p->errFlag, 0, sizeof(int), h->stream);
                st = e == cudaSuccess ? csr5_tiles(rowPtr, R, N, sigma, p->csr5TileRow, p->csr5TileOff, h->stream)
                                      : cuda_fail(e, "plan build", __FILE__, __LINE__);
                long long empties = 1;
                if (st == SPMV_SUCCESS) st = count_empty_rows(rowPtr, R, &empties, h->stream);
                p->noEmptyRows = st == SPMV_SUCCESS && empties == 0;
                if (st == SPMV_SUCCESS)
                    st = csr5_chains(rowPtr, R, N, sigma, p->csr5TileRow, T, &p->chainBuf, &p->chains, h->stream);
                // ordered tiles (the CSR5 ordered kernels and the x-window kernel) take row-start masks
                const bool ordered = v.kernel != SPMV_KERNEL_CSR5 || v.vectorWidth >= 32;
                if (st == SPMV_SUCCESS && ordered && p->noEmptyRows)
                    st = csr5_tile_bits(rowPtr, R, sigma, T, &p->tileBits, h->stream);
                if (st == SPMV_SUCCESS) {
                    e = cudaStreamSynchronize(h->stream);
                    if (e != cudaSuccess) st = cuda_fail(e, "plan build", __FILE__, __LINE__);
                }
            }
        }
    } else if (v.kernel == SPMV_KERNEL_ELL) {
        int W = 0;
        st = max_row_length(rowPtr, R, &W, h->stream);
        // ELL stores rows*width slots; it pays only while padding stays within 2x.
        if (st == SPMV_SUCCESS && (long long)R * W > 2LL * (N > 0 ? N : 1)) {
            set_error(__FILE__, __LINE__, "ELL padding %lld slots for %d nonzeros exceeds 2x", (long long)R * W, N);
            st = SPMV_ERROR_UNSUPPORTED_FORMAT;
        }
        if (st == SPMV_SUCCESS && R > 0 && W > 0) {
            const size_t slots = (size_t)R * W;
            const size_t a4 = (sizeof(int) * slots + 255) & ~size_t(255);
            const size_t bytes = a4 + vs * slots;
            cudaError_t e = dev_malloc(&p->ellBuf, bytes);
            if (e != cudaSuccess) {
                set_error(__FILE__, __LINE__, "plan allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
                st = SPMV_ERROR_MEMORY_ALLOC;
            } else {
                p->ellWidth = W;
                p->ellCol = static_cast<int*>(p->ellBuf);
                p->ellVal = static_cast<char*>(p->ellBuf) + a4;
                p->workspaceBytes = bytes;
                long long trunc = 0;
                if (type == SPMV_TYPE_FLOAT)
                    st = csr_to_ell<float>(R, rowPtr, colIdx, static_cast<const float*>(values), W, p->ellCol,
                                           static_cast<float*>(p->ellVal), &trunc, h->stream);
                else
                    st = csr_to_ell<double>(R, rowPtr, colIdx, static_cast<const double*>(values), W, p->ellCol,
                                            static_cast<double*>(p->ellVal), &trunc, h->stream);
            }
        }
    } else if (v.kernel == SPMV_KERNEL_SCALAR || v.kernel == SPMV_KERNEL_VECTOR) {
        if (v.threadsPerRow < 1 || v.threadsPerRow > 32 || (v.threadsPerRow & (v.threadsPerRow - 1))) {
            set_error(__FILE__, __LINE__, "threadsPerRow must be a power of two in [1,32]");
            st = SPMV_ERROR_INTERNAL;
        }
    } else {
        set_error(__FILE__, __LINE__, "kernel %d is not available for plans yet", (int)v.kernel);
        st = SPMV_ERROR_UNSUPPORTED_FORMAT;
    }
    if (st != SPMV_SUCCESS) {
        if (p->mergeBuf) dev_free(p->mergeBuf);
        if (p->csr5Buf) dev_free(p->csr5Buf);
        if (p->chainBuf) dev_free(p->chainBuf);
        if (p->tileBits) dev_free(p->tileBits);
        if (p->ellBuf) dev_free(p->ellBuf);
        delete p;
        return st;
    }
    *out = p;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_device_error(spmv_plan_t p, int* code) {
    clear_error();
    if (!p || !code) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL argument");
    *code = 0;
    if (!p->errFlag) return SPMV_SUCCESS;
    int h = 0;
    MXS_CUDA(cudaMemcpy(&h, p->errFlag, sizeof(int), cudaMemcpyDeviceToHost));
    *code = h;
    if (h) {
        MXS_CUDA(cudaMemset(p->errFlag, 0, sizeof(int)));
        MXS_FAIL(SPMV_ERROR_DEVICE, "an SpMV kernel gave up a bounded wait (code %d); its output is invalid", h);
    }
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_inject_wait_timeout(spmv_plan_t p, int enable, long long limitCycles) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan is NULL");
    if (p->variant.kernel != SPMV_KERNEL_BAND && p->variant.kernel != SPMV_KERNEL_STREAM)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "only BAND and STREAM plans have bounded waits to inject into");
    if (limitCycles < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative wait limit");
    p->bandTest.inject = enable != 0;
    p->bandTest.waitLimit = enable ? (limitCycles > 0 ? limitCycles : 100000) : 0;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_profile(spmv_plan_t p, int enable) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan is NULL");
    p->profiling = enable != 0;
    p->eventsUsed = 0;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_profile_read(spmv_plan_t p, double* kernel_ms, int* launches) {
    clear_error();
    if (!p || !kernel_ms || !launches) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL argument");
    double total = 0.0;
    for (size_t i = 0; i < p->eventsUsed; ++i) {
        MXS_CUDA(cudaEventSynchronize(p->events[i].second));
        float ms = 0.f;
        MXS_CUDA(cudaEventElapsedTime(&ms, p->events[i].first, p->events[i].second));
        total += ms;
    }
    *kernel_ms = total;
    *launches = (int)p->eventsUsed;
    p->eventsUsed = 0;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_destroy(spmv_plan_t p) {
    clear_error();
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan is NULL");
    for (auto& e : p->events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    if (p->mergeBuf) dev_free(p->mergeBuf);
    if (p->csr5Buf) dev_free(p->csr5Buf);
    if (p->chainBuf) dev_free(p->chainBuf);
    if (p->tileBits) dev_free(p->tileBits);
    if (p->ellBuf) dev_free(p->ellBuf);
    if (p->ownedCsr) dev_free(p->ownedCsr);
    if (p->tPlan) spmv_plan_destroy(p->tPlan);
    if (p->tBuf) dev_free(p->tBuf);
    delete p;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_create_ex(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                                  const int* colIdx, const void* values, const spmv_variant_t* variant, int flags,
                                  spmv_plan_t* out) {
    clear_error();
    if (!(flags & SPMV_PLAN_COPY)) return spmv_plan_create(h, type, R, C, N, rowPtr, colIdx, values, variant, out);
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan pointer is NULL");
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    if (type != SPMV_TYPE_FLOAT && type != SPMV_TYPE_DOUBLE)
        MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "only SPMV_TYPE_FLOAT and SPMV_TYPE_DOUBLE are supported");
    if (R > 0 && !rowPtr) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "rowPtr is NULL");
    if (N > 0 && (!colIdx || !values)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "colIdx/values is NULL");
    // One allocation: rowPtr, colIdx and values, each 256-byte aligned.
    const size_t vs = type == SPMV_TYPE_FLOAT ? 4 : 8;
    const size_t a0 = (sizeof(int) * ((size_t)R + 1) + 255) & ~size_t(255);
    const size_t a1 = (sizeof(int) * (size_t)N + 255) & ~size_t(255);
    char* buf = nullptr;
    MXS_CUDA(dev_malloc(&buf, a0 + a1 + vs * (size_t)N + 256));
    int* rp = reinterpret_cast<int*>(buf);
    int* ci = reinterpret_cast<int*>(buf + a0);
    void* va = buf + a0 + a1;
    cudaError_t e = R > 0 ? cudaMemcpyAsync(rp, rowPtr, sizeof(int) * ((size_t)R + 1), cudaMemcpyDeviceToDevice,
                                            h->stream)
                          : cudaSuccess;
    if (e == cudaSuccess && N > 0)
        e = cudaMemcpyAsync(ci, colIdx, sizeof(int) * (size_t)N, cudaMemcpyDeviceToDevice, h->stream);
    if (e == cudaSuccess && N > 0) e = cudaMemcpyAsync(va, values, vs * (size_t)N, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) {
        dev_free(buf);
        return cuda_fail(e, "plan matrix copy", __FILE__, __LINE__);
    }
    const spmv_status_t st = spmv_plan_create(h, type, R, C, N, R > 0 ? rp : nullptr, N > 0 ? ci : nullptr,
                                              N > 0 ? va : nullptr, variant, out);
    if (st != SPMV_SUCCESS) {
        dev_free(buf);
        return st;
    }
    e = cudaStreamSynchronize(h->stream);  // the caller may free its arrays on return
    (*out)->ownedCsr = buf;
    if (e != cudaSuccess) return cuda_fail(e, "plan matrix copy", __FILE__, __LINE__);
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_get_variant(spmv_plan_t p, spmv_variant_t* v) {
    clear_error();
    if (!p || !v) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL argument");
    *v = p->variant;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_get_workspace_bytes(spmv_plan_t p, size_t* bytes) {
    clear_error();
    if (!p || !bytes) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "NULL argument");
    *bytes = p->workspaceBytes;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_plan_exec_f32(spmv_handle_t* h, spmv_plan_t p, float alpha, const float* x, float beta,
                                 float* y) {
    return plan_exec<float>(h, p, alpha, x, beta, y);
}

}  // extern "C"

namespace mxs {
// op = SPMV_OP_TRANSPOSE: y = alpha*A^T*x + beta*y through a plan of A^T
// built (csr_transpose, AUTO variant) on the first such call and kept.
template <typename T>
static spmv_status_t plan_exec_op(spmv_handle_t* h, spmv_plan_t p, spmv_operation_t op, T alpha, const T* x, T beta,
                                  T* y) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "plan is NULL");
    if (op == SPMV_OP_NORMAL) return plan_exec<T>(h, p, alpha, x, beta, y);
    if (op != SPMV_OP_TRANSPOSE) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT, "SPMV_OP_CONJUGATE is not supported");
    const spmv_type_t want = sizeof(T) == 4 ? SPMV_TYPE_FLOAT : SPMV_TYPE_DOUBLE;
    if (p->type != want) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "plan value type does not match the call");
    if (!p->tPlan) {
        const int R = p->numRows, C = p->numCols, N = p->nnz;
        const size_t a = (sizeof(int) * ((size_t)C + 1) + 255) & ~size_t(255);
        const size_t b = (sizeof(int) * (size_t)(N > 0 ? N : 1) + 255) & ~size_t(255);
        char* buf = nullptr;
        MXS_CUDA(dev_malloc(&buf, a + b + sizeof(T) * (size_t)(N > 0 ? N : 1)));
        int* tRp = reinterpret_cast<int*>(buf);
        int* tCi = reinterpret_cast<int*>(buf + a);
        T* tVa = reinterpret_cast<T*>(buf + a + b);
        spmv_status_t st = csr_transpose<T>(R, C, N, p->rowPtr, p->colIdx, static_cast<const T*>(p->values), tRp,
                                            tCi, tVa, h->stream);
        spmv_plan_t q = nullptr;
        if (st == SPMV_SUCCESS)
            st = spmv_plan_create(h, p->type, C, R, N, C > 0 ? tRp : nullptr, N > 0 ? tCi : nullptr,
                                  N > 0 ? static_cast<const void*>(tVa) : nullptr, nullptr, &q);
        if (st != SPMV_SUCCESS) {
            dev_free(buf);
            return st;
        }
        p->tPlan = q;
        p->tBuf = buf;
    }
    return plan_exec<T>(h, p->tPlan, alpha, x, beta, y);
}
}  // namespace mxs

extern "C" {

spmv_status_t spmv_convert(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                           const int* colIdx, const void* values, spmv_format_t format,
                           const spmv_variant_t* params, spmv_plan_t* out) {
    clear_error();
    if (out) *out = nullptr;
    spmv_variant_t v{};
    switch (format) {
        case SPMV_FORMAT_CSR:  // any CSR kernel; NULL: AUTO
            if (params) v = *params;
            else v.kernel = SPMV_KERNEL_AUTO;
            break;
        case SPMV_FORMAT_CSR5:  // CSR5 tiles; NULL: the default tile shape
            if (params) {
                v = *params;
                v.kernel = SPMV_KERNEL_CSR5;
            } else {
                v = resolve(nullptr, type, R, N);
                if (v.kernel != SPMV_KERNEL_CSR5) {
                    v = spmv_variant_t{};
                    v.kernel = SPMV_KERNEL_CSR5;
                    v.blockSize = 128;
                    v.itemsPerThread = 8;
                    v.vectorWidth = 32;
                }
                if (h && v.itemsPerThread == 16 && R > 0 && rowPtr) {  // as AUTO: 256-nonzero tiles with empty rows
                    long long empties = 0;
                    MXS_TRY(count_empty_rows(rowPtr, R, &empties, h->stream));
                    if (empties > 0) v.itemsPerThread = 8;
                }
            }
            break;
        case SPMV_FORMAT_ELL:  // column-major ELLPACK; refused beyond 2x padding
            v.kernel = SPMV_KERNEL_ELL;
            break;
        default:
            MXS_FAIL(SPMV_ERROR_UNSUPPORTED_FORMAT,
                     "spmv_convert builds CSR, CSR5 or ELL plans (COO: spmv_coo_to_csr_*; BSR: spmv_csr_to_bsr_*)");
    }
    return spmv_plan_create(h, type, R, C, N, rowPtr, colIdx, values, &v, out);
}

spmv_status_t spmv_exec_f32(spmv_handle_t* h, spmv_plan_t p, spmv_operation_t op, float alpha, const float* x,
                            float beta, float* y) {
    return plan_exec_op<float>(h, p, op, alpha, x, beta, y);
}
spmv_status_t spmv_exec_f64(spmv_handle_t* h, spmv_plan_t p, spmv_operation_t op, double alpha, const double* x,
                            double beta, double* y) {
    return plan_exec_op<double>(h, p, op, alpha, x, beta, y);
}

spmv_status_t spmv_plan_exec_op_f32(spmv_handle_t* h, spmv_plan_t p, spmv_operation_t op, float alpha,
                                    const float* x, float beta, float* y) {
    return plan_exec_op<float>(h, p, op, alpha, x, beta, y);
}
spmv_status_t spmv_plan_exec_op_f64(spmv_handle_t* h, spmv_plan_t p, spmv_operation_t op, double alpha,
                                    const double* x, double beta, double* y) {
    return plan_exec_op<double>(h, p, op, alpha, x, beta, y);
}
spmv_status_t spmv_plan_exec_f64(spmv_handle_t* h, spmv_plan_t p, double alpha, const double* x, double beta,
                                 double* y) {
    return plan_exec<double>(h, p, alpha, x, beta, y);
}

}  // extern "C"
