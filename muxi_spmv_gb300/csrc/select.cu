// Kernel selection: the reference's fixed rule, the exhaustive autotuner,
// and the learned selector (features -> MLP -> smallest predicted slowdown).
// The reference's only selection is the integer mean-row-length rule of
// src/spmv/csr/spmv_csr.cu:115-153 (kept as SPMV_SELECT_HEURISTIC).
#include <algorithm>
#include <numeric>
#include <vector>

#include "internal.h"
#include "kernels.h"
#include "plan.h"

namespace mxs {

int variant_space(spmv_variant_t* out, int cap);
spmv_status_t matrix_features(int R, int C, int N, const int* rowPtr, const int* colIdx, size_t vsize, float* dOut,
                              cudaStream_t s, long long* maxLenOut);
spmv_status_t mlp_predict_one(spmv_mlp_t n, const float* dX, float* hY, cudaStream_t s);
int mlp_outputs(spmv_mlp_t n);
int mlp_inputs(spmv_mlp_t n);

// Mirrors the refusals of spmv_plan_create for a matrix with the given
// nonzero count and longest row.
static bool variant_applicable(const spmv_variant_t& v, int R, int N, long long maxLen) {
    switch (v.kernel) {
        case SPMV_KERNEL_SCALAR:
        case SPMV_KERNEL_VECTOR:
            return true;
        case SPMV_KERNEL_MERGE:
            return merge_geom_supported(merge_geom_of(v));
        case SPMV_KERNEL_CSR5:
        case SPMV_KERNEL_BAND:
        case SPMV_KERNEL_STREAM: {
            const int sigma = 32 * v.itemsPerThread;
            if (sigma != 128 && sigma != 256 && sigma != 512) return false;
            if (N > 0x7fffffff - 32768) return false;
            if (v.kernel == SPMV_KERNEL_STREAM)  // the selector's space is FP32
                return stream_shape_supported(v.blockSize, v.itemsPerThread, v.threadsPerRow, false);
            return v.kernel != SPMV_KERNEL_BAND || band_shape_supported(v.blockSize, v.itemsPerThread);
        }
        case SPMV_KERNEL_ELL:
            return (long long)R * maxLen <= 2LL * (N > 0 ? N : 1);
        default:
            return false;
    }
}

// Predicted log-time gap under which the learned pick counts as uncertain
// (SPMV_SELECT_LEARNED_FALLBACK): 0.12, about 12%; at most kFallbackMax
// candidates (the pick included) are timed unless topK says otherwise.
constexpr float kFallbackMargin = 0.12f;
constexpr int kFallbackMax = 4;

static bool same_variant(const spmv_variant_t& a, const spmv_variant_t& b) {
    return a.kernel == b.kernel && a.blockSize == b.blockSize && a.threadsPerRow == b.threadsPerRow &&
           a.itemsPerThread == b.itemsPerThread && a.vectorWidth == b.vectorWidth;
}

// Space indices of the applicable variants, best predicted first; `predOut`
// (optional) receives the model's output per space index (predicted log of
// the time over the best variant's).
spmv_status_t learned_rank(spmv_mlp_t model, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                           const int* colIdx, cudaStream_t s, std::vector<int>& order,
                           std::vector<float>* predOut) {
    std::vector<spmv_variant_t> space(variant_space(nullptr, 0));
    variant_space(space.data(), (int)space.size());
    if (mlp_inputs(model) != SPMV_NUM_FEATURES || mlp_outputs(model) != (int)space.size())
        MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "selector model shape %d->%d does not match %d features -> %d variants",
                 mlp_inputs(model), mlp_outputs(model), SPMV_NUM_FEATURES, (int)space.size());
    void* buf = nullptr;
    MXS_TRY(scratch_alloc(&buf, sizeof(float) * SPMV_NUM_FEATURES, s));
    float* dF = static_cast<float*>(buf);
    long long maxLen = 0;
    std::vector<float> pred(space.size());
    spmv_status_t st =
        matrix_features(R, C, N, rowPtr, colIdx, type == SPMV_TYPE_FLOAT ? 4 : 8, dF, s, &maxLen);
    if (st == SPMV_SUCCESS) st = mlp_predict_one(model, dF, pred.data(), s);
    scratch_free(buf, s);
    MXS_TRY(st);
    order.clear();
    for (int i = 0; i < (int)space.size(); ++i)
        if (variant_applicable(space[i], R, N, maxLen)) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pred[a] < pred[b]; });
    if (order.empty()) MXS_FAIL(SPMV_ERROR_INTERNAL, "no applicable variant");
    if (predOut) *predOut = pred;
    return SPMV_SUCCESS;
}

}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_select(spmv_handle_t* h, spmv_select_mode_t mode, spmv_mlp_t model, int topK, spmv_type_t type,
                          int R, int C, int N, const int* rowPtr, const int* colIdx, const void* values,
                          spmv_variant_t* out, int* spaceIndex) {
    clear_error();
    if (!h) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (!out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "out is NULL");
    if (type != SPMV_TYPE_FLOAT && type != SPMV_TYPE_DOUBLE) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "float or double");
    if (R < 0 || C < 0 || N < 0) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "negative dimension");
    std::vector<spmv_variant_t> space(variant_space(nullptr, 0));
    variant_space(space.data(), (int)space.size());
    int idx = -1;
    switch (mode) {
        case SPMV_SELECT_HEURISTIC: {
            *out = heuristic_variant(R, N);
            for (int i = 0; i < (int)space.size(); ++i)
                if (same_variant(space[i], *out)) idx = i;
            break;
        }
        case SPMV_SELECT_AUTOTUNE: {
            std::vector<float> ms(space.size());
            MXS_TRY(spmv_autotune(h, type, R, C, N, rowPtr, colIdx, values, space.data(), (int)space.size(), 5,
                                  ms.data(), &idx));
            *out = space[idx];
            break;
        }
        case SPMV_SELECT_LEARNED:
        case SPMV_SELECT_LEARNED_TOPK:
        case SPMV_SELECT_LEARNED_FALLBACK: {
            if (!model) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "learned selection needs a model");
            std::vector<int> order;
            std::vector<float> pred;
            MXS_TRY(learned_rank(model, type, R, C, N, rowPtr, colIdx, h->stream, order, &pred));
            idx = order[0];
            int k = 1;
            if (mode == SPMV_SELECT_LEARNED_TOPK && topK > 1) k = std::min<int>(topK, (int)order.size());
            if (mode == SPMV_SELECT_LEARNED_FALLBACK) {
                // Low confidence: other variants predicted within kFallbackMargin
                // of the best are timed too (at most topK, default kFallbackMax).
                const int kmax = std::min<int>(topK > 1 ? topK : kFallbackMax, (int)order.size());
                while (k < kmax && pred[order[k]] - pred[order[0]] <= kFallbackMargin) ++k;
            }
            if (k > 1) {
                std::vector<spmv_variant_t> cand(k);
                for (int i = 0; i < k; ++i) cand[i] = space[order[i]];
                std::vector<float> ms(k);
                int best = -1;
                MXS_TRY(spmv_autotune(h, type, R, C, N, rowPtr, colIdx, values, cand.data(), k, 5, ms.data(), &best));
                idx = order[best];
            }
            *out = space[idx];
            break;
        }
        default:
            MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "unknown selection mode %d", (int)mode);
    }
    if (spaceIndex) *spaceIndex = idx;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_set_selector_mode(spmv_handle_t* h, spmv_select_mode_t mode) {
    clear_error();
    if (!h || !h->internal) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (mode != SPMV_SELECT_LEARNED && mode != SPMV_SELECT_LEARNED_FALLBACK)
        MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "AUTO plans take SPMV_SELECT_LEARNED or SPMV_SELECT_LEARNED_FALLBACK");
    static_cast<HandleState*>(h->internal)->selectorMode = mode;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_set_selector(spmv_handle_t* h, spmv_mlp_t model) {
    clear_error();
    if (!h || !h->internal) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "handle is NULL");
    if (model && (mlp_inputs(model) != SPMV_NUM_FEATURES || mlp_outputs(model) != variant_space(nullptr, 0)))
        MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "model shape does not match the feature and variant spaces");
    static_cast<HandleState*>(h->internal)->selector = model;
    return SPMV_SUCCESS;
}

}  // extern "C"
