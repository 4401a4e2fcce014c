// Plan object: a borrowed CSR matrix plus what one kernel variant needs.
#pragma once

#include <utility>
#include <vector>

#include "internal.h"
#include "kernels.h"
#include "formats.h"

struct spmv_plan_s {
    spmv_type_t type = SPMV_TYPE_FLOAT;
    int numRows = 0, numCols = 0, nnz = 0;
    const int* rowPtr = nullptr;
    const int* colIdx = nullptr;
    const void* values = nullptr;
    spmv_variant_t variant{};
    int device = 0;
    // merge path
    long long mergeTiles = 0;
    void* mergeBuf = nullptr;  // tile coordinates + carries (cudaMalloc)
    mxs::MergeScratch merge{};
    // CSR5: sigma = 32 * itemsPerThread; tile rows / offsets / carries
    long long csr5Tiles = 0;
    void* csr5Buf = nullptr;
    int* csr5TileRow = nullptr;
    int* csr5TileOff = nullptr;
    int* csr5CarryRow = nullptr;
    void* csr5CarryVal = nullptr;
    int* errFlag = nullptr;  // device word raised by a kernel whose bounded wait gave up
    mxs::BandTest bandTest{};  // BAND plans: fault injection into the window wait (tests)
    bool noEmptyRows = false;  // checked at plan creation (CSR5 kernels skip the empty-row pass)
    void* chainBuf = nullptr;  // CSR5 carry chains (start / end / row), see Csr5Chains
    void* tileBits = nullptr;  // ordered CSR5 on a matrix without empty rows: row-start masks
    mxs::Csr5Chains chains{};
    // ELL: column-major copy of the matrix
    int ellWidth = 0;
    void* ellBuf = nullptr;
    int* ellCol = nullptr;
    void* ellVal = nullptr;
    size_t workspaceBytes = 0;
    void* ownedCsr = nullptr;  // SPMV_PLAN_COPY: the plan's own copy of rowPtr / colIdx / values
    // SPMV_OP_TRANSPOSE executions: A^T built on first use, with its own plan
    spmv_plan_s* tPlan = nullptr;
    void* tBuf = nullptr;
    // main-kernel timing (spmv_plan_profile)
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;
    size_t eventsUsed = 0;
};

namespace mxs {
// The reference's NVIDIA dispatch rule (spmv_csr.cu:115-153): integer
// avgNnz = nnz / rows; scalar kernel below 32, one warp per row from 32 up.
spmv_variant_t heuristic_variant(int numRows, int nnz);
// The AUTO plan's variant without a selector model (plan.cu).
spmv_variant_t auto_variant(spmv_type_t type, int nnz);
// Learned selector: indices into the variant space of the variants that
// apply to this matrix, best predicted first (select.cu).
spmv_status_t learned_rank(spmv_mlp_t model, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                           const int* colIdx, cudaStream_t s, std::vector<int>& order,
                           std::vector<float>* predOut = nullptr);
// The variant a plan on this matrix runs: AUTO / HEURISTIC resolved, the
// learned pick when the handle has a selector model (plan.cu).
spmv_status_t plan_variant(spmv_handle_t* h, spmv_type_t type, int R, int C, int N, const int* rowPtr,
                           const int* colIdx, const void* values, const spmv_variant_t* variant,
                           spmv_variant_t* out);
// One SpMV of a plan on stream s (no handle; spmv_plan_exec_* without opts.sync).
template <typename T>
spmv_status_t plan_exec_stream(spmv_plan_t p, T alpha, const T* x, T beta, T* y, cudaStream_t s);
}  // namespace mxs
