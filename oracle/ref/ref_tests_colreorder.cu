// Builds the reference's tests/test_column_reordering.cu where it lies (its
// main() renamed) and exposes the two column reorders it defines,
// reorderColumnsRCM (:156-199) and reorderColumnsByFrequency (:116-154), to
// ctypes.  Only the host functions are called.  Output goes to oracle/_ref/.
// The standard headers the reference file uses are included first (it uses
// std::tuple without including <tuple>), so that its own includes are no-ops
// inside the namespace that keeps its global names apart from the other
// reference test file built into the same library.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>
#include <cuda_runtime.h>
#define main muxi_ref_unused_main_colreorder
namespace ref_colreorder {
#include "tests/test_column_reordering.cu"
}  // namespace ref_colreorder
#undef main

using namespace ref_colreorder;

namespace {
template <typename Fn>
void run_reorder(Fn fn, int rows, int cols, int nnz, const int* rp, const int* ci, int* perm, int* newCol) {
    CSRMatrix m{};
    m.numRows = rows;
    m.numCols = cols;
    m.nnz = nnz;
    m.rowPtr = const_cast<int*>(rp);
    m.colIdx = const_cast<int*>(ci);
    std::vector<float> vals(nnz > 0 ? nnz : 1, 0.0f);
    m.values = vals.data();
    CSRMatrix out{};
    std::vector<int> p;
    fn(m, out, p);
    for (int i = 0; i < cols; ++i) perm[i] = p[i];
    if (newCol)
        for (int j = 0; j < nnz; ++j) newCol[j] = out.colIdx[j];
    delete[] out.rowPtr;
    delete[] out.colIdx;
    delete[] out.values;
}
}  // namespace

extern "C" void ref_rcm_perm(int rows, int cols, int nnz, const int* rp, const int* ci, int* perm, int* newCol) {
    run_reorder(reorderColumnsRCM, rows, cols, nnz, rp, ci, perm, newCol);
}

extern "C" void ref_frequency_perm(int rows, int cols, int nnz, const int* rp, const int* ci, int* perm,
                                   int* newCol) {
    run_reorder(reorderColumnsByFrequency, rows, cols, nnz, rp, ci, perm, newCol);
}
