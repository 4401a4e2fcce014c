// Builds the reference's tests/test_row_reordering.cu where it lies (main()
// renamed) and exposes reorderMatrixByRowLength (:99-143).
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
#define main muxi_ref_unused_main_rowreorder
namespace ref_rowreorder {
#include "tests/test_row_reordering.cu"
}  // namespace ref_rowreorder
#undef main
using namespace ref_rowreorder;

extern "C" void ref_row_reorder(int rows, int cols, int nnz, const int* rp, const int* ci, const float* v,
                                int* rowMap, int* newRowPtr, int* newCol, float* newVal) {
    CSRMatrix m{};
    m.numRows = rows;
    m.numCols = cols;
    m.nnz = nnz;
    m.rowPtr = const_cast<int*>(rp);
    m.colIdx = const_cast<int*>(ci);
    m.values = const_cast<float*>(v);
    CSRMatrix out{};
    std::vector<int> map, inv;
    reorderMatrixByRowLength(m, out, map, inv);
    for (int i = 0; i < rows; ++i) rowMap[i] = map[i];
    for (int i = 0; i <= rows; ++i) newRowPtr[i] = out.rowPtr[i];
    for (int j = 0; j < nnz; ++j) {
        newCol[j] = out.colIdx[j];
        newVal[j] = out.values[j];
    }
    delete[] out.rowPtr;
    delete[] out.colIdx;
    delete[] out.values;
}
