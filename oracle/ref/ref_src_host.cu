// Builds host-side reference library code where it lies and exposes it to
// ctypes:
//   src/preprocessing/column_reorder.cuh  reorderColumns (:42-141),
//                                         sortColumnsWithinRows (:175-201)
//   src/spmv/ellpack/spmv_ellpack.cu      csr_to_ellpack (:11-70)
//   src/generators/mtx_io.cu              readMTXFile (:111-222)
// csr_to_ellpack finishes with cudaMalloc/cudaMemcpy into device arrays; the
// recipe links this unit against ref_host_cudart.cpp, whose cudaMalloc and
// cudaMemcpy work on host memory, so the converted arrays can be read back
// on a machine without a GPU.
#include <vector>
#include "preprocessing/column_reorder.cuh"
#include "spmv/ellpack/spmv_ellpack.cu"
#include "generators/mtx_io.cu"

using namespace muxi_spmv;

extern "C" void ref_center_of_mass_perm(int rows, int cols, int nnz, const int* rp, const int* ci, int* forwardMap,
                                        int* newCol) {
    CSRMatrix<float> m;
    m.numRows = rows;
    m.numCols = cols;
    m.nnz = nnz;
    m.rowPtr = const_cast<int*>(rp);
    m.colIdx = const_cast<int*>(ci);
    std::vector<float> vals(nnz > 0 ? nnz : 1, 0.0f);
    m.values = vals.data();
    CSRMatrix<float> out;
    std::vector<int> fm;
    ColumnReorderStats stats{};
    reorderColumns(m, out, fm, stats);
    for (int i = 0; i < cols; ++i) forwardMap[i] = fm[i];
    for (int j = 0; j < nnz; ++j) newCol[j] = out.colIdx[j];
    m.rowPtr = nullptr;  // borrowed; the destructor frees only owned memory
}

extern "C" void ref_sort_within_rows(int rows, int cols, int nnz, const int* rp, int* ci, float* v) {
    CSRMatrix<float> m;
    m.numRows = rows;
    m.numCols = cols;
    m.nnz = nnz;
    m.rowPtr = const_cast<int*>(rp);
    m.colIdx = ci;
    m.values = v;
    sortColumnsWithinRows(m);
}

extern "C" int ref_csr_to_ell(int rows, int cols, int nnz, const int* rp, const int* ci, const float* v,
                              int maxElements, int* ellCol, float* ellVal) {
    CSRMatrix<float> m;
    m.numRows = rows;
    m.numCols = cols;
    m.nnz = nnz;
    m.rowPtr = const_cast<int*>(rp);
    m.colIdx = const_cast<int*>(ci);
    m.values = const_cast<float*>(v);
    ELLPACKMatrix<float> e;
    csr_to_ellpack(m, e, maxElements);
    const long long total = (long long)rows * e.numElements;
    for (long long i = 0; i < total; ++i) {
        ellCol[i] = e.d_colIdx[i];
        ellVal[i] = e.d_values[i];
    }
    free(e.d_colIdx);
    free(e.d_values);
    return e.numElements;
}

// readMTXFile into a reference CSRMatrix; with out arrays NULL only the sizes
// are returned (rows, cols, nnz), else the CSR is copied out.  Returns the
// reference's status.
extern "C" int ref_mtx_read_f64(const char* path, int expand, int* dims, int* rp, int* ci, double* v) {
    CSRMatrix<double> m;
    const int st = (int)io::readMTXFile<double>(path, m, expand != 0);
    if (st != 0) return st;
    dims[0] = m.numRows;
    dims[1] = m.numCols;
    dims[2] = m.nnz;
    if (rp) {
        for (int r = 0; r <= m.numRows; ++r) rp[r] = m.rowPtr[r];
        for (int j = 0; j < m.nnz; ++j) {
            ci[j] = m.colIdx[j];
            v[j] = m.values[j];
        }
    }
    return 0;
}
