// Drop-in check: reference-style call sites (tests/correctness/test_spmv.cu,
// tests/benchmark/test_runner.cu:265-329, src/benchmark/performance_benchmark.cu:
// 383-422, tests/benchmark/test_ellpack.cu:46-115, tests/test_sparse_optimized.cu:80)
// compiled unchanged against
// include/muxi_spmv.hpp and linked to libmuxispmv.so.  Prints PASSED/FAILED
// per check and exits non-zero on any failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <unistd.h>
#include <vector>

#include "muxi_spmv.hpp"

using namespace muxi_spmv;

static int failures = 0;

static void report(const char* what, bool ok) {
    std::printf("%-40s %s\n", what, ok ? "PASSED" : "FAILED");
    if (!ok) ++failures;
}

// Diagonal matrix, as tests/correctness/test_spmv.cu:15-30 builds it.
static void generateDiagonalMatrix(int n, CSRMatrix<float>& matrix) {
    matrix.allocateHost(n, n, n);
    for (int i = 0; i <= n; i++) matrix.rowPtr[i] = i;
    for (int i = 0; i < n; i++) {
        matrix.colIdx[i] = i;
        matrix.values[i] = 1.0f;
    }
}

// A ragged matrix with empty rows and one long row (host arrays).
static void generateRagged(int n, CSRMatrix<float>& m) {
    std::vector<int> lens(n);
    for (int r = 0; r < n; ++r) lens[r] = (r % 7 == 3) ? 0 : 1 + (r * 37 % 11);
    lens[n / 2] = 3000;
    int nnz = 0;
    for (int r = 0; r < n; ++r) nnz += lens[r];
    m.allocateHost(n, n, nnz);
    m.rowPtr[0] = 0;
    for (int r = 0; r < n; ++r) m.rowPtr[r + 1] = m.rowPtr[r] + lens[r];
    for (int r = 0; r < n; ++r)
        for (int j = m.rowPtr[r]; j < m.rowPtr[r + 1]; ++j) {
            m.colIdx[j] = (int)((r * 131 + (j - m.rowPtr[r]) * 17) % n);
            m.values[j] = (float)((j % 13) - 6) / 7.0f;
        }
}

static bool close(const std::vector<float>& a, const std::vector<double>& b, const std::vector<double>& s) {
    for (size_t i = 0; i < a.size(); ++i)
        if (std::fabs(a[i] - b[i]) > 1e-5 * s[i] + 1e-30) {
            std::printf("  row %zu: got %g want %g\n", i, a[i], b[i]);
            return false;
        }
    return true;
}

int main() {
    // --- test_spmv.cu: diagonal KAT ---
    const int n = 1024;
    CSRMatrix<float> matrix;
    generateDiagonalMatrix(n, matrix);
    std::vector<float> h_x(n), h_y(n);
    for (int i = 0; i < n; i++) h_x[i] = (float)(i + 1);
    matrix.allocateDevice();
    matrix.copyToDevice();
    float *d_x, *d_y;
    cudaMalloc(&d_x, n * sizeof(float));
    cudaMalloc(&d_y, n * sizeof(float));
    cudaMemcpy(d_x, h_x.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    spmv_handle_t* handle;
    report("spmv_create_handle", spmv_create_handle(&handle) == SPMV_SUCCESS && handle->warpSize == 32);
    spmv_opts_t opts = spmv_default_opts();
    opts.sync = 1;
    spmv_status_t status = spmv_csr<float>(matrix, d_x, d_y, 1.0f, 0.0f, opts);
    cudaMemcpy(h_y.data(), d_y, n * sizeof(float), cudaMemcpyDeviceToHost);
    bool ok = status == SPMV_SUCCESS;
    for (int i = 0; i < n && ok; i++) ok = std::fabs(h_y[i] - h_x[i]) <= 1e-5f;
    report("spmv_csr diagonal KAT", ok);
    status = spmv_csr_exec<float>(matrix, d_x, d_y);
    report("spmv_csr_exec defaults", status == SPMV_SUCCESS);

    // --- ragged matrix through every format ---
    const int m = 5000;
    CSRMatrix<float> A;
    generateRagged(m, A);
    A.allocateDevice();
    A.copyToDevice();
    std::vector<float> x(m);
    for (int i = 0; i < m; ++i) x[i] = (float)((i % 100) + 1) / 100.0f;  // test_runner.cu x
    std::vector<double> want(m), scale(m);
    for (int r = 0; r < m; ++r) {
        double s = 0, a = 0;
        for (int j = A.rowPtr[r]; j < A.rowPtr[r + 1]; ++j) {
            s += (double)A.values[j] * x[A.colIdx[j]];
            a += std::fabs((double)A.values[j] * x[A.colIdx[j]]);
        }
        want[r] = s;
        scale[r] = a;
    }
    float *dx, *dy;
    cudaMalloc(&dx, m * sizeof(float));
    cudaMalloc(&dy, m * sizeof(float));
    cudaMemcpy(dx, x.data(), m * sizeof(float), cudaMemcpyHostToDevice);
    std::vector<float> y(m);
    auto fetch = [&]() {
        cudaDeviceSynchronize();
        cudaMemcpy(y.data(), dy, m * sizeof(float), cudaMemcpyDeviceToHost);
    };

    status = spmv_merge_based<float>(A, dx, dy, 0);
    fetch();
    report("spmv_merge_based", status == SPMV_SUCCESS && close(y, want, scale));

    status = spmv_sparse_optimized<float>(A, dx, dy, 0);  // tests/test_sparse_optimized.cu:80
    fetch();
    report("spmv_sparse_optimized", status == SPMV_SUCCESS && close(y, want, scale));

    CSR5Matrix<float> csr5;
    status = csr5_preprocess<float>(A, csr5, 0, 0);
    bool tiles_ok = status == SPMV_SUCCESS && csr5.sigma == 128 && csr5.numTiles == (A.nnz + 127) / 128;
    for (int t = 0; t < csr5.numTiles && tiles_ok; ++t) {
        const int start = t * csr5.sigma, r = csr5.tile_row_ptr[t];
        tiles_ok = A.rowPtr[r] <= start && (r + 1 >= m || A.rowPtr[r + 1] > start) &&
                   csr5.tile_nnz_offset[t] == start - A.rowPtr[r];
    }
    report("csr5_preprocess tile metadata", tiles_ok);
    status = spmv_csr5<float>(csr5, dx, dy, 1.0f, 0.0f, opts);
    fetch();
    report("spmv_csr5", status == SPMV_SUCCESS && close(y, want, scale));

    ELLPACKMatrix<float> ell;
    status = csr_to_ellpack<float>(A, ell);
    report("csr_to_ellpack width", status == SPMV_SUCCESS && ell.numElements == 3000 && ell.truncatedRows == 0);
    status = spmv_ellpack<float>(ell, dx, dy, 0);
    fetch();
    report("spmv_ellpack", status == SPMV_SUCCESS && close(y, want, scale));
    cudaFree(ell.d_colIdx);
    cudaFree(ell.d_values);

    cudaStream_t st;
    cudaStreamCreate(&st);
    spmv_set_stream(handle, st);
    report("spmv_set_stream stores the stream", handle->stream == st && handle->opts.stream == (void*)st);
    cudaMemset(dy, 0, m * sizeof(float));
    status = spmv_exec<float>(handle, SPMV_FORMAT_CSR, &A, dx, dy, 2.0f, 0.0f);
    cudaStreamSynchronize(st);
    cudaMemcpy(y.data(), dy, m * sizeof(float), cudaMemcpyDeviceToHost);
    for (auto& v : y) v *= 0.5f;
    report("spmv_exec CSR alpha=2", status == SPMV_SUCCESS && close(y, want, scale));
    status = spmv_exec<float>(handle, SPMV_FORMAT_CSR5, &csr5, dx, dy);
    cudaStreamSynchronize(st);
    cudaMemcpy(y.data(), dy, m * sizeof(float), cudaMemcpyDeviceToHost);
    report("spmv_exec CSR5", status == SPMV_SUCCESS && close(y, want, scale));
    // COO (sparse_formats.h:113-162), entries in reverse order: converted on the device.
    {
        COOMatrix<float> coo;
        coo.allocateHost(m, m, A.nnz);
        int k = 0;
        for (int r = m - 1; r >= 0; --r)
            for (int j = A.rowPtr[r + 1] - 1; j >= A.rowPtr[r]; --j, ++k) {
                coo.rowIdx[k] = r;
                coo.colIdx[k] = A.colIdx[j];
                coo.values[k] = A.values[j];
            }
        coo.allocateDevice();
        coo.copyToDevice(st);
        cudaMemset(dy, 0, m * sizeof(float));
        status = spmv_exec<float>(handle, SPMV_FORMAT_COO, &coo, dx, dy);
        cudaStreamSynchronize(st);
        cudaMemcpy(y.data(), dy, m * sizeof(float), cudaMemcpyDeviceToHost);
        report("spmv_exec COO", status == SPMV_SUCCESS && close(y, want, scale));
    }
    // BSR (sparse_formats.h:207-269) from the column-sorted copy B below
    report("spmv_exec CSR2 unsupported",
           spmv_exec<float>(handle, SPMV_FORMAT_CSR2, &A, dx, dy) == SPMV_ERROR_UNSUPPORTED_FORMAT);

    // spmv_exec_transpose (spmv_api.h:70-78): y = A^T x.
    {
        std::vector<double> wantT(m, 0.0), scaleT(m, 0.0);
        for (int r = 0; r < m; ++r)
            for (int j = A.rowPtr[r]; j < A.rowPtr[r + 1]; ++j) {
                wantT[A.colIdx[j]] += (double)A.values[j] * x[r];
                scaleT[A.colIdx[j]] += std::fabs((double)A.values[j] * x[r]);
            }
        status = spmv_exec_transpose<float>(handle, SPMV_FORMAT_CSR, &A, dx, dy);
        cudaStreamSynchronize(st);
        cudaMemcpy(y.data(), dy, m * sizeof(float), cudaMemcpyDeviceToHost);
        report("spmv_exec_transpose CSR", status == SPMV_SUCCESS && close(y, wantT, scaleT));
        report("spmv_exec_transpose CSR5 unsupported",
               spmv_exec_transpose<float>(handle, SPMV_FORMAT_CSR5, &csr5, dx, dy) == SPMV_ERROR_UNSUPPORTED_FORMAT);
    }

    // column_reorder.cuh: reorderColumns + reorderXVector keep y.
    CSRMatrix<float> B;
    std::vector<int> fmap;
    ColumnReorderStats stats{};
    status = reorderColumns<float>(A, B, fmap, stats);
    std::vector<float> xr(m);
    reorderXVector<float>(x.data(), xr.data(), fmap);
    B.allocateDevice();
    B.copyToDevice();
    cudaMemcpy(dx, xr.data(), m * sizeof(float), cudaMemcpyHostToDevice);
    opts.stream = nullptr;
    status = status == SPMV_SUCCESS ? spmv_csr<float>(B, dx, dy, 1.0f, 0.0f, opts) : status;
    fetch();
    report("reorderColumns + reorderXVector", status == SPMV_SUCCESS && close(y, want, scale));
    status = sortColumnsWithinRows<float>(B);
    bool sorted = status == SPMV_SUCCESS;
    for (int r = 0; r < m && sorted; ++r)
        for (int j = B.rowPtr[r]; j + 1 < B.rowPtr[r + 1] && sorted; ++j) sorted = B.colIdx[j] <= B.colIdx[j + 1];
    report("sortColumnsWithinRows", sorted);

    // BSR of the column-sorted B (dx still holds the reordered x): spmv_bsr and spmv_exec
    B.copyToDevice();
    {
        BSRMatrix<float, 4> bsr;
        status = csr_to_bsr<float, 4>(B, bsr);
        bool ok = status == SPMV_SUCCESS && bsr.numBlockRows == (m + 3) / 4 && bsr.numBlocks > 0;
        cudaMemset(dy, 0, m * sizeof(float));
        ok = ok && spmv_bsr<float, 4>(bsr, dx, dy) == SPMV_SUCCESS;
        fetch();
        report("csr_to_bsr + spmv_bsr", ok && close(y, want, scale));
        cudaMemset(dy, 0, m * sizeof(float));
        status = spmv_exec<float>(handle, SPMV_FORMAT_BSR, &bsr, dx, dy);
        cudaStreamSynchronize(st);
        cudaMemcpy(y.data(), dy, m * sizeof(float), cudaMemcpyDeviceToHost);
        report("spmv_exec BSR", status == SPMV_SUCCESS && close(y, want, scale));
    }

    // Matrix Market round trip through muxi_spmv::io (src/generators/mtx_io.h).
    {
        char path[] = "/tmp/muxi_dropin_XXXXXX";
        const int fd = mkstemp(path);
        bool ok = fd >= 0;
        if (ok) close(fd);
        ok = ok && io::writeMTXFile<float>(path, B) == SPMV_SUCCESS;
        io::MTXHeader hdr{};
        ok = ok && io::readMTXHeader(path, hdr) == SPMV_SUCCESS && hdr.numRows == B.numRows && hdr.nnz == B.nnz;
        CSRMatrix<float> R;
        ok = ok && io::readMTXFile<float>(path, R) == SPMV_SUCCESS && R.nnz == B.nnz;
        for (int r = 0; ok && r <= B.numRows; ++r) ok = R.rowPtr[r] == B.rowPtr[r];
        for (int j = 0; ok && j < B.nnz; ++j) ok = R.colIdx[j] == B.colIdx[j] && R.values[j] == B.values[j];
        std::remove(path);
        report("io::writeMTXFile + io::readMTXFile", ok);
    }

    spmv_destroy_handle(handle);
    cudaStreamDestroy(st);
    cudaFree(d_x);
    cudaFree(d_y);
    cudaFree(dx);
    cudaFree(dy);
    std::printf("\nTest: %s\n", failures == 0 ? "PASSED" : "FAILED");
    return failures == 0 ? 0 : 1;
}
