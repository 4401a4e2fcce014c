// Matrix Market coordinate files <-> host CSR.
//
// Follows the reference's reader (src/generators/mtx_io.cu:17-222): banner
// "%%MatrixMarket matrix coordinate <real|integer|pattern> <general|symmetric>",
// '%' comment lines, a "rows cols entries" line, 1-based entries; pattern
// entries get value 1; symmetric files are expanded to both triangles (the
// mirror of every off-diagonal entry) unless asked not to; entries are sorted
// by (row, column) and duplicates are kept.  Differences: ties between
// duplicate (row, column) entries keep file order (the reference's std::sort
// leaves them unspecified); complex files are refused instead of misread;
// entries outside the declared shape are refused.  The writer emits the
// banner the reader accepts (the reference's writer prints "%MatrixMarket",
// mtx_io.cu:234, which its own reader rejects) and writes values with enough
// digits to read back exactly (the reference used %g).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace mxs {
namespace {

struct Banner {
    spmv_mtx_header_t h{};
    bool ok = false;
};

bool starts(const char* p, const char* w) { return std::strncmp(p, w, std::strlen(w)) == 0; }

const char* skip_ws(const char* p) {
    while (*p == ' ' || *p == '\t') ++p;
    return p;
}

// Lower-cased copy of the banner tokens after "%%MatrixMarket".
Banner parse_banner(const std::string& line) {
    Banner b;
    if (!starts(line.c_str(), "%%MatrixMarket")) return b;
    std::string low;
    for (char c : line.substr(14)) low += (char)std::tolower((unsigned char)c);
    const char* p = skip_ws(low.c_str());
    if (!starts(p, "matrix")) return b;
    p = skip_ws(p + 6);
    if (!starts(p, "coordinate")) return b;
    p = skip_ws(p + 10);
    if (starts(p, "real")) {
        p += 4;
    } else if (starts(p, "integer")) {
        b.h.isInteger = 1;
        p += 7;
    } else if (starts(p, "pattern")) {
        b.h.isPattern = 1;
        p += 7;
    } else if (starts(p, "complex")) {
        b.h.isComplex = 1;
        p += 7;
    } else {
        return b;
    }
    p = skip_ws(p);
    if (starts(p, "symmetric")) b.h.isSymmetric = 1;
    else if (starts(p, "skew-symmetric")) b.h.isSkew = 1;
    else if (starts(p, "hermitian")) b.h.isSymmetric = 1;
    b.ok = true;
    return b;
}

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

bool read_line(FILE* f, std::string& line) {
    line.clear();
    int c;
    while ((c = std::fgetc(f)) != EOF) {
        if (c == '\n') return true;
        line += (char)c;
    }
    return !line.empty();
}

// Reads banner, comments and the size line.
spmv_status_t read_head(FILE* f, const char* path, spmv_mtx_header_t* h) {
    std::string line;
    if (!read_line(f, line)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: empty file", path);
    const Banner b = parse_banner(line);
    if (!b.ok) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: not a Matrix Market coordinate banner", path);
    *h = b.h;
    do {
        if (!read_line(f, line)) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: no size line", path);
    } while (line.empty() || line[0] == '%');
    long long r = 0, c = 0, n = 0;
    if (std::sscanf(line.c_str(), "%lld %lld %lld", &r, &c, &n) != 3 || r < 0 || c < 0 || n < 0 ||
        r > 0x7fffffff || c > 0x7fffffff || n > 0x7fffffff)
        MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: bad size line '%s'", path, line.c_str());
    h->numRows = (int)r;
    h->numCols = (int)c;
    h->nnz = (int)n;
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t read_csr(const char* path, int expand, spmv_host_csr_t* out) {
    File F;
    F.f = std::fopen(path, "rb");
    if (!F.f) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "cannot open %s", path);
    spmv_mtx_header_t h;
    MXS_TRY(read_head(F.f, path, &h));
    if (h.isComplex) MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "%s: complex matrices are not supported", path);
    // Body: the rest of the file in one buffer, parsed with strtol/strtod.
    std::vector<char> buf;
    {
        char tmp[1 << 16];
        size_t got;
        while ((got = std::fread(tmp, 1, sizeof tmp, F.f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
        buf.push_back('\0');
    }
    const bool mirror = expand && (h.isSymmetric || h.isSkew);
    const long long cap = (long long)h.nnz * (mirror ? 2 : 1);
    if (cap > 0x7fffffff) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: more than 2^31-1 entries after expansion", path);
    std::vector<int> ri, ci;
    std::vector<T> va;
    ri.reserve(cap);
    ci.reserve(cap);
    va.reserve(cap);
    char* p = buf.data();
    for (int k = 0; k < h.nnz; ++k) {
        // skip blank and comment lines between entries
        for (;;) {
            while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') ++p;
            if (*p != '%') break;
            while (*p && *p != '\n') ++p;
        }
        char* e;
        errno = 0;
        const long r = std::strtol(p, &e, 10);
        if (e == p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: entry %d: missing row index", path, k + 1);
        p = e;
        const long c = std::strtol(p, &e, 10);
        if (e == p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: entry %d: missing column index", path, k + 1);
        p = e;
        double v = 1.0;
        if (!h.isPattern) {
            v = std::strtod(p, &e);
            if (e == p) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: entry %d: missing value", path, k + 1);
            p = e;
        }
        if (r < 1 || r > h.numRows || c < 1 || c > h.numCols)
            MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: entry %d (%ld, %ld) outside %d x %d", path, k + 1, r, c,
                     h.numRows, h.numCols);
        ri.push_back((int)r - 1);
        ci.push_back((int)c - 1);
        va.push_back((T)v);
        if (mirror && r != c) {
            if (c > h.numRows || r > h.numCols)
                MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "%s: symmetric entry %d outside a square shape", path, k + 1);
            ri.push_back((int)c - 1);
            ci.push_back((int)r - 1);
            va.push_back(h.isSkew ? (T)(-v) : (T)v);
        }
    }
    // Stable counting sort by row, then stable sort by column within rows.
    const int R = h.numRows;
    const size_t N = va.size();
    std::vector<int> rp(R + 1, 0);
    for (int r : ri) ++rp[r + 1];
    for (int r = 0; r < R; ++r) rp[r + 1] += rp[r];
    std::vector<int> pos(rp.begin(), rp.end() - 1);
    std::vector<int> order(N);
    for (size_t k = 0; k < N; ++k) order[pos[ri[k]]++] = (int)k;
    int* outRp = static_cast<int*>(std::malloc(sizeof(int) * (R + 1)));
    int* outCi = static_cast<int*>(std::malloc(sizeof(int) * (N ? N : 1)));
    T* outVa = static_cast<T*>(std::malloc(sizeof(T) * (N ? N : 1)));
    if (!outRp || !outCi || !outVa) {
        std::free(outRp);
        std::free(outCi);
        std::free(outVa);
        MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory for %zu entries", N);
    }
    std::vector<int> seg;
    for (int r = 0; r < R; ++r) {
        outRp[r] = rp[r];
        seg.assign(order.begin() + rp[r], order.begin() + rp[r + 1]);
        std::stable_sort(seg.begin(), seg.end(), [&](int a, int b) { return ci[a] < ci[b]; });
        for (size_t i = 0; i < seg.size(); ++i) {
            outCi[rp[r] + i] = ci[seg[i]];
            outVa[rp[r] + i] = va[seg[i]];
        }
    }
    outRp[R] = (int)N;
    out->numRows = R;
    out->numCols = h.numCols;
    out->nnz = (int)N;
    out->rowPtr = outRp;
    out->colIdx = outCi;
    out->values = outVa;
    out->type = sizeof(T) == 4 ? SPMV_TYPE_FLOAT : SPMV_TYPE_DOUBLE;
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t write_csr(const char* path, const spmv_host_csr_t* m, int symmetric) {
    const T* v = static_cast<const T*>(m->values);
    long long n = 0;
    for (int r = 0; r < m->numRows; ++r)
        for (int j = m->rowPtr[r]; j < m->rowPtr[r + 1]; ++j)
            if (!symmetric || m->colIdx[j] >= r) ++n;
    File F;
    F.f = std::fopen(path, "w");
    if (!F.f) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "cannot open %s for writing", path);
    std::fprintf(F.f, "%%%%MatrixMarket matrix coordinate real %s\n", symmetric ? "symmetric" : "general");
    std::fprintf(F.f, "%% rows %d, columns %d, nonzeros %d\n", m->numRows, m->numCols, m->nnz);
    std::fprintf(F.f, "%d %d %lld\n", m->numRows, m->numCols, n);
    const char* fmt = sizeof(T) == 4 ? "%d %d %.9g\n" : "%d %d %.17g\n";
    for (int r = 0; r < m->numRows; ++r)
        for (int j = m->rowPtr[r]; j < m->rowPtr[r + 1]; ++j)
            if (!symmetric || m->colIdx[j] >= r) std::fprintf(F.f, fmt, r + 1, m->colIdx[j] + 1, (double)v[j]);
    if (std::ferror(F.f)) MXS_FAIL(SPMV_ERROR_INTERNAL, "write error on %s", path);
    return SPMV_SUCCESS;
}

}  // namespace
}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_mtx_read_header(const char* path, spmv_mtx_header_t* header) {
    clear_error();
    if (!path || !header) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    File F;
    F.f = std::fopen(path, "rb");
    if (!F.f) MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "cannot open %s", path);
    return read_head(F.f, path, header);
}

spmv_status_t spmv_mtx_read(const char* path, spmv_type_t type, int expandSymmetric, spmv_host_csr_t* out) {
    clear_error();
    if (!path || !out) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    if (type == SPMV_TYPE_FLOAT) return read_csr<float>(path, expandSymmetric, out);
    if (type == SPMV_TYPE_DOUBLE) return read_csr<double>(path, expandSymmetric, out);
    MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "float or double");
}

spmv_status_t spmv_mtx_write(const char* path, const spmv_host_csr_t* m, int writeSymmetric) {
    clear_error();
    if (!path || !m) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    if (m->numRows < 0 || m->nnz < 0 || (m->numRows > 0 && !m->rowPtr) || (m->nnz > 0 && (!m->colIdx || !m->values)))
        MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "bad host CSR");
    if (m->type == SPMV_TYPE_FLOAT) return write_csr<float>(path, m, writeSymmetric);
    if (m->type == SPMV_TYPE_DOUBLE) return write_csr<double>(path, m, writeSymmetric);
    MXS_FAIL(SPMV_ERROR_UNSUPPORTED_TYPE, "float or double");
}

void spmv_host_csr_free(spmv_host_csr_t* m) {
    if (!m) return;
    std::free(m->rowPtr);
    std::free(m->colIdx);
    std::free(m->values);
    m->rowPtr = nullptr;
    m->colIdx = nullptr;
    m->values = nullptr;
}

}  // extern "C"
