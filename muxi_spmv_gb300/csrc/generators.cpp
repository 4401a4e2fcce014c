// Seeded synthetic CSR generators (host).  They replace the libc-rand()
// generators of src/generators/matrix_generator.cu:29-345, which produce
// duplicate entries and cannot be seeded per matrix.
//
// Determinism: every row draws from its own counter-based stream
// (splitmix64 over (seed, row, purpose)), so the output does not depend on the
// number of threads.  Sampling uses only +,-,*,/, sqrt and exact scaling by
// powers of two (the logarithm and exponential below are series written out
// here, built with -ffp-contract=off), so x86-64 and AArch64 hosts produce the
// same bits.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "muxi_spmv.h"

namespace {

// ---------------------------------------------------------------------------
// Counter-based random streams
// ---------------------------------------------------------------------------
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

struct Stream {
    uint64_t s;
    Stream(uint64_t seed, uint64_t row, uint64_t purpose)
        : s(mix64(seed * 0x9e3779b97f4a7c15ULL + mix64(row * 4 + purpose + 0x632be59bd9b4e019ULL))) {}
    uint64_t next() {
        s += 0x9e3779b97f4a7c15ULL;
        return mix64(s);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    // Uniform integer in [0, n) by multiply-shift (n < 2^32).
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
};

// ---------------------------------------------------------------------------
// Deterministic log / exp from their series.
// ---------------------------------------------------------------------------
const double kLn2 = 0.6931471805599453094172321;

double det_log(double x) {
    // x = m * 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(z), z=(m-1)/(m+1).
    int e = 0;
    double m = std::frexp(x, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    const double z = (m - 1.0) / (m + 1.0);
    const double z2 = z * z;
    double term = z, sum = 0.0;
    for (int k = 0; k < 40; ++k) {
        sum += term / (double)(2 * k + 1);
        term *= z2;
    }
    return 2.0 * sum + (double)e * kLn2;
}

double det_exp(double x) {
    if (x < -745.0) return 0.0;
    const double n = std::floor(x / kLn2 + 0.5);
    const double r = x - n * kLn2;  // |r| <= ~0.35
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 30; ++k) {
        term *= r / (double)k;
        sum += term;
    }
    return std::ldexp(sum, (int)n);
}

// Standard normal by Marsaglia's polar method.
double normal(Stream& st) {
    for (;;) {
        const double u = 2.0 * st.uniform() - 1.0;
        const double v = 2.0 * st.uniform() - 1.0;
        const double s = u * u + v * v;
        if (s > 0.0 && s < 1.0) return u * std::sqrt(-2.0 * det_log(s) / s);
    }
}

// ---------------------------------------------------------------------------
// Length laws as inverse-CDF tables.
// ---------------------------------------------------------------------------
struct Table {
    int first = 0;            // value of cdf[0]
    std::vector<double> cdf;  // cumulative probability, last == 1
    int sample(Stream& st) const {
        const double u = st.uniform();
        const size_t k = std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin();
        return first + (int)std::min(k, cdf.size() - 1);
    }
};

// Poisson(lambda) clamped to [lo, hi]: mass below lo moves to lo, above hi to hi.
Table poisson_table(double lambda, int lo, int hi) {
    Table t;
    t.first = lo;
    const int kmax = (int)(lambda + 40.0 * std::sqrt(lambda + 1.0) + 40.0);
    std::vector<double> pmf(kmax + 1);
    // log pmf(k) = -lambda + k log lambda - log k!
    double lfact = 0.0;
    const double llam = lambda > 0 ? det_log(lambda) : 0.0;
    for (int k = 0; k <= kmax; ++k) {
        if (k > 0) lfact += det_log((double)k);
        pmf[k] = lambda > 0 ? det_exp(-lambda + k * llam - lfact) : (k == 0 ? 1.0 : 0.0);
    }
    const int top = std::max(lo, hi);
    t.cdf.assign(top - lo + 1, 0.0);
    for (int k = 0; k <= kmax; ++k) {
        const int c = std::min(std::max(k, lo), top);
        t.cdf[c - lo] += pmf[k];
    }
    double acc = 0.0;
    for (double& v : t.cdf) v = (acc += v);
    for (double& v : t.cdf) v /= acc;
    t.cdf.back() = 1.0;
    return t;
}

// Zipf(s) on {1..M}: P(k) proportional to k^-s (support truncated to [1,M]).
Table zipf_table(double s, int M) {
    Table t;
    t.first = 1;
    t.cdf.resize(M);
    double acc = 0.0;
    for (int k = 1; k <= M; ++k) {
        acc += det_exp(-s * det_log((double)k));
        t.cdf[k - 1] = acc;
    }
    for (double& v : t.cdf) v /= acc;
    t.cdf.back() = 1.0;
    return t;
}

// ---------------------------------------------------------------------------
// Per-row column sets
// ---------------------------------------------------------------------------
// k distinct values from [base, base+range), sorted ascending.
void distinct_sorted(Stream& st, int base, int range, int k, std::vector<int>& out) {
    out.clear();
    if (k <= 0 || range <= 0) return;
    if (k >= range) {
        for (int i = 0; i < range; ++i) out.push_back(base + i);
        return;
    }
    if ((long long)k * 2 > range) {
        // Draw the complement instead.
        std::vector<int> skip;
        distinct_sorted(st, 0, range, range - k, skip);
        size_t p = 0;
        for (int i = 0; i < range; ++i) {
            if (p < skip.size() && skip[p] == i) {
                ++p;
                continue;
            }
            out.push_back(base + i);
        }
        return;
    }
    while ((int)out.size() < k) {
        const int need = k - (int)out.size();
        for (int i = 0; i < need; ++i) out.push_back((int)st.below((uint32_t)range));
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }
    for (int& v : out) v += base;
}

int reflect(long long c, int n) {
    if (n <= 1) return 0;
    while (c < 0 || c >= n) {
        if (c < 0) c = -c;
        if (c >= n) c = 2LL * (n - 1) - c;
    }
    return (int)c;
}

struct Gen {
    spmv_gen_params_t p;
    Table lenTable;
    bool hasTable = false;

    explicit Gen(const spmv_gen_params_t& q) : p(q) {
        switch (p.kind) {
            case SPMV_GEN_POISSON_UNIFORM: {
                const int lo = std::max(0, (int)p.p1);
                const int hi = std::min((int)p.p2, p.numCols);
                lenTable = poisson_table(p.p0, lo, std::max(lo, hi));
                hasTable = true;
                break;
            }
            case SPMV_GEN_POWERLAW:
                lenTable = zipf_table(p.p0, std::max(1, (int)p.p1));
                hasTable = true;
                break;
            case SPMV_GEN_ZIPF_UNIFORM:
                // p2 >= 1 shifts every length up by p2 (mean beyond Zipf's own).
                lenTable = zipf_table(p.p0, std::max(1, (int)p.p1));
                lenTable.first += std::max(0, (int)p.p2);
                hasTable = true;
                break;
            case SPMV_GEN_BANDED:
                lenTable = poisson_table(p.p0, 1, std::max(1, std::min((int)p.p1, p.numCols)));
                hasTable = true;
                break;
            case SPMV_GEN_BLOCKDIAG:
                lenTable = poisson_table(p.p1, 1, std::max(1, p.numCols));
                hasTable = true;
                break;
            default:
                break;
        }
    }

    void block_of(int row, int& b0, int& bsz) const {
        const long long nb = std::max(1LL, (long long)p.p0);
        const long long b = (long long)row * nb / p.numRows;
        const long long c0 = b * p.numCols / nb, c1 = (b + 1) * p.numCols / nb;
        b0 = (int)c0;
        bsz = (int)(c1 - c0);
    }

    int row_len(int row) const {
        switch (p.kind) {
            case SPMV_GEN_DIAGONAL:
                return row < p.numCols ? 1 : 0;
            case SPMV_GEN_STENCIL2D: {
                const int nx = (int)p.p0, ny = (int)p.p1;
                const int i = row / ny, j = row % ny;
                return 1 + (i > 0) + (i < nx - 1) + (j > 0) + (j < ny - 1);
            }
            case SPMV_GEN_STENCIL3D: {
                const long long n1 = (long long)p.p1, n2 = (long long)p.p2;
                const long long k = row / (n1 * n2), rem = row % (n1 * n2);
                const long long j = rem / n2, i = rem % n2;
                const long long n0 = (long long)p.p0;
                auto span = [](long long v, long long n) { return (int)(1 + (v > 0) + (v < n - 1)); };
                return span(k, n0) * span(j, n1) * span(i, n2);
            }
            case SPMV_GEN_BLOCKDIAG: {
                Stream st(p.seed, row, 0);
                int b0, bsz;
                block_of(row, b0, bsz);
                return std::min(lenTable.sample(st), std::max(bsz, 0));
            }
            default: {
                Stream st(p.seed, row, 0);
                int k = lenTable.sample(st);
                if (p.kind == SPMV_GEN_POISSON_UNIFORM || p.kind == SPMV_GEN_ZIPF_UNIFORM)
                    k = std::min(k, p.numCols);
                if (p.kind == SPMV_GEN_BANDED) {
                    const int w = std::max(1, (int)p.p1);
                    k = std::min(k, w);
                }
                return k;
            }
        }
    }

    template <typename T>
    void fill_row(int row, int len, int* col, T* val, std::vector<int>& tmp) const {
        Stream cs(p.seed, row, 1), vs(p.seed, row, 2);
        switch (p.kind) {
            case SPMV_GEN_DIAGONAL:
                if (len) {
                    col[0] = row;
                    val[0] = T(1);
                }
                return;
            case SPMV_GEN_STENCIL2D: {
                const int ny = (int)p.p1, nx = (int)p.p0;
                const int i = row / ny, j = row % ny;
                int n = 0;
                if (i > 0) { col[n] = row - ny; val[n++] = T(-1); }
                if (j > 0) { col[n] = row - 1; val[n++] = T(-1); }
                col[n] = row; val[n++] = T(4);
                if (j < ny - 1) { col[n] = row + 1; val[n++] = T(-1); }
                if (i < nx - 1) { col[n] = row + ny; val[n++] = T(-1); }
                return;
            }
            case SPMV_GEN_STENCIL3D: {
                const long long n0 = (long long)p.p0, n1 = (long long)p.p1, n2 = (long long)p.p2;
                const long long k = row / (n1 * n2), rem = row % (n1 * n2);
                const long long j = rem / n2, i = rem % n2;
                int n = 0;
                for (int dk = -1; dk <= 1; ++dk)
                    for (int dj = -1; dj <= 1; ++dj)
                        for (int di = -1; di <= 1; ++di) {
                            const long long kk = k + dk, jj = j + dj, ii = i + di;
                            if (kk < 0 || kk >= n0 || jj < 0 || jj >= n1 || ii < 0 || ii >= n2) continue;
                            col[n] = (int)((kk * n1 + jj) * n2 + ii);
                            val[n++] = T(normal(vs));
                        }
                return;
            }
            case SPMV_GEN_POISSON_UNIFORM:
            case SPMV_GEN_ZIPF_UNIFORM:
                distinct_sorted(cs, 0, p.numCols, len, tmp);
                break;
            case SPMV_GEN_BANDED: {
                const int w = std::max(1, (int)p.p1);
                long long lo = (long long)row - w / 2;
                lo = std::max(0LL, std::min(lo, (long long)p.numCols - w));
                const int range = (int)std::min<long long>(w, p.numCols - lo);
                distinct_sorted(cs, (int)lo, range, len, tmp);
                break;
            }
            case SPMV_GEN_BLOCKDIAG: {
                int b0, bsz;
                block_of(row, b0, bsz);
                distinct_sorted(cs, b0, bsz, len, tmp);
                break;
            }
            case SPMV_GEN_POWERLAW: {
                tmp.resize(len);
                const int band = (int)p.p2;
                for (int e = 0; e < len; ++e) {
                    const double u = cs.uniform();
                    if (u < p.p3) {
                        const long long off = (long long)cs.below((uint32_t)(2 * band + 1)) - band;
                        tmp[e] = reflect((long long)row + off, p.numCols);
                    } else {
                        tmp[e] = (int)cs.below((uint32_t)p.numCols);
                    }
                }
                std::sort(tmp.begin(), tmp.end());
                break;
            }
            default:
                break;
        }
        const bool uniform_vals = p.kind == SPMV_GEN_POISSON_UNIFORM;
        for (int e = 0; e < len; ++e) {
            col[e] = tmp[e];
            val[e] = uniform_vals ? T(2.0 * vs.uniform() - 1.0) : T(normal(vs));
        }
    }
};

int thread_count(int requested) {
    if (requested > 0) return requested;
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

template <typename F>
void parallel_rows(long long n, int threads, F&& body) {
    const long long chunk = 2048;
    std::atomic<long long> next(0);
    auto worker = [&]() {
        for (;;) {
            const long long b = next.fetch_add(chunk);
            if (b >= n) return;
            body(b, std::min(n, b + chunk));
        }
    };
    const int t = (int)std::min<long long>(thread_count(threads), (n + chunk - 1) / chunk);
    if (t <= 1) {
        worker();
        return;
    }
    std::vector<std::thread> pool;
    for (int i = 0; i < t; ++i) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
}

bool params_ok(const spmv_gen_params_t* p) {
    if (!p || p->numRows < 0 || p->numCols < 0) return false;
    switch (p->kind) {
        case SPMV_GEN_STENCIL2D:
            return (long long)p->p0 * (long long)p->p1 == p->numRows && p->numRows == p->numCols;
        case SPMV_GEN_STENCIL3D:
            return (long long)p->p0 * (long long)p->p1 * (long long)p->p2 == p->numRows &&
                   p->numRows == p->numCols;
        case SPMV_GEN_POWERLAW:
            return p->p0 > 0 && p->p1 >= 1 && p->p2 >= 0 && p->p3 >= 0 && p->p3 <= 1 && p->numCols > 0;
        case SPMV_GEN_POISSON_UNIFORM:
        case SPMV_GEN_BANDED:
        case SPMV_GEN_BLOCKDIAG:
        case SPMV_GEN_ZIPF_UNIFORM:
            return p->numCols > 0 || p->numRows == 0;
        case SPMV_GEN_DIAGONAL:
            return true;
    }
    return false;
}

template <typename T>
spmv_status_t fill(const spmv_gen_params_t* p, const int* rowPtr, int* colIdx, T* values) {
    if (!params_ok(p) || !rowPtr) return SPMV_ERROR_INVALID_MATRIX;
    if (rowPtr[p->numRows] > 0 && (!colIdx || !values)) return SPMV_ERROR_INVALID_VECTOR;
    Gen g(*p);
    parallel_rows(p->numRows, p->threads, [&](long long b, long long e) {
        std::vector<int> tmp;
        for (long long r = b; r < e; ++r) {
            const int s = rowPtr[r], len = rowPtr[r + 1] - s;
            g.fill_row<T>((int)r, len, colIdx + s, values + s, tmp);
        }
    });
    return SPMV_SUCCESS;
}

template <typename T>
spmv_status_t vec(long long n, unsigned long long seed, double lo, double hi, T* out, int threads) {
    if (n < 0 || (n > 0 && !out)) return SPMV_ERROR_INVALID_VECTOR;
    parallel_rows(n, threads, [&](long long b, long long e) {
        for (long long i = b; i < e; ++i) {
            const double u = (double)(mix64(seed * 0xd1b54a32d192ed03ULL + mix64((uint64_t)i + 1)) >> 11) *
                             (1.0 / 9007199254740992.0);
            out[i] = T(lo + (hi - lo) * u);
        }
    });
    return SPMV_SUCCESS;
}

}  // namespace

namespace mxs {
// Inverse-CDF table of the row-length law of `p` (POISSON_UNIFORM, POWERLAW,
// ZIPF_UNIFORM, BANDED, BLOCKDIAG): lengths are first + index of the first
// cdf entry above a uniform draw.  Returns false for laws without a table.
bool gen_length_table(const spmv_gen_params_t& p, std::vector<double>& cdf, int& first) {
    Gen g(p);
    if (!g.hasTable) return false;
    cdf = g.lenTable.cdf;
    first = g.lenTable.first;
    return true;
}
// Mean of the truncated Zipf(s) law on [1, M].
double zipf_mean(double s, int M) {
    double num = 0.0, den = 0.0;
    for (int k = 1; k <= M; ++k) {
        const double w = det_exp(-s * det_log((double)k));
        num += k * w;
        den += w;
    }
    return num / den;
}
}  // namespace mxs

extern "C" {

spmv_status_t spmv_gen_row_ptr(const spmv_gen_params_t* p, int* rowPtr, long long* nnz) {
    if (!params_ok(p) || !rowPtr || !nnz) return SPMV_ERROR_INVALID_MATRIX;
    Gen g(*p);
    const int R = p->numRows;
    parallel_rows(R, p->threads, [&](long long b, long long e) {
        for (long long r = b; r < e; ++r) rowPtr[r + 1] = g.row_len((int)r);
    });
    long long acc = 0;
    rowPtr[0] = 0;
    for (int r = 0; r < R; ++r) {
        acc += rowPtr[r + 1];
        if (acc > 0x7fffffffLL) {
            *nnz = acc;
            return SPMV_ERROR_INVALID_MATRIX;
        }
        rowPtr[r + 1] = (int)acc;
    }
    *nnz = acc;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_gen_fill_f32(const spmv_gen_params_t* p, const int* rowPtr, int* colIdx, float* values) {
    return fill<float>(p, rowPtr, colIdx, values);
}
spmv_status_t spmv_gen_fill_f64(const spmv_gen_params_t* p, const int* rowPtr, int* colIdx, double* values) {
    return fill<double>(p, rowPtr, colIdx, values);
}
spmv_status_t spmv_gen_vector_f32(long long n, unsigned long long seed, double lo, double hi, float* out,
                                  int threads) {
    return vec<float>(n, seed, lo, hi, out, threads);
}
spmv_status_t spmv_gen_vector_f64(long long n, unsigned long long seed, double lo, double hi, double* out,
                                  int threads) {
    return vec<double>(n, seed, lo, hi, out, threads);
}

}  // extern "C"
