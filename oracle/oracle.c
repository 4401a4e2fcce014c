/*
 * oracle.c -- CPU restatement of the muxi_spmv hot path (test
 * infrastructure; see oracle.h).  Built with -ffp-contract=off so that every
 * float operation is the one written.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------ */
/* Row-parallel driver: chunks of rows handed out by an atomic counter. */
/* ------------------------------------------------------------------ */
typedef void (*row_fn)(void* ctx, int r0, int r1);

typedef struct {
    row_fn fn;
    void* ctx;
    int rows;
    int chunk;
    atomic_int next;
} par_t;

static void* par_worker(void* arg) {
    par_t* p = (par_t*)arg;
    for (;;) {
        int b = atomic_fetch_add(&p->next, p->chunk);
        if (b >= p->rows) break;
        int e = b + p->chunk < p->rows ? b + p->chunk : p->rows;
        p->fn(p->ctx, b, e);
    }
    return NULL;
}

static int hw_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

static void parallel_rows(int rows, int threads, int chunk, row_fn fn, void* ctx) {
    if (threads <= 0) threads = hw_threads();
    if (threads > 256) threads = 256;
    if (rows <= chunk || threads == 1) {
        fn(ctx, 0, rows);
        return;
    }
    par_t p;
    p.fn = fn;
    p.ctx = ctx;
    p.rows = rows;
    p.chunk = chunk;
    atomic_init(&p.next, 0);
    pthread_t th[256];
    int started = 0;
    for (int i = 0; i < threads - 1; ++i)
        if (pthread_create(&th[started], NULL, par_worker, &p) == 0) ++started;
    par_worker(&p);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
}

/* ------------------------------------------------------------------ */
/* FP64 oracles                                                         */
/* ------------------------------------------------------------------ */
typedef struct {
    const int* rowPtr;
    const int* colIdx;
    const void* values;
    const void* x;
    double* y;
    double* absum;
} spmv_ctx;

static void rows_f32_ref(void* c, int r0, int r1) {
    spmv_ctx* k = (spmv_ctx*)c;
    const float* v = (const float*)k->values;
    const float* x = (const float*)k->x;
    for (int r = r0; r < r1; ++r) {
        double s = 0.0, comp = 0.0, a = 0.0;
        for (int j = k->rowPtr[r]; j < k->rowPtr[r + 1]; ++j) {
            const double p = (double)v[j] * (double)x[k->colIdx[j]]; /* exact */
            const double t = s + p;
            if (fabs(s) >= fabs(p)) comp += (s - t) + p;
            else comp += (p - t) + s;
            s = t;
            a += fabs(p);
        }
        k->y[r] = s + comp;
        if (k->absum) k->absum[r] = a;
    }
}

void oracle_spmv_f32(int rows, const int* rowPtr, const int* colIdx, const float* values, const float* x,
                     double* y_ref, double* absum, int threads) {
    spmv_ctx c = {rowPtr, colIdx, values, x, y_ref, absum};
    parallel_rows(rows, threads, 4096, rows_f32_ref, &c);
}

/* Double-double helpers: TwoSum (Knuth) and TwoProduct through fma. */
static inline void two_sum(double a, double b, double* s, double* e) {
    double t = a + b;
    double bb = t - a;
    *e = (a - (t - bb)) + (b - bb);
    *s = t;
}

static void rows_f64_ref(void* c, int r0, int r1) {
    spmv_ctx* k = (spmv_ctx*)c;
    const double* v = (const double*)k->values;
    const double* x = (const double*)k->x;
    for (int r = r0; r < r1; ++r) {
        double hi = 0.0, lo = 0.0, a = 0.0;
        for (int j = k->rowPtr[r]; j < k->rowPtr[r + 1]; ++j) {
            const double xv = x[k->colIdx[j]];
            const double p = v[j] * xv;
            const double pe = fma(v[j], xv, -p); /* exact product error */
            double s, e;
            two_sum(hi, p, &s, &e);
            e += lo + pe;
            two_sum(s, e, &hi, &lo);
            a += fabs(p);
        }
        k->y[r] = hi + lo;
        if (k->absum) k->absum[r] = a;
    }
}

void oracle_spmv_f64(int rows, const int* rowPtr, const int* colIdx, const double* values, const double* x,
                     double* y_ref, double* absum, int threads) {
    spmv_ctx c = {rowPtr, colIdx, values, x, y_ref, absum};
    parallel_rows(rows, threads, 4096, rows_f64_ref, &c);
}

/* ------------------------------------------------------------------ */
/* The reference's CPU loop (tests/deep_analysis.cu:189-195)            */
/* ------------------------------------------------------------------ */
typedef struct {
    const int* rowPtr;
    const int* colIdx;
    const void* values;
    const void* x;
    void* y;
} cpu_ctx;

static void rows_cpu_f32(void* c, int r0, int r1) {
    cpu_ctx* k = (cpu_ctx*)c;
    const float* v = (const float*)k->values;
    const float* x = (const float*)k->x;
    float* y = (float*)k->y;
    for (int r = r0; r < r1; ++r) {
        float sum = 0;
        for (int j = k->rowPtr[r]; j < k->rowPtr[r + 1]; ++j) sum += v[j] * x[k->colIdx[j]];
        y[r] = sum;
    }
}

static void rows_cpu_f64(void* c, int r0, int r1) {
    cpu_ctx* k = (cpu_ctx*)c;
    const double* v = (const double*)k->values;
    const double* x = (const double*)k->x;
    double* y = (double*)k->y;
    for (int r = r0; r < r1; ++r) {
        double sum = 0;
        for (int j = k->rowPtr[r]; j < k->rowPtr[r + 1]; ++j) sum += v[j] * x[k->colIdx[j]];
        y[r] = sum;
    }
}

void oracle_cpu_spmv_f32(int rows, const int* rowPtr, const int* colIdx, const float* values, const float* x,
                         float* y, int threads) {
    cpu_ctx c = {rowPtr, colIdx, values, x, y};
    if (threads == 1) rows_cpu_f32(&c, 0, rows);
    else parallel_rows(rows, threads, 1024, rows_cpu_f32, &c);
}

void oracle_cpu_spmv_f64(int rows, const int* rowPtr, const int* colIdx, const double* values, const double* x,
                         double* y, int threads) {
    cpu_ctx c = {rowPtr, colIdx, values, x, y};
    if (threads == 1) rows_cpu_f64(&c, 0, rows);
    else parallel_rows(rows, threads, 1024, rows_cpu_f64, &c);
}

/* ------------------------------------------------------------------ */
/* Index outputs                                                        */
/* ------------------------------------------------------------------ */
/* csr5_binary_search_row (spmv_csr5.cuh:44-61): lo=0, hi=rows; move lo
 * past every row start <= idx; answer lo-1. */
static int last_row_starting_at_or_before(const int* rowPtr, int rows, long long idx) {
    int lo = 0, hi = rows;
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (rowPtr[mid] <= idx) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

void oracle_csr5_tiles(int rows, int nnz, const int* rowPtr, int sigma, int* tile_row_ptr,
                       int* tile_nnz_offset) {
    const long long tiles = ((long long)nnz + sigma - 1) / sigma;
    for (long long t = 0; t < tiles; ++t) {
        const long long start = t * sigma;
        const int r = last_row_starting_at_or_before(rowPtr, rows, start);
        tile_row_ptr[t] = r;
        tile_nnz_offset[t] = (int)(start - rowPtr[r]);
    }
}

void oracle_merge_partitions(int rows, int nnz, int P, int* pos) {
    const long long L = (long long)rows + nnz;
    const long long per = (L + P - 1) / P;
    for (long long t = 0; t <= P; ++t) {
        const long long v = t * per;
        pos[t] = (int)(v < L ? v : L);
    }
}

/* merge_path_search (spmv_csr5.cu:497-533): search window
 * [max(0,k-nnz), min(k,rows)]; step right while the nnz coordinate lies
 * past the row's end, left while it lies before the row's start, stop when
 * it lies inside; then clamp. */
void oracle_merge_search(const int* rowPtr, int rows, int nnz, const int* diag, int count, int* rowIdx,
                         int* nnzIdx) {
    for (int i = 0; i < count; ++i) {
        const long long k = diag[i];
        long long lo = k - nnz > 0 ? k - nnz : 0;
        long long hi = k < rows ? k : rows;
        while (lo < hi) {
            const long long mid = (lo + hi) / 2;
            const long long nz = k - mid;
            if (mid < rows && nz > rowPtr[mid + 1]) {
                lo = mid + 1;
            } else if (mid > 0 && nz < rowPtr[mid]) {
                hi = mid;
            } else {
                lo = mid;
                hi = mid;
            }
        }
        long long r = lo, z = k - lo;
        if (r > rows) r = rows;
        if (z > nnz) z = nnz;
        rowIdx[i] = (int)r;
        nnzIdx[i] = (int)z;
    }
}

int oracle_merge_default_partitions(int rows, int nnz) {
    const long long L = (long long)rows + nnz;
    const long long target = L / 32, maxP = 128LL * 8 * 8;
    long long p = target < maxP ? target : maxP;
    return (int)(p < 1 ? 1 : p);
}

int oracle_max_row_length(int rows, const int* rowPtr) {
    int m = 0;
    for (int r = 0; r < rows; ++r) {
        const int l = rowPtr[r + 1] - rowPtr[r];
        if (l > m) m = l;
    }
    return m;
}

#define DEFINE_ELL(SUF, T)                                                                              \
    long long oracle_csr_to_ell_##SUF(int rows, const int* rowPtr, const int* colIdx, const T* values, \
                                      int width, int* width_out, int* ellCol, T* ellVal) {              \
        if (width <= 0) width = oracle_max_row_length(rows, rowPtr);                                    \
        *width_out = width;                                                                             \
        const long long total = (long long)rows * width;                                                \
        for (long long i = 0; i < total; ++i) {                                                         \
            ellCol[i] = -1;                                                                             \
            ellVal[i] = (T)0;                                                                           \
        }                                                                                               \
        long long truncated = 0;                                                                        \
        for (int r = 0; r < rows; ++r) {                                                                \
            const int s = rowPtr[r], len = rowPtr[r + 1] - s;                                           \
            if (len > width) ++truncated;                                                               \
            for (int i = 0; i < len && i < width; ++i) {                                                \
                ellCol[r + (long long)i * rows] = colIdx[s + i];                                        \
                ellVal[r + (long long)i * rows] = values[s + i];                                        \
            }                                                                                           \
        }                                                                                               \
        return truncated;                                                                               \
    }
DEFINE_ELL(f32, float)
DEFINE_ELL(f64, double)

/* ------------------------------------------------------------------ */
/* Reorders                                                             */
/* ------------------------------------------------------------------ */
typedef struct {
    long long key;
    int id;
} keyed_t;

/* Ascending key, then ascending id: equals a stable sort of ids by key. */
static int cmp_keyed(const void* a, const void* b) {
    const keyed_t* x = (const keyed_t*)a;
    const keyed_t* y = (const keyed_t*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return (x->id > y->id) - (x->id < y->id);
}

void oracle_row_reorder_f32(int rows, const int* rowPtr, const int* colIdx, const float* values, int* rowMap,
                            int* newRowPtr, int* newColIdx, float* newValues) {
    keyed_t* k = (keyed_t*)malloc(sizeof(keyed_t) * (rows > 0 ? rows : 1));
    for (int r = 0; r < rows; ++r) {
        k[r].key = rowPtr[r + 1] - rowPtr[r];
        k[r].id = r;
    }
    qsort(k, rows, sizeof(keyed_t), cmp_keyed);
    newRowPtr[0] = 0;
    int pos = 0;
    for (int i = 0; i < rows; ++i) {
        const int o = k[i].id;
        rowMap[i] = o;
        for (int j = rowPtr[o]; j < rowPtr[o + 1]; ++j) {
            newColIdx[pos] = colIdx[j];
            newValues[pos] = values[j];
            ++pos;
        }
        newRowPtr[i + 1] = pos;
    }
    free(k);
}

void oracle_restore_order_f32(int rows, const float* y_perm, const int* rowMap, float* y) {
    for (int i = 0; i < rows; ++i) y[rowMap[i]] = y_perm[i];
}

typedef struct {
    float key;
    int id;
} fkeyed_t;

/* pair<float,int> ordering (column_reorder.cuh:84-87). */
static int cmp_fkeyed(const void* a, const void* b) {
    const fkeyed_t* x = (const fkeyed_t*)a;
    const fkeyed_t* y = (const fkeyed_t*)b;
    if (x->key < y->key) return -1;
    if (y->key < x->key) return 1;
    return (x->id > y->id) - (x->id < y->id);
}

void oracle_colperm_center_of_mass(int rows, int cols, const int* rowPtr, const int* colIdx, int* forwardMap,
                                   float* key_out) {
    float* com = (float*)calloc(cols > 0 ? cols : 1, sizeof(float));
    int* cnt = (int*)calloc(cols > 0 ? cols : 1, sizeof(int));
    for (int r = 0; r < rows; ++r)
        for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) {
            const int c = colIdx[j];
            com[c] = com[c] + (float)r;
            cnt[c]++;
        }
    fkeyed_t* k = (fkeyed_t*)malloc(sizeof(fkeyed_t) * (cols > 0 ? cols : 1));
    for (int c = 0; c < cols; ++c) {
        if (cnt[c] > 0) com[c] = com[c] / (float)cnt[c];
        k[c].key = com[c];
        k[c].id = c;
        if (key_out) key_out[c] = com[c];
    }
    qsort(k, cols, sizeof(fkeyed_t), cmp_fkeyed);
    for (int i = 0; i < cols; ++i) forwardMap[i] = k[i].id;
    free(k);
    free(cnt);
    free(com);
}

void oracle_colperm_min_row(int rows, int cols, const int* rowPtr, const int* colIdx, int* perm, int* key_out) {
    keyed_t* k = (keyed_t*)malloc(sizeof(keyed_t) * (cols > 0 ? cols : 1));
    for (int c = 0; c < cols; ++c) {
        k[c].key = rows;
        k[c].id = c;
    }
    for (int r = 0; r < rows; ++r)
        for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j)
            if (r < k[colIdx[j]].key) k[colIdx[j]].key = r;
    if (key_out)
        for (int c = 0; c < cols; ++c) key_out[c] = (int)k[c].key;
    qsort(k, cols, sizeof(keyed_t), cmp_keyed);
    for (int i = 0; i < cols; ++i) perm[i] = k[i].id;
    free(k);
}

void oracle_colperm_frequency(int cols, int nnz, const int* colIdx, int* perm, int* key_out) {
    keyed_t* k = (keyed_t*)malloc(sizeof(keyed_t) * (cols > 0 ? cols : 1));
    for (int c = 0; c < cols; ++c) {
        k[c].key = 0;
        k[c].id = c;
    }
    for (int j = 0; j < nnz; ++j) k[colIdx[j]].key++;
    if (key_out)
        for (int c = 0; c < cols; ++c) key_out[c] = (int)k[c].key;
    for (int c = 0; c < cols; ++c) k[c].key = -k[c].key; /* descending count */
    qsort(k, cols, sizeof(keyed_t), cmp_keyed);
    for (int i = 0; i < cols; ++i) perm[i] = k[i].id;
    free(k);
}

void oracle_apply_colperm(int cols, int nnz, const int* perm, const int* colIdx, int* newColIdx) {
    int* inv = (int*)malloc(sizeof(int) * (cols > 0 ? cols : 1));
    for (int i = 0; i < cols; ++i) inv[perm[i]] = i;
    for (int j = 0; j < nnz; ++j) newColIdx[j] = inv[colIdx[j]];
    free(inv);
}

void oracle_permute_x_f32(int cols, const int* forwardMap, const float* x, float* xr) {
    for (int i = 0; i < cols; ++i) xr[i] = x[forwardMap[i]];
}

typedef struct {
    int col;
    float val;
} colval_t;

static int cmp_colval(const void* a, const void* b) {
    const colval_t* x = (const colval_t*)a;
    const colval_t* y = (const colval_t*)b;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    if (x->val < y->val) return -1;
    if (y->val < x->val) return 1;
    return 0;
}

void oracle_sort_within_rows_f32(int rows, const int* rowPtr, int* colIdx, float* values) {
    int cap = 0;
    colval_t* buf = NULL;
    for (int r = 0; r < rows; ++r) {
        const int s = rowPtr[r], len = rowPtr[r + 1] - s;
        if (len > cap) {
            free(buf);
            cap = len;
            buf = (colval_t*)malloc(sizeof(colval_t) * cap);
        }
        for (int i = 0; i < len; ++i) {
            buf[i].col = colIdx[s + i];
            buf[i].val = values[s + i];
        }
        qsort(buf, len, sizeof(colval_t), cmp_colval);
        for (int i = 0; i < len; ++i) {
            colIdx[s + i] = buf[i].col;
            values[s + i] = buf[i].val;
        }
    }
    free(buf);
}

long long oracle_distinct_columns(int cols, long long nnz, const int* colIdx) {
    unsigned char* seen = (unsigned char*)calloc(cols > 0 ? cols : 1, 1);
    long long d = 0;
    for (long long j = 0; j < nnz; ++j) {
        const int c = colIdx[j];
        if (c >= 0 && c < cols && !seen[c]) {
            seen[c] = 1;
            ++d;
        }
    }
    free(seen);
    return d;
}
