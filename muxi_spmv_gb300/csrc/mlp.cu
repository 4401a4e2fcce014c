// The learned kernel selector's network: a 3-layer MLP (in -> h1 -> h2 -> out,
// ReLU) trained on the GPU with hand-written forward, backward and Adam
// kernels.  It maps the 32 matrix features (features.cu) to the predicted
// log slowdown of every variant of the search space (autotune.cu) relative to
// the fastest; the selector picks the smallest prediction.
//
// Parameter order (also the file and get/set order): W1 [h1 x in], b1 [h1],
// W2 [h2 x h1], b2 [h2], W3 [out x h2], b3 [out]; row-major, FP32.
// Loss: masked mean squared error, sum(M*(Y-T)^2) / sum(M).
// Model file: "MXSMLP01", int32 version = 1, int32 in/h1/h2/out, params,
// input mean[in], input std[in], uint64 FNV-1a of every byte before it.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "internal.h"
#include "device.cuh"
#include "kernels.h"
#include "plan.h"

struct spmv_mlp_s {
    int in = 0, h1 = 0, h2 = 0, out = 0;
    int nparams = 0;
    float* params = nullptr;  // device
    float* grads = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* mean = nullptr;  // device, in
    float* stdv = nullptr;
    std::vector<float> hMean, hStd;
    long long step = 0;
    int cap = 0;              // batch capacity of the workspace
    float* work = nullptr;    // activations and deltas
    float* lossAcc = nullptr; // [sum M*(Y-T)^2, sum M]
};

namespace mxs {
namespace {

constexpr int TS = 16;

// C[M x N] = op(A) op(B) (+ bias[n]) (ReLU if relu); row-major; op = transpose
// when the flag is set: op(A)[m,k] = TA ? A[k*lda+m] : A[m*lda+k].
template <bool TA, bool TB>
__global__ void gemm_kernel(int M, int N, int K, const float* __restrict__ A, int lda, const float* __restrict__ B,
                            int ldb, float* __restrict__ C, int ldc, const float* __restrict__ bias, int relu) {
    __shared__ float As[TS][TS + 1];
    __shared__ float Bs[TS][TS + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int m = blockIdx.y * TS + ty, n = blockIdx.x * TS + tx;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += TS) {
        const int ka = k0 + tx, kb = k0 + ty;
        As[ty][tx] = (m < M && ka < K) ? (TA ? A[(long long)ka * lda + m] : A[(long long)m * lda + ka]) : 0.f;
        Bs[ty][tx] = (n < N && kb < K) ? (TB ? B[(long long)n * ldb + kb] : B[(long long)kb * ldb + n]) : 0.f;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < TS; ++k) acc = fmaf(As[ty][k], Bs[k][tx], acc);
        __syncthreads();
    }
    if (m < M && n < N) {
        if (bias) acc += bias[n];
        if (relu) acc = fmaxf(acc, 0.f);
        C[(long long)m * ldc + n] = acc;
    }
}

template <bool TA, bool TB>
void gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc, const float* bias,
          bool relu, cudaStream_t s) {
    dim3 blk(TS, TS), grd((N + TS - 1) / TS, (M + TS - 1) / TS);
    gemm_kernel<TA, TB><<<grd, blk, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu ? 1 : 0);
}

__global__ void normalize_kernel(int B, int I, const float* __restrict__ X, const float* __restrict__ mean,
                                 const float* __restrict__ sd, float* __restrict__ Xn) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)B * I) return;
    const int i = (int)(t % I);
    Xn[t] = (X[t] - mean[i]) / sd[i];
}

__global__ void loss_kernel(int n, const float* __restrict__ Y, const float* __restrict__ T,
                            const float* __restrict__ Mk, float* __restrict__ acc) {
    float se = 0.f, cnt = 0.f;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const float d = Y[t] - T[t];
        se += Mk[t] * d * d;
        cnt += Mk[t];
    }
    for (int off = 16; off > 0; off >>= 1) {
        se += __shfl_xor_sync(kFull, se, off);
        cnt += __shfl_xor_sync(kFull, cnt, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc, se);
        atomicAdd(acc + 1, cnt);
    }
}

__global__ void dloss_kernel(int n, const float* __restrict__ Y, const float* __restrict__ T,
                             const float* __restrict__ Mk, const float* __restrict__ acc, float* __restrict__ dY) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float cnt = acc[1] > 0.f ? acc[1] : 1.f;
    dY[t] = 2.f * Mk[t] * (Y[t] - T[t]) / cnt;
}

// db[o] = sum_b dZ[b, o]
__global__ void colsum_kernel(int B, int O, const float* __restrict__ dZ, float* __restrict__ db) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= O) return;
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += dZ[(long long)b * O + o];
    db[o] = s;
}

// dA *= (A > 0): ReLU backward through the stored activation.
__global__ void relu_back_kernel(long long n, const float* __restrict__ A, float* __restrict__ dA) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n && A[t] <= 0.f) dA[t] = 0.f;
}

__global__ void adam_kernel(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.f - b1) * gt;
    const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

struct Views {
    float *W1, *b1, *W2, *b2, *W3, *b3;
};
Views views(const spmv_mlp_s* n, float* base) {
    Views w;
    w.W1 = base;
    w.b1 = w.W1 + (size_t)n->h1 * n->in;
    w.W2 = w.b1 + n->h1;
    w.b2 = w.W2 + (size_t)n->h2 * n->h1;
    w.W3 = w.b2 + n->h2;
    w.b3 = w.W3 + (size_t)n->out * n->h2;
    return w;
}

struct Work {
    float *Xn, *A1, *A2, *Y, *dY, *dA2, *dA1;
};

spmv_status_t ensure_work(spmv_mlp_s* n, int B, Work& w) {
    const size_t per = (size_t)n->in + n->h1 + n->h2 + 2 * (size_t)n->out + n->h2 + n->h1;
    if (B > n->cap) {
        if (n->work) dev_free(n->work);
        n->work = nullptr;
        n->cap = 0;
        MXS_CUDA(dev_malloc(&n->work, sizeof(float) * per * (size_t)B));
        n->cap = B;
    }
    float* p = n->work;
    w.Xn = p;
    p += (size_t)B * n->in;
    w.A1 = p;
    p += (size_t)B * n->h1;
    w.A2 = p;
    p += (size_t)B * n->h2;
    w.Y = p;
    p += (size_t)B * n->out;
    w.dY = p;
    p += (size_t)B * n->out;
    w.dA2 = p;
    p += (size_t)B * n->h2;
    w.dA1 = p;
    return SPMV_SUCCESS;
}

spmv_status_t forward(spmv_mlp_s* n, const float* X, int B, Work& w, float* Yout, cudaStream_t s) {
    const Views P = views(n, n->params);
    const long long ni = (long long)B * n->in;
    normalize_kernel<<<grid_for(ni, 256), 256, 0, s>>>(B, n->in, X, n->mean, n->stdv, w.Xn);
    gemm<false, true>(B, n->h1, n->in, w.Xn, n->in, P.W1, n->in, w.A1, n->h1, P.b1, true, s);
    gemm<false, true>(B, n->h2, n->h1, w.A1, n->h1, P.W2, n->h1, w.A2, n->h2, P.b2, true, s);
    gemm<false, true>(B, n->out, n->h2, w.A2, n->h2, P.W3, n->h2, Yout, n->out, P.b3, false, s);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

// Fills n->grads for the batch and accumulates the loss in n->lossAcc.
spmv_status_t backward(spmv_mlp_s* n, const float* X, const float* T, const float* Mk, int B, cudaStream_t s) {
    (void)X;
    Work w;
    MXS_TRY(ensure_work(n, B, w));
    MXS_TRY(forward(n, X, B, w, w.Y, s));
    const Views P = views(n, n->params), G = views(n, n->grads);
    const int no = B * n->out;
    MXS_CUDA(cudaMemsetAsync(n->lossAcc, 0, 2 * sizeof(float), s));
    loss_kernel<<<grid_for(no, 256) < 64u ? grid_for(no, 256) : 64u, 256, 0, s>>>(no, w.Y, T, Mk, n->lossAcc);
    dloss_kernel<<<grid_for(no, 256), 256, 0, s>>>(no, w.Y, T, Mk, n->lossAcc, w.dY);
    // layer 3: dW3 = dY^T A2, db3 = colsum dY, dA2 = dY W3
    gemm<true, false>(n->out, n->h2, B, w.dY, n->out, w.A2, n->h2, G.W3, n->h2, nullptr, false, s);
    colsum_kernel<<<grid_for(n->out, 128), 128, 0, s>>>(B, n->out, w.dY, G.b3);
    gemm<false, false>(B, n->h2, n->out, w.dY, n->out, P.W3, n->h2, w.dA2, n->h2, nullptr, false, s);
    relu_back_kernel<<<grid_for((long long)B * n->h2, 256), 256, 0, s>>>((long long)B * n->h2, w.A2, w.dA2);
    // layer 2
    gemm<true, false>(n->h2, n->h1, B, w.dA2, n->h2, w.A1, n->h1, G.W2, n->h1, nullptr, false, s);
    colsum_kernel<<<grid_for(n->h2, 128), 128, 0, s>>>(B, n->h2, w.dA2, G.b2);
    gemm<false, false>(B, n->h1, n->h2, w.dA2, n->h2, P.W2, n->h1, w.dA1, n->h1, nullptr, false, s);
    relu_back_kernel<<<grid_for((long long)B * n->h1, 256), 256, 0, s>>>((long long)B * n->h1, w.A1, w.dA1);
    // layer 1 (input gradient not needed)
    gemm<true, false>(n->h1, n->in, B, w.dA1, n->h1, w.Xn, n->in, G.W1, n->in, nullptr, false, s);
    colsum_kernel<<<grid_for(n->h1, 128), 128, 0, s>>>(B, n->h1, w.dA1, G.b1);
    MXS_LAUNCH_CHECK();
    return SPMV_SUCCESS;
}

unsigned long long fnv1a(const void* p, size_t n, unsigned long long h = 1469598103934665603ULL) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ULL;
    }
    return h;
}

spmv_status_t upload_norm(spmv_mlp_s* n) {
    MXS_CUDA(cudaMemcpy(n->mean, n->hMean.data(), sizeof(float) * n->in, cudaMemcpyHostToDevice));
    MXS_CUDA(cudaMemcpy(n->stdv, n->hStd.data(), sizeof(float) * n->in, cudaMemcpyHostToDevice));
    return SPMV_SUCCESS;
}

}  // namespace

// Used by the selector (select.cu): outputs for one feature vector (device).
spmv_status_t mlp_predict_one(spmv_mlp_t n, const float* dX, float* hY, cudaStream_t s) {
    Work w;
    MXS_TRY(ensure_work(n, 1, w));
    MXS_TRY(forward(n, dX, 1, w, w.Y, s));
    MXS_CUDA(cudaMemcpyAsync(hY, w.Y, sizeof(float) * n->out, cudaMemcpyDeviceToHost, s));
    MXS_CUDA(cudaStreamSynchronize(s));
    return SPMV_SUCCESS;
}

int mlp_outputs(spmv_mlp_t n) { return n ? n->out : 0; }
int mlp_inputs(spmv_mlp_t n) { return n ? n->in : 0; }

}  // namespace mxs

using namespace mxs;

extern "C" {

spmv_status_t spmv_mlp_destroy(spmv_mlp_t n) {
    clear_error();
    if (!n) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "model is NULL");
    dev_free(n->params);
    dev_free(n->grads);
    dev_free(n->m);
    dev_free(n->v);
    dev_free(n->mean);
    dev_free(n->stdv);
    dev_free(n->work);
    dev_free(n->lossAcc);
    delete n;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_create(int in, int h1, int h2, int out, unsigned long long seed, spmv_mlp_t* outp) {
    clear_error();
    if (!outp) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "output is NULL");
    *outp = nullptr;
    if (in <= 0 || h1 <= 0 || h2 <= 0 || out <= 0 || in > 4096 || h1 > 4096 || h2 > 4096 || out > 4096)
        MXS_FAIL(SPMV_ERROR_INVALID_MATRIX, "layer sizes must be in [1, 4096]");
    spmv_mlp_s* n = new (std::nothrow) spmv_mlp_s();
    if (!n) MXS_FAIL(SPMV_ERROR_MEMORY_ALLOC, "out of host memory");
    n->in = in;
    n->h1 = h1;
    n->h2 = h2;
    n->out = out;
    n->nparams = h1 * in + h1 + h2 * h1 + h2 + out * h2 + out;
    const size_t pb = sizeof(float) * n->nparams;
    cudaError_t e = dev_malloc(&n->params, pb);
    if (e == cudaSuccess) e = dev_malloc(&n->grads, pb);
    if (e == cudaSuccess) e = dev_malloc(&n->m, pb);
    if (e == cudaSuccess) e = dev_malloc(&n->v, pb);
    if (e == cudaSuccess) e = dev_malloc(&n->mean, sizeof(float) * in);
    if (e == cudaSuccess) e = dev_malloc(&n->stdv, sizeof(float) * in);
    if (e == cudaSuccess) e = dev_malloc(&n->lossAcc, 2 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(n->m, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(n->v, 0, pb);
    if (e != cudaSuccess) {
        spmv_mlp_destroy(n);
        return cuda_fail(e, "model allocation", __FILE__, __LINE__);
    }
    // He-uniform initialisation from a seeded host generator; biases zero.
    std::vector<float> h(n->nparams, 0.f);
    std::mt19937_64 rng(seed);
    auto initW = [&](size_t off, int rows, int cols) {
        const float lim = std::sqrt(6.f / (float)cols);
        for (size_t i = 0; i < (size_t)rows * cols; ++i)
            h[off + i] = ((float)((rng() >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f) * lim;
    };
    size_t off = 0;
    initW(off, h1, in);
    off += (size_t)h1 * in + h1;
    initW(off, h2, h1);
    off += (size_t)h2 * h1 + h2;
    initW(off, out, h2);
    n->hMean.assign(in, 0.f);
    n->hStd.assign(in, 1.f);
    e = cudaMemcpy(n->params, h.data(), pb, cudaMemcpyHostToDevice);
    if (e != cudaSuccess || upload_norm(n) != SPMV_SUCCESS) {
        spmv_mlp_destroy(n);
        return cuda_fail(e == cudaSuccess ? cudaErrorUnknown : e, "model init", __FILE__, __LINE__);
    }
    *outp = n;
    return SPMV_SUCCESS;
}

int spmv_mlp_num_params(spmv_mlp_t n) { return n ? n->nparams : 0; }

spmv_status_t spmv_mlp_shape(spmv_mlp_t n, int* in, int* h1, int* h2, int* out) {
    clear_error();
    if (!n) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "model is NULL");
    if (in) *in = n->in;
    if (h1) *h1 = n->h1;
    if (h2) *h2 = n->h2;
    if (out) *out = n->out;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_get_params(spmv_mlp_t n, float* host, int count) {
    clear_error();
    if (!n || !host || count != n->nparams) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "bad parameter buffer");
    MXS_CUDA(cudaMemcpy(host, n->params, sizeof(float) * count, cudaMemcpyDeviceToHost));
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_set_params(spmv_mlp_t n, const float* host, int count) {
    clear_error();
    if (!n || !host || count != n->nparams) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "bad parameter buffer");
    MXS_CUDA(cudaMemcpy(n->params, host, sizeof(float) * count, cudaMemcpyHostToDevice));
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_set_normalization(spmv_mlp_t n, const float* mean, const float* sd) {
    clear_error();
    if (!n || !mean || !sd) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    for (int i = 0; i < n->in; ++i) {
        n->hMean[i] = mean[i];
        n->hStd[i] = sd[i] > 1e-6f ? sd[i] : 1.f;
    }
    return upload_norm(n);
}

spmv_status_t spmv_mlp_forward(spmv_mlp_t n, const float* X, float* Y, int batch, cudaStream_t s) {
    clear_error();
    if (!n) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "model is NULL");
    if (batch <= 0) return SPMV_SUCCESS;
    if (!X || !Y) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    Work w;
    MXS_TRY(ensure_work(n, batch, w));
    return forward(n, X, batch, w, Y, s);
}

spmv_status_t spmv_mlp_gradients(spmv_mlp_t n, const float* X, const float* T, const float* M, int batch,
                                 float* loss, float* grads, cudaStream_t s) {
    clear_error();
    if (!n) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "model is NULL");
    if (batch <= 0 || !X || !T || !M) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "bad batch");
    MXS_TRY(backward(n, X, T, M, batch, s));
    float acc[2] = {0.f, 0.f};
    MXS_CUDA(cudaMemcpyAsync(acc, n->lossAcc, sizeof(acc), cudaMemcpyDeviceToHost, s));
    if (grads) MXS_CUDA(cudaMemcpyAsync(grads, n->grads, sizeof(float) * n->nparams, cudaMemcpyDeviceToHost, s));
    MXS_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = acc[1] > 0.f ? acc[0] / acc[1] : 0.f;
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_train_step(spmv_mlp_t n, const float* X, const float* T, const float* M, int batch, float lr,
                                  float* loss, cudaStream_t s) {
    clear_error();
    if (!n) MXS_FAIL(SPMV_ERROR_INVALID_HANDLE, "model is NULL");
    if (batch <= 0 || !X || !T || !M) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "bad batch");
    MXS_TRY(backward(n, X, T, M, batch, s));
    ++n->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
    adam_kernel<<<grid_for(n->nparams, 256), 256, 0, s>>>(n->nparams, n->params, n->grads, n->m, n->v, lr, b1, b2,
                                                         1e-8f, c1, c2);
    MXS_LAUNCH_CHECK();
    if (loss) {
        float acc[2] = {0.f, 0.f};
        MXS_CUDA(cudaMemcpyAsync(acc, n->lossAcc, sizeof(acc), cudaMemcpyDeviceToHost, s));
        MXS_CUDA(cudaStreamSynchronize(s));
        *loss = acc[1] > 0.f ? acc[0] / acc[1] : 0.f;
    }
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_save(spmv_mlp_t n, const char* path) {
    clear_error();
    if (!n || !path) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    std::vector<unsigned char> buf;
    auto put = [&](const void* p, size_t b) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        buf.insert(buf.end(), c, c + b);
    };
    std::vector<float> h(n->nparams);
    MXS_CUDA(cudaMemcpy(h.data(), n->params, sizeof(float) * n->nparams, cudaMemcpyDeviceToHost));
    const int hdr[5] = {1, n->in, n->h1, n->h2, n->out};
    put("MXSMLP01", 8);
    put(hdr, sizeof(hdr));
    put(h.data(), sizeof(float) * h.size());
    put(n->hMean.data(), sizeof(float) * n->in);
    put(n->hStd.data(), sizeof(float) * n->in);
    const unsigned long long sum = fnv1a(buf.data(), buf.size());
    put(&sum, sizeof(sum));
    FILE* f = std::fopen(path, "wb");
    if (!f) MXS_FAIL(SPMV_ERROR_INTERNAL, "cannot open %s for writing", path);
    const size_t w = std::fwrite(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    if (w != buf.size()) MXS_FAIL(SPMV_ERROR_INTERNAL, "short write to %s", path);
    return SPMV_SUCCESS;
}

spmv_status_t spmv_mlp_load(const char* path, spmv_mlp_t* outp) {
    clear_error();
    if (!path || !outp) MXS_FAIL(SPMV_ERROR_INVALID_VECTOR, "NULL argument");
    *outp = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) MXS_FAIL(SPMV_ERROR_INTERNAL, "cannot open %s", path);
    std::vector<unsigned char> buf;
    unsigned char tmp[65536];
    size_t r;
    while ((r = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
    std::fclose(f);
    const size_t head = 8 + 5 * sizeof(int);
    if (buf.size() < head + sizeof(unsigned long long) || std::memcmp(buf.data(), "MXSMLP01", 8) != 0)
        MXS_FAIL(SPMV_ERROR_INTERNAL, "%s is not a selector model (bad magic or truncated)", path);
    int hdr[5];
    std::memcpy(hdr, buf.data() + 8, sizeof(hdr));
    if (hdr[0] != 1) MXS_FAIL(SPMV_ERROR_INTERNAL, "%s: unsupported model version %d", path, hdr[0]);
    for (int i = 1; i < 5; ++i)
        if (hdr[i] <= 0 || hdr[i] > 4096) MXS_FAIL(SPMV_ERROR_INTERNAL, "%s: bad layer size", path);
    const long long np = (long long)hdr[2] * hdr[1] + hdr[2] + (long long)hdr[3] * hdr[2] + hdr[3] +
                         (long long)hdr[4] * hdr[3] + hdr[4];
    const size_t need = head + sizeof(float) * (np + 2 * (size_t)hdr[1]) + sizeof(unsigned long long);
    if (buf.size() != need) MXS_FAIL(SPMV_ERROR_INTERNAL, "%s: truncated or oversized model file", path);
    unsigned long long sum;
    std::memcpy(&sum, buf.data() + need - sizeof(sum), sizeof(sum));
    if (fnv1a(buf.data(), need - sizeof(sum)) != sum) MXS_FAIL(SPMV_ERROR_INTERNAL, "%s: checksum mismatch", path);
    spmv_mlp_t n = nullptr;
    MXS_TRY(spmv_mlp_create(hdr[1], hdr[2], hdr[3], hdr[4], 0, &n));
    const float* p = reinterpret_cast<const float*>(buf.data() + head);
    spmv_status_t st = spmv_mlp_set_params(n, p, (int)np);
    if (st == SPMV_SUCCESS) st = spmv_mlp_set_normalization(n, p + np, p + np + hdr[1]);
    if (st != SPMV_SUCCESS) {
        spmv_mlp_destroy(n);
        return st;
    }
    *outp = n;
    return SPMV_SUCCESS;
}

}  // extern "C"
