// Multilayer perceptron of the parameter tuner: forward pass, mean-squared-
// error gradients and Adam updates as hand-written CUDA kernels (FP32).
//
// Network: in -> hidden (ReLU) -> ... (hiddenLayers times) -> out, every
// layer y = x W^T + b with W stored row-major [outDim][inDim]. Parameters
// are one flat array: for each layer W then b. The tuner's network is small
// (32 inputs, 3 x 128 hidden, 1 output) and its batches are a few thousand
// rows, so every product is a few million multiply-adds: one tiled FP32
// kernel (32 x 32 output tile, 16-deep k slices in shared memory) serves the
// forward product (X W^T), the data gradient (dY W) and the weight gradient
// (dY^T X), with the bias, ReLU and ReLU-mask epilogues fused. Each output
// sums its k terms in order with fmaf, so results do not depend on the grid.
// The loss reduction runs in one block in a fixed order (deterministic).
#include <algorithm>
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"

namespace race {

namespace {

constexpr int kT = 32;   // output tile
constexpr int kK = 16;   // k slice

enum Epilogue { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_RELU = 2, EPI_RELU_MASK = 3 };

// C[M][N] = op(A)[M][K] op(B)[K][N]; op(A)[m][k] = TA ? A[k*lda+m] : A[m*lda+k],
// op(B)[k][n] = TB ? B[n*ldb+k] : B[k*ldb+n]. Epilogues: + bias[n]; + bias
// then ReLU; multiply by (mask[m*ldc+n] > 0) (gradient through a ReLU whose
// output is mask).
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) kGemm(int M, int N, int K, const float *__restrict__ A, int lda,
                                             const float *__restrict__ B, int ldb, float *__restrict__ C, int ldc,
                                             int epi, const float *__restrict__ bias, const float *__restrict__ mask) {
    __shared__ float sA[kK][kT + 1];
    __shared__ float sB[kK][kT + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 16 x 16 threads, 2 x 2 outputs each
    const int m0 = blockIdx.y * kT, n0 = blockIdx.x * kT;
    float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int k0 = 0; k0 < K; k0 += kK) {
        for (int i = threadIdx.x; i < kK * kT; i += 256) {
            const int kk = i / kT, mm = i % kT;
            const int m = m0 + mm, k = k0 + kk;
            sA[kk][mm] = (m < M && k < K) ? (TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : 0.f;
            const int n = n0 + mm;
            sB[kk][mm] = (n < N && k < K) ? (TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]) : 0.f;
        }
        __syncthreads();
        const int kEnd = min(kK, K - k0);
        for (int kk = 0; kk < kEnd; ++kk) {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) acc[i][j] = fmaf(sA[kk][ty + 16 * i], sB[kk][tx + 16 * j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j];
            if (epi == EPI_BIAS || epi == EPI_BIAS_RELU) v += bias[n];
            if (epi == EPI_BIAS_RELU) v = fmaxf(v, 0.f);
            if (epi == EPI_RELU_MASK && !(mask[(size_t)m * ldc + n] > 0.f)) v = 0.f;
            C[(size_t)m * ldc + n] = v;
        }
}

// db[n] = sum_m dY[m][n], in order of m.
__global__ void kColSum(int M, int N, const float *__restrict__ dY, float *__restrict__ db) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += dY[(size_t)m * N + n];
    db[n] = s;
}

// Mean squared error over B x O outputs: loss = sum (y-t)^2 / (B O);
// dY = 2 (y - t) / (B O). One block, fixed reduction order.
__global__ void __launch_bounds__(256) kMse(int count, const float *__restrict__ y, const float *__restrict__ t,
                                            float *__restrict__ dY, float *__restrict__ loss) {
    __shared__ float part[256];
    float s = 0.f;
    const float scale = 2.f / (float)count;
    for (int i = threadIdx.x; i < count; i += 256) {
        const float d = y[i] - t[i];
        dY[i] = scale * d;
        s = fmaf(d, d, s);
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = part[0] / (float)count;
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void kAdam(long long n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                      float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

template <bool TA, bool TB>
void gemm(cudaStream_t s, int M, int N, int K, const float *A, int lda, const float *B, int ldb, float *C, int ldc,
          int epi, const float *bias, const float *mask) {
    dim3 grid(ceilDiv(N, kT), ceilDiv(M, kT));
    kGemm<TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, epi, bias, mask);
    RACE_CUDA(cudaGetLastError());
}

}  // namespace

struct Mlp {
    int in = 0, hidden = 0, hiddenLayers = 0, out = 0;
    std::vector<int> dimIn, dimOut;
    std::vector<size_t> wOff, bOff;
    size_t numParams = 0;
    DevBuf<float> params, grads, m1, m2;
    DevBuf<float> acts, deltas, lossBuf;  // activations per layer, gradient workspace
    int batchCap = 0;
    long long steps = 0;

    Mlp(int in_, int hidden_, int layers_, int out_) : in(in_), hidden(hidden_), hiddenLayers(layers_), out(out_) {
        if (in < 1 || hidden < 1 || layers_ < 1 || out < 1) throw Error(RACE_ERR_INVALID_ARG, "bad MLP shape");
        for (int l = 0; l <= hiddenLayers; ++l) {
            dimIn.push_back(l == 0 ? in : hidden);
            dimOut.push_back(l == hiddenLayers ? out : hidden);
            wOff.push_back(numParams);
            numParams += (size_t)dimIn.back() * dimOut.back();
            bOff.push_back(numParams);
            numParams += dimOut.back();
        }
        params.alloc(numParams);
        grads.alloc(numParams);
        m1.alloc(numParams);
        m2.alloc(numParams);
        lossBuf.alloc(1);
        RACE_CUDA(cudaMemset(params.p, 0, sizeof(float) * numParams));
        RACE_CUDA(cudaMemset(m1.p, 0, sizeof(float) * numParams));
        RACE_CUDA(cudaMemset(m2.p, 0, sizeof(float) * numParams));
    }
    int layers() const { return hiddenLayers + 1; }
    // activation l (l = 1..layers) of a batch row: output of layer l-1
    size_t actOff(int l, int B) const {
        size_t o = 0;
        for (int i = 1; i < l; ++i) o += (size_t)B * dimOut[i - 1];
        return o;
    }
    void ensure(int B) {
        if (B <= batchCap) return;
        size_t total = 0, widest = 0;
        for (int l = 0; l < layers(); ++l) {
            total += (size_t)B * dimOut[l];
            widest = std::max(widest, (size_t)B * std::max(dimOut[l], dimIn[l]));
        }
        acts.alloc(total);
        deltas.alloc(2 * widest);
        batchCap = B;
    }
    // forward: activations of every layer into acts; returns the output pointer
    float *forward(const float *X, int B, cudaStream_t s) {
        ensure(B);
        const float *x = X;
        for (int l = 0; l < layers(); ++l) {
            float *y = acts.p + actOff(l + 1, B);
            const bool last = l == layers() - 1;
            gemm<false, true>(s, B, dimOut[l], dimIn[l], x, dimIn[l], params.p + wOff[l], dimIn[l], y, dimOut[l],
                              last ? EPI_BIAS : EPI_BIAS_RELU, params.p + bOff[l], nullptr);
            x = y;
        }
        return acts.p + actOff(layers(), B);
    }
    // loss and gradients of the MSE against targets T (B x out)
    void lossGrad(const float *X, const float *T, int B, cudaStream_t s) {
        float *y = forward(X, B, s);
        float *d = deltas.p, *dNext = deltas.p + deltas.n / 2;
        kMse<<<1, 256, 0, s>>>(B * out, y, T, d, lossBuf.p);
        RACE_CUDA(cudaGetLastError());
        for (int l = layers() - 1; l >= 0; --l) {
            const float *xin = l == 0 ? X : acts.p + actOff(l, B);
            // dW = d^T xin  [out_l x in_l], db = column sums of d
            gemm<true, false>(s, dimOut[l], dimIn[l], B, d, dimOut[l], xin, dimIn[l], grads.p + wOff[l], dimIn[l],
                              EPI_NONE, nullptr, nullptr);
            kColSum<<<ceilDiv(dimOut[l], 128), 128, 0, s>>>(B, dimOut[l], d, grads.p + bOff[l]);
            RACE_CUDA(cudaGetLastError());
            if (l > 0) {
                // d_prev = (d W) * (xin > 0): xin is the ReLU output of layer l-1
                gemm<false, false>(s, B, dimIn[l], dimOut[l], d, dimOut[l], params.p + wOff[l], dimIn[l], dNext,
                                   dimIn[l], EPI_RELU_MASK, nullptr, xin);
                std::swap(d, dNext);
            }
        }
    }
    void adam(float lr, float b1, float b2, float eps, cudaStream_t s) {
        ++steps;
        const float c1 = 1.f - std::pow(b1, (float)steps), c2 = 1.f - std::pow(b2, (float)steps);
        kAdam<<<ceilDiv((long long)numParams, 256), 256, 0, s>>>((long long)numParams, params.p, grads.p, m1.p, m2.p,
                                                                lr, b1, b2, eps, c1, c2);
        RACE_CUDA(cudaGetLastError());
    }
};

}  // namespace race

struct race_mlp {
    std::unique_ptr<race::Mlp> net;
    std::string err;
};

namespace {
template <typename F>
int guardMlp(race_mlp *h, F &&f) {
    try {
        f();
        return RACE_SUCCESS;
    } catch (const race::Error &ex) {
        if (h) h->err = ex.what();
        return ex.code;
    } catch (const std::exception &ex) {
        if (h) h->err = ex.what();
        return RACE_ERR_INTERNAL;
    }
}
}  // namespace

extern "C" {

int race_mlp_create(race_mlp **out, int in, int hidden, int hiddenLayers, int outDim) {
    if (!out) return RACE_ERR_INVALID_ARG;
    *out = nullptr;
    race_mlp *h = new race_mlp;
    int rc = guardMlp(h, [&] { h->net = std::make_unique<race::Mlp>(in, hidden, hiddenLayers, outDim); });
    if (rc != RACE_SUCCESS) {
        delete h;
        return rc;
    }
    *out = h;
    return RACE_SUCCESS;
}

int race_mlp_destroy(race_mlp *h) {
    delete h;
    return RACE_SUCCESS;
}

int race_mlp_num_params(race_mlp *h, long long *count) {
    if (!h || !count) return RACE_ERR_INVALID_ARG;
    *count = (long long)h->net->numParams;
    return RACE_SUCCESS;
}

int race_mlp_set_params(race_mlp *h, const float *host, long long count) {
    if (!h || !host || count != (long long)h->net->numParams) return RACE_ERR_INVALID_ARG;
    return guardMlp(h, [&] {
        RACE_CUDA(cudaMemcpy(h->net->params.p, host, sizeof(float) * count, cudaMemcpyHostToDevice));
        RACE_CUDA(cudaMemset(h->net->m1.p, 0, sizeof(float) * count));
        RACE_CUDA(cudaMemset(h->net->m2.p, 0, sizeof(float) * count));
        h->net->steps = 0;
    });
}

int race_mlp_get_params(race_mlp *h, float *host, long long count) {
    if (!h || !host || count != (long long)h->net->numParams) return RACE_ERR_INVALID_ARG;
    return guardMlp(h, [&] {
        RACE_CUDA(cudaMemcpy(host, h->net->params.p, sizeof(float) * count, cudaMemcpyDeviceToHost));
    });
}

int race_mlp_forward(race_mlp *h, const float *X, int batch, float *Y, void *stream) {
    if (!h || !X || !Y || batch < 1) return RACE_ERR_INVALID_ARG;
    return guardMlp(h, [&] {
        cudaStream_t s = (cudaStream_t)stream;
        float *y = h->net->forward(X, batch, s);
        RACE_CUDA(cudaMemcpyAsync(Y, y, sizeof(float) * batch * h->net->out, cudaMemcpyDeviceToDevice, s));
    });
}

int race_mlp_loss_grad(race_mlp *h, const float *X, const float *T, int batch, float *loss_host, float *grad_host,
                       void *stream) {
    if (!h || !X || !T || batch < 1) return RACE_ERR_INVALID_ARG;
    return guardMlp(h, [&] {
        cudaStream_t s = (cudaStream_t)stream;
        h->net->lossGrad(X, T, batch, s);
        if (loss_host) RACE_CUDA(cudaMemcpyAsync(loss_host, h->net->lossBuf.p, sizeof(float), cudaMemcpyDeviceToHost, s));
        if (grad_host)
            RACE_CUDA(cudaMemcpyAsync(grad_host, h->net->grads.p, sizeof(float) * h->net->numParams,
                                      cudaMemcpyDeviceToHost, s));
        if (loss_host || grad_host) RACE_CUDA(cudaStreamSynchronize(s));
    });
}

int race_mlp_adam_step(race_mlp *h, float lr, float beta1, float beta2, float eps, void *stream) {
    if (!h || !(lr > 0.f)) return RACE_ERR_INVALID_ARG;
    return guardMlp(h, [&] { h->net->adam(lr, beta1, beta2, eps, (cudaStream_t)stream); });
}

const char *race_mlp_last_error(race_mlp *h) { return h ? h->err.c_str() : "null network"; }

}  // extern "C"
