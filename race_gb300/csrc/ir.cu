// Mixed-precision symmetric Gauss-Seidel with FP64 iterative refinement.
//
// The reference's Gauss-Seidel drivers iterate forward + backward sweeps in
// FP64 and check the residual every few iterations (examples/src/
// colorSymmGS.cpp:31-99, 147-267). Here the sweeps run on an inner problem
// A d = r whose matrix values are stored in FP32 or BF16 and whose vectors
// are FP32 (accumulation in FP32), while the residual r = b - A x and the
// update x += d stay in FP64 on the GPU:
//
//   repeat: r = b - A x (FP64), stop if ||r|| <= tol ||b||
//           d = 0; `sweeps` times: GS forward, GS backward on (A32, d, r32)
//           x = x + d (FP64)
//
// The inner function is a registered RACE_K_GS function (its operands name
// the FP32 d and r buffers), so the sweeps use RACE's coloring and the wave
// plan like any other call. With an FP64 inner function the same loop is the
// plain FP64 symmetric Gauss-Seidel iteration (one symmetric sweep from the
// current x equals x plus one symmetric sweep on the residual equation).
#include "engine.h"

namespace race {

namespace {

constexpr int kThreads = 256;

// r = b - A x (FP64 fma chain per row), r32 = (float) r or r64 copy, and
// sum of r^2 into *acc.
template <bool F32>
__global__ void __launch_bounds__(kThreads) kResidual(int n, const int *__restrict__ rowPtr,
                                                      const int *__restrict__ col, const double *__restrict__ val,
                                                      const double *__restrict__ b, const double *__restrict__ x,
                                                      void *rOut, double *acc) {
    __shared__ double sm[kThreads / 32];
    double local = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double t = b[r];
        for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) t = fma(-val[j], x[col[j]], t);
        if (F32)
            ((float *)rOut)[r] = (float)t;
        else
            ((double *)rOut)[r] = t;
        local = fma(t, t, local);
    }
    for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += sm[w];
        atomicAdd(acc, s);
    }
}

__global__ void kSumSq(int n, const double *__restrict__ v, double *acc) {
    __shared__ double sm[kThreads / 32];
    double local = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) local = fma(v[i], v[i], local);
    for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += sm[w];
        atomicAdd(acc, s);
    }
}

template <bool F32>
__global__ void kUpdate(int n, double *__restrict__ x, const void *d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += F32 ? (double)((const float *)d)[i] : ((const double *)d)[i];
}

}  // namespace

void symmGsIr(Engine &e, int inner, int n, const int *rowPtr, const int *col, const double *val, const double *b,
              double *x, double tol, int maxIter, int sweeps, int *itersOut, double *relresOut) {
    if (inner < 0 || inner >= (int)e.funcs.size()) throw Error(RACE_ERR_INVALID_ARG, "unknown inner function");
    FuncEntry &f = e.funcs[inner];
    if (f.kernel != RACE_K_GS) throw Error(RACE_ERR_INVALID_ARG, "inner function must be RACE_K_GS");
    if (f.ops.n != n) throw Error(RACE_ERR_INVALID_ARG, "size mismatch");
    const bool f32 = f.ops.vec_type == RACE_VAL_F32;
    cudaStream_t s = e.stream;
    DevBuf<double> acc(2);
    int dev = 0, sms = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = std::min(ceilDiv(n, kThreads), sms * 8);
    RACE_CUDA(cudaMemsetAsync(acc.p, 0, 2 * sizeof(double), s));
    kSumSq<<<blocks, kThreads, 0, s>>>(n, b, acc.p + 1);
    double bn2 = 0;
    RACE_CUDA(cudaMemcpyAsync(&bn2, acc.p + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    const double bnorm = std::sqrt(bn2) > 0 ? std::sqrt(bn2) : 1.0;
    const size_t vb = f32 ? sizeof(float) : sizeof(double);
    int it = 0;
    double rel = 0;
    for (;;) {
        RACE_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(double), s));
        if (f32)
            kResidual<true><<<blocks, kThreads, 0, s>>>(n, rowPtr, col, val, b, x, f.ops.b, acc.p);
        else
            kResidual<false><<<blocks, kThreads, 0, s>>>(n, rowPtr, col, val, b, x, f.ops.b, acc.p);
        double rn2 = 0;
        RACE_CUDA(cudaMemcpyAsync(&rn2, acc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        RACE_CUDA(cudaStreamSynchronize(s));
        rel = std::sqrt(rn2) / bnorm;
        if (rel <= tol || it >= maxIter || !std::isfinite(rel)) break;
        RACE_CUDA(cudaMemsetAsync(f.ops.x, 0, vb * n, s));
        for (int k = 0; k < sweeps; ++k) {
            e.launch(inner, false);
            e.launch(inner, true);
        }
        if (f32)
            kUpdate<true><<<ceilDiv(n, kThreads), kThreads, 0, s>>>(n, x, f.ops.x);
        else
            kUpdate<false><<<ceilDiv(n, kThreads), kThreads, 0, s>>>(n, x, f.ops.x);
        RACE_CUDA(cudaGetLastError());
        ++it;
    }
    e.checkStatus();
    *itersOut = it;
    *relresOut = rel;
}

}  // namespace race
