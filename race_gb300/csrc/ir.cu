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
#include <algorithm>
#include <vector>

#include "engine.h"

namespace race {

namespace {

constexpr int kThreads = 256;

// r = b - A x in FP64. Rows of at most kShortRow entries: one thread, one
// fma chain in CRS order. Longer rows (hubs of power-law graphs; one reaches
// a quarter of a million entries) would make one thread's dependent gather
// chain the whole kernel's duration: they are cut into segments of at most
// kSegLen entries, each summed by a warp (kSegDot), and combined per row in
// segment order (kResidualLong); their sums are reassociated. The squared
// norm is reduced per block in a fixed order and then by one block
// (kFinalSum), so the refinement is deterministic run to run.
constexpr int kShortRow = 32;
constexpr int kSegLen = 1024;

__device__ __forceinline__ double blockSum(double v, double *sm) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; ++w) s += sm[w];
    return s;
}

template <bool F32>
__global__ void __launch_bounds__(kThreads) kResidualShort(int n, const int *__restrict__ rowPtr,
                                                           const int *__restrict__ col,
                                                           const double *__restrict__ val,
                                                           const double *__restrict__ b,
                                                           const double *__restrict__ x, void *rOut, double *part) {
    __shared__ double sm[kThreads / 32];
    double local = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int s0 = rowPtr[r], s1 = rowPtr[r + 1];
        if (s1 - s0 > kShortRow) continue;
        double t = b[r];
        for (int j = s0; j < s1; ++j) t = fma(-val[j], x[col[j]], t);
        if (F32)
            ((float *)rOut)[r] = (float)t;
        else
            ((double *)rOut)[r] = t;
        local = fma(t, t, local);
    }
    const double s = blockSum(local, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// segment g: sum of val*x over [segBeg[g], segEnd[g]), one warp
__global__ void __launch_bounds__(kThreads) kSegDot(int numSegs, const int *__restrict__ segBeg,
                                                    const int *__restrict__ segEnd, const int *__restrict__ col,
                                                    const double *__restrict__ val, const double *__restrict__ x,
                                                    double *__restrict__ segSum) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < numSegs; g += nw) {
        double t = 0.0;
        for (int j = segBeg[g] + lane; j < segEnd[g]; j += 32) t = fma(val[j], x[col[j]], t);
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) segSum[g] = t;
    }
}

// long row i: r = b - (sum of its segments in order), one warp per row
template <bool F32>
__global__ void __launch_bounds__(kThreads) kResidualLong(int numLong, const int *__restrict__ longRow,
                                                          const int *__restrict__ segFirst,
                                                          const double *__restrict__ segSum,
                                                          const double *__restrict__ b, void *rOut, double *part) {
    __shared__ double sm[kThreads / 32];
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double local = 0.0;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < numLong; i += nw) {
        double S = 0.0;
        for (int g = segFirst[i] + lane; g < segFirst[i + 1]; g += 32) S += segSum[g];
        for (int o = 16; o; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
        const int r = longRow[i];
        const double t = b[r] - S;
        if (lane == 0) {
            if (F32)
                ((float *)rOut)[r] = (float)t;
            else
                ((double *)rOut)[r] = t;
            local = fma(t, t, local);
        }
    }
    const double s = blockSum(local, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// *out = sum of part[0..count) in a fixed order (one block)
__global__ void __launch_bounds__(kThreads) kFinalSum(int count, const double *__restrict__ part, double *out) {
    __shared__ double sm[kThreads / 32];
    double local = 0.0;
    for (int i = threadIdx.x; i < count; i += kThreads) local += part[i];
    const double s = blockSum(local, sm);
    if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kThreads) kSumSq(int n, const double *__restrict__ v, double *part) {
    __shared__ double sm[kThreads / 32];
    double local = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) local = fma(v[i], v[i], local);
    const double s = blockSum(local, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
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
    {
        DevBuf<double> bpart(blocks);
        kSumSq<<<blocks, kThreads, 0, s>>>(n, b, bpart.p);
        kFinalSum<<<1, kThreads, 0, s>>>(blocks, bpart.p, acc.p + 1);
        RACE_CUDA(cudaStreamSynchronize(s));
    }
    double bn2 = 0;
    RACE_CUDA(cudaMemcpyAsync(&bn2, acc.p + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    const double bnorm = std::sqrt(bn2) > 0 ? std::sqrt(bn2) : 1.0;
    const size_t vb = f32 ? sizeof(float) : sizeof(double);
    // long rows and their segments (host scan of the row offsets, once per solve)
    std::vector<int> rp(n + 1);
    RACE_CUDA(cudaMemcpyAsync(rp.data(), rowPtr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    std::vector<int> longRow, segFirst{0}, segBeg, segEnd;
    for (int r = 0; r < n; ++r) {
        if (rp[r + 1] - rp[r] <= kShortRow) continue;
        longRow.push_back(r);
        for (int j = rp[r]; j < rp[r + 1]; j += kSegLen) {
            segBeg.push_back(j);
            segEnd.push_back(std::min(rp[r + 1], j + kSegLen));
        }
        segFirst.push_back((int)segBeg.size());
    }
    const int numLong = (int)longRow.size(), numSegs = (int)segBeg.size();
    DevBuf<int> dLongRow, dSegFirst, dSegBeg, dSegEnd;
    DevBuf<double> dSegSum(std::max(numSegs, 1));
    dLongRow.upload(numLong ? longRow.data() : nullptr, std::max(numLong, 1), s);
    dSegFirst.upload(segFirst.data(), segFirst.size(), s);
    dSegBeg.upload(numSegs ? segBeg.data() : nullptr, std::max(numSegs, 1), s);
    dSegEnd.upload(numSegs ? segEnd.data() : nullptr, std::max(numSegs, 1), s);
    const int blocksLong = std::max(1, std::min(ceilDiv(numLong, kThreads / 32), sms * 8));
    const int blocksSeg = std::max(1, std::min(ceilDiv(numSegs, kThreads / 32), sms * 8));
    DevBuf<double> part(blocks + blocksLong);
    int it = 0;
    double rel = 0;
    for (;;) {
        if (f32)
            kResidualShort<true><<<blocks, kThreads, 0, s>>>(n, rowPtr, col, val, b, x, f.ops.b, part.p);
        else
            kResidualShort<false><<<blocks, kThreads, 0, s>>>(n, rowPtr, col, val, b, x, f.ops.b, part.p);
        if (numLong) {
            kSegDot<<<blocksSeg, kThreads, 0, s>>>(numSegs, dSegBeg.p, dSegEnd.p, col, val, x, dSegSum.p);
            if (f32)
                kResidualLong<true><<<blocksLong, kThreads, 0, s>>>(numLong, dLongRow.p, dSegFirst.p, dSegSum.p, b,
                                                                    f.ops.b, part.p + blocks);
            else
                kResidualLong<false><<<blocksLong, kThreads, 0, s>>>(numLong, dLongRow.p, dSegFirst.p, dSegSum.p, b,
                                                                     f.ops.b, part.p + blocks);
        }
        kFinalSum<<<1, kThreads, 0, s>>>(numLong ? blocks + blocksLong : blocks, part.p, acc.p);
        RACE_CUDA(cudaGetLastError());
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
