// Persistent colored sweeps: SymmSpMV, SpMTV, SpMV, Gauss-Seidel and
// Kaczmarz over a RACE zone tree.
//
// RACE runs the zone tree with nested thread teams: at every node the
// threads run block 0 of their zones, meet at a barrier, then block 1, and a
// zone with one thread calls the kernel on its row range in order
// (src/functionManager.cpp:201-265). Two GPU executions of that schedule:
//
// * Wave mode (default). The execution order is compiled into conflict-free
//   waves (waves.cpp). One cooperative launch walks the waves with a bounded
//   grid barrier between them; inside a wave every row is independent and
//   one thread runs it with the kernel body's own operation order
//   (examples/src/helpers/kernels.cpp), so FP64 results are identical bit for
//   bit to RACE's sequential walk, and rows that RACE keeps in one long leaf
//   still run in parallel when they do not conflict.
// * Leaf mode (RACE_GPU_SWEEP_MODE=leaf). The flattened phases run with a
//   grid barrier between phases; one warp owns one leaf and walks its rows in
//   order, lanes splitting a row's non-zeros with warp-shuffle reductions.
//   Sums are reassociated (within 1e-12 relative of the sequential result).
//
// Neither mode needs atomics on the transpose scatter: the coloring (leaf
// mode) or the wave plan (wave mode) gives every written entry one writer.
#include <cuda_bf16.h>

#include "engine.h"

namespace race {
namespace {

constexpr int kSweepThreads = 256;
constexpr int kWarps = kSweepThreads / 32;

__device__ __forceinline__ unsigned ldAcquireU(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void stReleaseU(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Sense-reversing grid barrier. bar[0] arrivals, bar[1] generation. Returns
// false (and sets *status) if the wait exceeded the spin limit.
__device__ bool gridBarrier(unsigned *bar, int *status) {
    __shared__ int sOk;
    __syncthreads();
    if (threadIdx.x == 0) {
        sOk = 1;
        unsigned gen = ldAcquireU(bar + 1);
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u) + 1;
        if (arrived == gridDim.x) {
            bar[0] = 0;
            __threadfence();
            stReleaseU(bar + 1, gen + 1);
        } else {
            long long spins = 0;
            while (ldAcquireU(bar + 1) == gen) {
                if (++spins > kSpinLimit) {
                    atomicCAS(status, DEV_OK, DEV_WAIT_TIMEOUT);
                    sOk = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
    }
    __syncthreads();
    return sOk != 0;
}

template <typename VT>
__device__ __forceinline__ float toF(VT v) { return (float)v; }
template <>
__device__ __forceinline__ float toF<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

// a*b + c in the accumulation type
__device__ __forceinline__ double mac(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float mac(float a, float b, float c) { return fmaf(a, b, c); }

template <typename VT, typename XT>
__device__ __forceinline__ XT ld(const VT *val, int j) {
    if constexpr (sizeof(XT) == 8) return (XT)val[j];
    else return toF<VT>(val[j]);
}

struct SweepArgs {
    int kernel;
    const int *rowPtr;
    const int *col;
    const void *val;
    void *x;
    void *b;
    const int *ptr;   // wave mode: wavePtr; leaf mode: phasePtr
    const int *rows;  // wave mode: rows by wave; leaf mode: leafLo
    const int *hi;    // leaf mode: leafHi
    int num;          // waves or phases
    unsigned *bar;
    int *status;
};

// One row with the kernel body's own operation order (thread per row).
template <typename VT, typename XT>
__device__ __forceinline__ void rowSerial(const SweepArgs &a, int r) {
    const VT *val = (const VT *)a.val;
    XT *x = (XT *)a.x;
    XT *b = (XT *)a.b;
    const int s = a.rowPtr[r], e = a.rowPtr[r + 1];
    switch (a.kernel) {
    case RACE_K_SPMV: {  // kernels.cpp:5-15
        XT t = XT(0);
        for (int j = s; j < e; ++j) t = mac(ld<VT, XT>(val, j), x[a.col[j]], t);
        b[r] = t;
        break;
    }
    case RACE_K_SPMTV: {  // kernels.cpp:107-115
        const XT xr = x[r];
        for (int j = s; j < e; ++j) {
            const int c = a.col[j];
            b[c] = mac(ld<VT, XT>(val, j), xr, b[c]);
        }
        break;
    }
    case RACE_K_SYMMSPMV: {  // kernels.cpp:403-417
        const XT xr = x[r];
        b[r] = mac(ld<VT, XT>(val, s), xr, b[r]);
        XT t = XT(0);
        for (int j = s + 1; j < e; ++j) {
            const int c = a.col[j];
            const XT v = ld<VT, XT>(val, j);
            t = mac(v, x[c], t);
            b[c] = mac(v, xr, b[c]);
        }
        b[r] += t;
        break;
    }
    case RACE_K_GS: {  // kernels.cpp:174-186
        XT t = b[r];
        for (int j = s + 1; j < e; ++j) t = mac(-ld<VT, XT>(val, j), x[a.col[j]], t);
        x[r] = t / ld<VT, XT>(val, s);
        break;
    }
    case RACE_K_KACZ: {  // kernels.cpp:285-302
        XT nrm = XT(0), sc = -b[r];
        for (int j = s; j < e; ++j) {
            const XT v = ld<VT, XT>(val, j);
            sc = mac(v, x[a.col[j]], sc);
            nrm = mac(v, v, nrm);
        }
        sc /= nrm;
        for (int j = s; j < e; ++j) {
            const int c = a.col[j];
            x[c] = mac(-sc, ld<VT, XT>(val, j), x[c]);
        }
        break;
    }
    default: break;
    }
}

// Rows longer than this are run by a whole warp with a shuffle reduction
// instead of one thread (hub rows of power-law graphs would otherwise turn
// one thread's sequential fma chain into the wave's critical path); their
// sums are reassociated, all other rows keep the sequential order.
constexpr int kLongRow = 512;

template <typename VT, typename XT>
__device__ __forceinline__ void rowWarp(const SweepArgs &a, int row, int lane);

template <typename VT, typename XT>
__global__ void __launch_bounds__(kSweepThreads) kWaveSweep(SweepArgs a) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = tid >> 5, nw = nt >> 5;
    for (int w = 0; w < a.num; ++w) {
        const int r0 = a.ptr[w], r1 = a.ptr[w + 1];
        for (int i = r0 + tid; i < r1; i += nt) {
            const int r = a.rows[i];
            if (a.rowPtr[r + 1] - a.rowPtr[r] <= kLongRow) rowSerial<VT, XT>(a, r);
        }
        // long rows of this wave: one warp each, distributed over all warps
        // of the grid (rows of a wave are independent, so the two passes may
        // interleave)
        for (int i = r0 + gw; i < r1; i += nw) {
            const int r = a.rows[i];
            if (a.rowPtr[r + 1] - a.rowPtr[r] > kLongRow) rowWarp<VT, XT>(a, r, lane);
        }
        if (w + 1 < a.num && !gridBarrier(a.bar, a.status)) return;
    }
}

// ---- leaf mode: warp per leaf, lanes over a row, shuffle reductions

template <typename XT>
__device__ __forceinline__ XT warpSum(XT v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename VT, typename XT>
__device__ __forceinline__ void rowWarp(const SweepArgs &a, int row, int lane) {
    const VT *val = (const VT *)a.val;
    XT *x = (XT *)a.x;
    XT *b = (XT *)a.b;
    const int s = a.rowPtr[row], e = a.rowPtr[row + 1];
    switch (a.kernel) {
    case RACE_K_SPMV: {
        XT t = XT(0);
        for (int j = s + lane; j < e; j += 32) t = mac(ld<VT, XT>(val, j), x[a.col[j]], t);
        t = warpSum(t);
        if (lane == 0) b[row] = t;
        break;
    }
    case RACE_K_SPMTV: {
        const XT xr = x[row];
        for (int j = s + lane; j < e; j += 32) {
            int c = a.col[j];
            b[c] = mac(ld<VT, XT>(val, j), xr, b[c]);
        }
        break;
    }
    case RACE_K_SYMMSPMV: {
        const XT xr = x[row];
        XT t = XT(0);
        for (int j = s + 1 + lane; j < e; j += 32) {
            int c = a.col[j];
            XT v = ld<VT, XT>(val, j);
            t = mac(v, x[c], t);
            b[c] = mac(v, xr, b[c]);
        }
        t = warpSum(t);
        if (lane == 0) b[row] = mac(ld<VT, XT>(val, s), xr, b[row]) + t;
        break;
    }
    case RACE_K_GS: {
        XT t = XT(0);
        for (int j = s + 1 + lane; j < e; j += 32) t = mac(-ld<VT, XT>(val, j), x[a.col[j]], t);
        t = warpSum(t);
        if (lane == 0) x[row] = (b[row] + t) / ld<VT, XT>(val, s);
        break;
    }
    case RACE_K_KACZ: {
        XT dot = XT(0), nrm = XT(0);
        for (int j = s + lane; j < e; j += 32) {
            XT v = ld<VT, XT>(val, j);
            dot = mac(v, x[a.col[j]], dot);
            nrm = mac(v, v, nrm);
        }
        dot = warpSum(dot);
        nrm = warpSum(nrm);
        const XT sc = (dot - b[row]) / nrm;
        __syncwarp();
        for (int j = s + lane; j < e; j += 32) {
            int c = a.col[j];
            x[c] = mac(-sc, ld<VT, XT>(val, j), x[c]);
        }
        break;
    }
    default: break;
    }
    __syncwarp();
}

template <typename VT, typename XT>
__global__ void __launch_bounds__(kSweepThreads) kLeafSweep(SweepArgs a) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarps;
    for (int ph = 0; ph < a.num; ++ph) {
        for (int l = a.ptr[ph] + gw; l < a.ptr[ph + 1]; l += nw) {
            const int lo = a.rows[l], hi = a.hi[l];
            if (lo <= hi)
                for (int r = lo; r < hi; ++r) rowWarp<VT, XT>(a, r, lane);
            else
                for (int r = lo; r > hi; --r) rowWarp<VT, XT>(a, r, lane);
        }
        if (ph + 1 < a.num && !gridBarrier(a.bar, a.status)) return;
    }
}

template <typename K>
int coopBlocks(K kernel, int want) {
    int dev = 0, sms = 0, occ = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kSweepThreads, 0));
    return std::max(1, std::min(sms * std::max(occ, 1), want));
}

template <typename VT, typename XT>
void launch(bool waveMode, SweepArgs &a, int maxWork, cudaStream_t s) {
    void *args[] = {&a};
    if (waveMode) {
        int blocks = coopBlocks(kWaveSweep<VT, XT>, ceilDiv(maxWork, kSweepThreads));
        RACE_CUDA(cudaLaunchCooperativeKernel((void *)kWaveSweep<VT, XT>, blocks, kSweepThreads, args, 0, s));
    } else {
        int blocks = coopBlocks(kLeafSweep<VT, XT>, ceilDiv(maxWork, kWarps));
        RACE_CUDA(cudaLaunchCooperativeKernel((void *)kLeafSweep<VT, XT>, blocks, kSweepThreads, args, 0, s));
    }
}

}  // namespace

// Execution mode of one sweep direction: the engine's setting, or (auto)
// the cheaper of the two by a cost model fitted to GB300 timings (3D
// stencils and power-law graphs): a wave costs about 12 us (barrier plus one
// row's latency), a leaf phase about 1.3 us plus 0.67 us per row of its
// longest leaf.
bool useWaveMode(const Engine &e, const FuncEntry &f, int dir) {
    if (e.sweepMode == SWEEP_WAVE) return f.waves[dir].numWaves > 0;
    if (e.sweepMode == SWEEP_LEAF) return false;
    const DevPhases &d = e.dPhases[dir];
    const double leafCost = d.numPhases * (1.3 + 0.67 * d.maxLeafRows);
    const double waveCost = 12.0 * f.waves[dir].numWaves;
    return f.waves[dir].numWaves > 0 && waveCost <= leafCost;
}

void uploadPhases(Engine &e, int dir) {
    const PhaseTable &pt = e.phases[dir];
    DevPhases &d = e.dPhases[dir];
    d.numPhases = pt.numPhases();
    d.numLeaves = (int)pt.leafLo.size();
    d.maxLeaves = 0;
    d.maxLeafRows = 0;
    for (int p = 0; p < d.numPhases; ++p) d.maxLeaves = std::max(d.maxLeaves, pt.phasePtr[p + 1] - pt.phasePtr[p]);
    for (size_t l = 0; l < pt.leafLo.size(); ++l) d.maxLeafRows = std::max(d.maxLeafRows, std::abs(pt.leafHi[l] - pt.leafLo[l]));
    d.phasePtr.upload(pt.phasePtr.data(), pt.phasePtr.size(), e.stream);
    d.leafLo.upload(pt.leafLo.data(), std::max<size_t>(pt.leafLo.size(), 1), e.stream);
    d.leafHi.upload(pt.leafHi.data(), std::max<size_t>(pt.leafHi.size(), 1), e.stream);
}

// Wave plans of a registered sweep function for both directions.
void buildSweepWaves(Engine &e, FuncEntry &f) {
    const int n = f.ops.n;
    std::vector<int> rp(n + 1);
    RACE_CUDA(cudaMemcpyAsync(rp.data(), f.ops.rowPtr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, e.stream));
    RACE_CUDA(cudaStreamSynchronize(e.stream));
    std::vector<int> cl(std::max(rp[n], 1));
    RACE_CUDA(cudaMemcpyAsync(cl.data(), f.ops.col, sizeof(int) * (size_t)rp[n], cudaMemcpyDeviceToHost, e.stream));
    RACE_CUDA(cudaStreamSynchronize(e.stream));
    for (int dir = 0; dir < 2; ++dir) {
        WavePlan wp = buildWavePlan(f.kernel, n, rp.data(), cl.data(), e.phases[dir]);
        DevWaves &w = f.waves[dir];
        w.numWaves = wp.numWaves();
        w.maxRows = 0;
        for (int i = 0; i < w.numWaves; ++i) w.maxRows = std::max(w.maxRows, wp.wavePtr[i + 1] - wp.wavePtr[i]);
        w.wavePtr.upload(wp.wavePtr.data(), wp.wavePtr.size(), e.stream);
        w.rows.upload(wp.rows.data(), std::max<size_t>(wp.rows.size(), 1), e.stream);
    }
    RACE_CUDA(cudaStreamSynchronize(e.stream));
}

void runSweep(Engine &e, FuncEntry &f, bool rev) {
    const race_operands &ops = f.ops;
    const int dir = rev ? 1 : 0;
    const bool waveMode = useWaveMode(e, f, dir);
    RACE_CUDA(cudaMemsetAsync(e.dStatus.p, 0, sizeof(int) * 4, e.stream));
    SweepArgs a{f.kernel, ops.rowPtr, ops.col, ops.val, ops.x, ops.b, nullptr, nullptr, nullptr, 0,
                (unsigned *)(e.dStatus.p + 2), e.dStatus.p};
    int maxWork = 0;
    if (waveMode) {
        DevWaves &w = f.waves[dir];
        a.ptr = w.wavePtr.p;
        a.rows = w.rows.p;
        a.num = w.numWaves;
        maxWork = w.maxRows;
    } else {
        DevPhases &d = e.dPhases[dir];
        if (d.numPhases == 0) return;
        a.ptr = d.phasePtr.p;
        a.rows = d.leafLo.p;
        a.hi = d.leafHi.p;
        a.num = d.numPhases;
        maxWork = d.maxLeaves;
    }
    if (a.num == 0) return;
    if (ops.vec_type == RACE_VAL_F64) {
        if (ops.val_type != RACE_VAL_F64) throw Error(RACE_ERR_INVALID_ARG, "FP64 vectors need FP64 values");
        launch<double, double>(waveMode, a, maxWork, e.stream);
    } else if (ops.vec_type == RACE_VAL_F32) {
        if (ops.val_type == RACE_VAL_F32)
            launch<float, float>(waveMode, a, maxWork, e.stream);
        else if (ops.val_type == RACE_VAL_BF16)
            launch<__nv_bfloat16, float>(waveMode, a, maxWork, e.stream);
        else
            throw Error(RACE_ERR_INVALID_ARG, "FP32 vectors need FP32 or BF16 values");
    } else {
        throw Error(RACE_ERR_INVALID_ARG, "unknown vector type");
    }
}

}  // namespace race
