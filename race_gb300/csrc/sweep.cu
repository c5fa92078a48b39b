// Persistent colored sweep: SymmSpMV, SpMTV, SpMV, Gauss-Seidel and
// Kaczmarz over a RACE zone tree flattened into phases.
//
// RACE runs the zone tree with nested thread teams: at every node the
// threads run block 0 of their zones, meet at a barrier, then block 1, and a
// zone with one thread calls the kernel on its row range
// (src/functionManager.cpp:201-265). Flattened, that is a sequence of
// phases; the leaves of one phase are row ranges whose neighbourhoods are
// disjoint (distance-1 or distance-2 coloring), so they run concurrently
// without atomics. Here one cooperative launch walks all phases; a grid-wide
// barrier with a bounded wait separates phases. One warp owns one leaf and
// processes its rows in order (ascending, or descending for the reverse
// sweep); the lanes of the warp split a row's non-zeros, reduce with warp
// shuffles, and scatter to distinct columns.
#include <cooperative_groups.h>

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

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct SweepArgs {
    int kernel;
    const int *rowPtr;
    const int *col;
    const double *val;
    double *x;
    double *b;
    const int *phasePtr;
    const int *leafLo;
    const int *leafHi;
    int numPhases;
    unsigned *bar;
    int *status;
};

// One row of the chosen kernel, executed by a full warp.
__device__ __forceinline__ void sweepRow(const SweepArgs &a, int row, int lane) {
    const int s = a.rowPtr[row], e = a.rowPtr[row + 1];
    switch (a.kernel) {
    case RACE_K_SPMV: {  // b[r] = sum a x (kernels.cpp:5-15)
        double t = 0.0;
        for (int j = s + lane; j < e; j += 32) t = fma(a.val[j], a.x[a.col[j]], t);
        t = warpSum(t);
        if (lane == 0) a.b[row] = t;
        break;
    }
    case RACE_K_SPMTV: {  // b[c] += a x[r] (kernels.cpp:107-115)
        const double xr = a.x[row];
        for (int j = s + lane; j < e; j += 32) {
            int c = a.col[j];
            a.b[c] = fma(a.val[j], xr, a.b[c]);
        }
        break;
    }
    case RACE_K_SYMMSPMV: {  // upper triangle, diagonal first (kernels.cpp:403-417)
        const double xr = a.x[row];
        double t = 0.0;
        for (int j = s + 1 + lane; j < e; j += 32) {
            int c = a.col[j];
            double v = a.val[j];
            t = fma(v, a.x[c], t);
            a.b[c] = fma(v, xr, a.b[c]);
        }
        t = warpSum(t);
        if (lane == 0) {
            double br = fma(a.val[s], xr, a.b[row]);
            a.b[row] = br + t;
        }
        break;
    }
    case RACE_K_GS: {  // x[r] = (b[r] - sum_{j!=r} a x_j) / a_rr (kernels.cpp:174-186)
        double t = 0.0;
        for (int j = s + 1 + lane; j < e; j += 32) t = fma(-a.val[j], a.x[a.col[j]], t);
        t = warpSum(t);
        if (lane == 0) a.x[row] = (a.b[row] + t) / a.val[s];
        break;
    }
    case RACE_K_KACZ: {  // projection onto row r (kernels.cpp:285-302)
        double dot = 0.0, nrm = 0.0;
        for (int j = s + lane; j < e; j += 32) {
            double v = a.val[j];
            dot = fma(v, a.x[a.col[j]], dot);
            nrm = fma(v, v, nrm);
        }
        dot = warpSum(dot);
        nrm = warpSum(nrm);
        const double scale = (dot - a.b[row]) / nrm;
        __syncwarp();
        for (int j = s + lane; j < e; j += 32) {
            int c = a.col[j];
            a.x[c] = fma(-scale, a.val[j], a.x[c]);
        }
        break;
    }
    default: break;
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kSweepThreads) kSweep(SweepArgs a) {
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarps;
    for (int ph = 0; ph < a.numPhases; ++ph) {
        const int l0 = a.phasePtr[ph], l1 = a.phasePtr[ph + 1];
        for (int l = l0 + gw; l < l1; l += nw) {
            const int lo = a.leafLo[l], hi = a.leafHi[l];
            if (lo <= hi) {
                for (int r = lo; r < hi; ++r) sweepRow(a, r, lane);
            } else {
                for (int r = lo; r > hi; --r) sweepRow(a, r, lane);
            }
        }
        if (ph + 1 < a.numPhases) {
            if (!gridBarrier(a.bar, a.status)) return;
        }
    }
}

}  // namespace

void uploadPhases(Engine &e, int dir) {
    const PhaseTable &pt = e.phases[dir];
    DevPhases &d = e.dPhases[dir];
    d.numPhases = pt.numPhases();
    d.numLeaves = (int)pt.leafLo.size();
    d.maxLeaves = 0;
    for (int p = 0; p < d.numPhases; ++p) d.maxLeaves = std::max(d.maxLeaves, pt.phasePtr[p + 1] - pt.phasePtr[p]);
    d.phasePtr.upload(pt.phasePtr.data(), pt.phasePtr.size(), e.stream);
    d.leafLo.upload(pt.leafLo.data(), pt.leafLo.size(), e.stream);
    d.leafHi.upload(pt.leafHi.data(), pt.leafHi.size(), e.stream);
}

void runSweep(Engine &e, int kernel, const race_operands &ops, bool rev) {
    DevPhases &d = e.dPhases[rev ? 1 : 0];
    if (d.numPhases == 0) return;
    if (ops.val_type != RACE_VAL_F64) throw Error(RACE_ERR_NOT_IMPLEMENTED, "colored sweeps take FP64 values");
    int dev = 0, sms = 0, occ = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kSweep, kSweepThreads, 0));
    int blocks = std::min(sms * std::max(occ, 1), std::max(1, ceilDiv(d.maxLeaves, kWarps)));
    RACE_CUDA(cudaMemsetAsync(e.dStatus.p, 0, sizeof(int) * 4, e.stream));
    SweepArgs a{kernel, ops.rowPtr, ops.col, (const double *)ops.val, ops.x, ops.b, d.phasePtr.p, d.leafLo.p,
                d.leafHi.p, d.numPhases, (unsigned *)(e.dStatus.p + 2), e.dStatus.p};
    void *args[] = {&a};
    RACE_CUDA(cudaLaunchCooperativeKernel((void *)kSweep, blocks, kSweepThreads, args, 0, e.stream));
}

}  // namespace race
