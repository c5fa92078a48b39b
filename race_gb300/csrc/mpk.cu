// Level-blocked matrix-power kernel (MPK): x_k = A x_{k-1}, k = 1..p.
//
// RACE's schedule (src/matrixPower.cpp consolidatePartition; executor
// src/functionManager.cpp:618-823) groups BFS levels so that p+1 powers of
// one group fit the cache, and runs a diagonal wavefront: at step s the
// group s-k is computed at power k for all k. Because BFS levels only couple
// neighbouring levels, power k of a group needs power k-1 of the group
// itself and its two neighbours, all of which come earlier in that order.
//
// GPU form: the permuted CRS is cut into tiles (contiguous rows, never
// crossing a level group, at most kTileRows rows and kTileNnz non-zeros).
// Work items (power, tile) are listed in the wavefront order; persistent
// CTAs take them in order from a global ticket. Before computing, an item
// waits until every tile up to the highest tile its columns touch is done at
// the previous power: a per-power watermark counts the completed prefix of
// tiles. Items only wait on earlier tickets, which are held by running CTAs,
// so the schedule cannot deadlock; each wait is bounded anyway and reports
// a timeout through the status word. Groups sized to the L2 keep a group's
// rows resident while its p powers are computed, so the matrix is read from
// HBM about once per call instead of p times.
//
// Each row is a sequential fma chain in CRS order (the order of
// MAT_SPMV_KERNEL, examples/src/helpers/kernels.cpp:749-777), so FP64 output
// is bit-identical to p plain sequential SpMVs with fused multiply-adds.
#include <algorithm>
#include <numeric>

#include <cuda_bf16.h>

#include "engine.h"

namespace race {

constexpr int kTileRows = 128;
constexpr int kTileNnz = 4096;
constexpr int kMpkThreads = 128;

namespace {

__device__ __forceinline__ int ldAcquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void stRelease(int *p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void backoff() { __nanosleep(64); }

// Row of the matrix times a vector. FP64 storage: fma chain in double.
// FP32/BF16 storage: fma chain in float (values and x rounded to float).
template <typename VT>
struct RowDot;
template <>
struct RowDot<double> {
    static __device__ __forceinline__ double run(const double *__restrict__ val, const int *__restrict__ col, int s,
                                                 int e, const double *__restrict__ x) {
        double t = 0.0;
#pragma unroll 4
        for (int j = s; j < e; ++j) t = fma(val[j], __ldcg(x + col[j]), t);
        return t;
    }
};
template <>
struct RowDot<float> {
    static __device__ __forceinline__ double run(const float *__restrict__ val, const int *__restrict__ col, int s,
                                                 int e, const double *__restrict__ x) {
        float t = 0.0f;
#pragma unroll 4
        for (int j = s; j < e; ++j) t = fmaf(val[j], (float)__ldcg(x + col[j]), t);
        return (double)t;
    }
};
template <>
struct RowDot<__nv_bfloat16> {
    static __device__ __forceinline__ double run(const __nv_bfloat16 *__restrict__ val, const int *__restrict__ col,
                                                 int s, int e, const double *__restrict__ x) {
        float t = 0.0f;
#pragma unroll 4
        for (int j = s; j < e; ++j) t = fmaf(__bfloat162float(val[j]), (float)__ldcg(x + col[j]), t);
        return (double)t;
    }
};

struct MpkArgs {
    const int *rowPtr;
    const int *col;
    const void *val;
    double *x;
    int n;
    const int *tileRow;
    const int *depHi;
    const int *itemTile;
    const unsigned char *itemPow;
    int numItems, numTiles;
    int *flags;
    int *watermark;
    int *ticket;
    int *status;
};

template <typename VT>
__global__ void __launch_bounds__(kMpkThreads) kMpk(MpkArgs a) {
    __shared__ int sItem;
    __shared__ int sBail;
    const VT *__restrict__ val = (const VT *)a.val;
    for (;;) {
        if (threadIdx.x == 0) {
            sItem = atomicAdd(a.ticket, 1);
            sBail = 0;
        }
        __syncthreads();
        const int it = sItem;
        if (it >= a.numItems) break;
        const int t = a.itemTile[it];
        const int k = a.itemPow[it];  // computes x_{k+1} from x_k
        if (threadIdx.x == 0 && k > 0) {
            const int need = a.depHi[t];
            const int *wm = a.watermark + (k - 1);
            long long spins = 0;
            while (ldAcquire(wm) <= need) {
                if (++spins > kSpinLimit || ldAcquire(a.status) != DEV_OK) {
                    atomicCAS(a.status, DEV_OK, DEV_WAIT_TIMEOUT);
                    sBail = 1;
                    break;
                }
                backoff();
            }
        }
        __syncthreads();
        if (sBail) break;
        const int r0 = a.tileRow[t], r1 = a.tileRow[t + 1];
        const double *__restrict__ xin = a.x + (size_t)k * a.n;
        double *__restrict__ xout = a.x + (size_t)(k + 1) * a.n;
        for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
            xout[r] = RowDot<VT>::run(val, a.col, a.rowPtr[r], a.rowPtr[r + 1], xin);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int *fl = a.flags + (size_t)k * a.numTiles;
            __threadfence();
            stRelease(fl + t, 1);
            __threadfence();
            // advance the completed prefix of power k past every done tile
            int *wm = a.watermark + k;
            int w = ldAcquire(wm);
            while (w < a.numTiles && ldAcquire(fl + w) == 1) {
                int old = atomicCAS(wm, w, w + 1);
                w = (old == w) ? w + 1 : old;
            }
        }
    }
}

// Highest column of every row, then per tile the highest tile it reads.
__global__ void kTileDeps(const int *__restrict__ rowPtr, const int *__restrict__ col, const int *__restrict__ tileRow,
                          int numTiles, int *__restrict__ depHi) {
    int t = blockIdx.x;
    if (t >= numTiles) return;
    int r0 = tileRow[t], r1 = tileRow[t + 1];
    int m = -1;
    for (int j = rowPtr[r0] + threadIdx.x; j < rowPtr[r1]; j += blockDim.x) m = max(m, col[j]);
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ int sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = max(m, sm[w]);
        m = max(m, sm[0]);
        // binary search: tile holding row m
        int lo = 0, hi = numTiles - 1;
        if (m < 0) m = r0;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (tileRow[mid] <= m) lo = mid; else hi = mid - 1;
        }
        depHi[t] = max(lo, t);
    }
}

__global__ void kSpmvPlain(int n, const int *__restrict__ rowPtr, const int *__restrict__ col,
                           const double *__restrict__ val, const double *__restrict__ x, double *__restrict__ b) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double t = 0.0;
#pragma unroll 4
    for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) t = fma(val[j], x[col[j]], t);
    b[r] = t;
}

}  // namespace

// Builds the tile table and the wavefront item order of one MPK operand set
// (the user's permuted matrix) for the engine's level groups.
std::unique_ptr<MpkPlan> buildMpkPlan(Engine &e, const race_operands &ops, int power) {
    auto plan = std::make_unique<MpkPlan>();
    const int n = ops.n;
    std::vector<int> rp(n + 1);
    RACE_CUDA(cudaMemcpyAsync(rp.data(), ops.rowPtr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, e.stream));
    RACE_CUDA(cudaStreamSynchronize(e.stream));
    const std::vector<int> &gp = e.groupPtr;
    const int G = (int)gp.size() - 1;
    std::vector<int> tileRow{0}, tileGroup;
    for (int g = 0; g < G; ++g) {
        int r = gp[g];
        while (r < gp[g + 1]) {
            int s = r;
            int lim = std::min(gp[g + 1], s + kTileRows);
            int e2 = s + 1;
            while (e2 < lim && rp[e2 + 1] - rp[s] <= kTileNnz) ++e2;
            tileRow.push_back(e2);
            tileGroup.push_back(g);
            plan->maxTileNnz = std::max(plan->maxTileNnz, rp[e2] - rp[s]);
            r = e2;
        }
    }
    const int T = (int)tileGroup.size();
    std::vector<int> groupFirst(G + 1, 0);
    for (int t = 0, g = 0; g <= G; ++g) {
        while (t < T && tileGroup[t] < g) ++t;
        groupFirst[g] = t;
    }
    // wavefront order: step s, power k, group s-k (functionManager.cpp:638-647)
    std::vector<int> itemTile;
    std::vector<unsigned char> itemPow;
    itemTile.reserve((size_t)T * power);
    for (int s = 0; s < G + power - 1; ++s)
        for (int k = 0; k < power; ++k) {
            int g = s - k;
            if (g < 0 || g >= G) continue;
            for (int t = groupFirst[g]; t < groupFirst[g + 1]; ++t) {
                itemTile.push_back(t);
                itemPow.push_back((unsigned char)k);
            }
        }
    plan->numTiles = T;
    plan->power = power;
    plan->numItems = (int)itemTile.size();
    plan->tileRow.upload(tileRow.data(), tileRow.size(), e.stream);
    plan->itemTile.upload(itemTile.data(), itemTile.size(), e.stream);
    plan->itemPow.upload(itemPow.data(), itemPow.size(), e.stream);
    plan->depHi.alloc(std::max(T, 1));
    plan->flags.alloc((size_t)std::max(T, 1) * power);
    plan->watermark.alloc(power);
    plan->ticket.alloc(1);
    plan->status.alloc(1);
    if (T > 0) kTileDeps<<<T, 128, 0, e.stream>>>(ops.rowPtr, ops.col, plan->tileRow.p, T, plan->depHi.p);
    RACE_CUDA(cudaGetLastError());
    std::vector<int> dep(std::max(T, 1));
    RACE_CUDA(cudaMemcpyAsync(dep.data(), plan->depHi.p, sizeof(int) * T, cudaMemcpyDeviceToHost, e.stream));
    RACE_CUDA(cudaStreamSynchronize(e.stream));
    // Every dependency must come earlier in the wavefront order: columns of
    // group g may reach at most group g+1 (BFS levels couple neighbours
    // only). A matrix not permuted with this engine's MPK permutation would
    // break that and is rejected here instead of stalling the kernel.
    for (int t = 0; t < T; ++t)
        if (tileGroup[dep[t]] > tileGroup[t] + 1)
            throw Error(RACE_ERR_INVALID_ARG,
                        "MPK operand is not in the engine's level order (permute it with getPerm/getInvPerm)");
    return plan;
}

void runMpk(Engine &e, MpkPlan &plan, const race_operands &ops, int power) {
    if (power > plan.power) throw Error(RACE_ERR_INVALID_ARG, "power above the planned power");
    cudaStream_t s = e.stream;
    RACE_CUDA(cudaMemsetAsync(plan.flags.p, 0, sizeof(int) * (size_t)plan.numTiles * plan.power, s));
    RACE_CUDA(cudaMemsetAsync(plan.watermark.p, 0, sizeof(int) * plan.power, s));
    RACE_CUDA(cudaMemsetAsync(plan.ticket.p, 0, sizeof(int), s));
    RACE_CUDA(cudaMemsetAsync(plan.status.p, 0, sizeof(int), s));
    MpkArgs a{ops.rowPtr, ops.col, ops.val, ops.x, ops.n, plan.tileRow.p, plan.depHi.p, plan.itemTile.p,
              plan.itemPow.p, 0, plan.numTiles, plan.flags.p, plan.watermark.p, plan.ticket.p, plan.status.p};
    // items of powers above `power` are skipped by truncating the item list:
    // the wavefront lists them interleaved, so run the full list only when
    // power equals the planned power.
    if (power != plan.power) throw Error(RACE_ERR_NOT_IMPLEMENTED, "power must equal the registered power");
    a.numItems = plan.numItems;
    int dev = 0, sms = 0, occ = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    switch (ops.val_type) {
    case RACE_VAL_F64:
        RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kMpk<double>, kMpkThreads, 0));
        kMpk<double><<<sms * std::max(occ, 1), kMpkThreads, 0, s>>>(a);
        break;
    case RACE_VAL_F32:
        RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kMpk<float>, kMpkThreads, 0));
        kMpk<float><<<sms * std::max(occ, 1), kMpkThreads, 0, s>>>(a);
        break;
    case RACE_VAL_BF16:
        RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kMpk<__nv_bfloat16>, kMpkThreads, 0));
        kMpk<__nv_bfloat16><<<sms * std::max(occ, 1), kMpkThreads, 0, s>>>(a);
        break;
    default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
    }
    RACE_CUDA(cudaGetLastError());
}

int mpkStatus(Engine &e, MpkPlan &plan) {
    int st = 0;
    RACE_CUDA(cudaMemcpyAsync(&st, plan.status.p, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
    RACE_CUDA(cudaStreamSynchronize(e.stream));
    return st;
}

void Engine::spmvPlain(int nr, const int *rowPtr, const int *col, const double *val, const double *x, double *b) {
    kSpmvPlain<<<ceilDiv(nr, 256), 256, 0, stream>>>(nr, rowPtr, col, val, x, b);
    RACE_CUDA(cudaGetLastError());
}

}  // namespace race
