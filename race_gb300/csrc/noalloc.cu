// Matrix-power kernel that allocates no memory.
//
// Some callers cannot allocate device memory at the point where they run
// the kernel: code that owns all device memory through its own pool and
// forbids driver allocations, real-time loops with a fixed memory budget,
// or library code called from a context where a cudaMalloc would
// synchronise the device. race_mpk_noalloc serves them. The caller passes
// the permuted CRS matrix, the level groups and the power vectors; every
// scratch word the kernel needs (completion flags, work ticket, status,
// small prefix tables) lives in one file-scope __device__ array of
// kNoAllocScratchInts ints. Each GPU that loads the library holds that
// array until the process exits.
//
// Work decomposition (same results as the registered MPK path, bit for bit,
// rows longer than kMpkHubRowLen included: they are summed by the whole warp
// in the same order): chunks of 32 consecutive rows inside each level group; work items
// (power k, chunk) in diagonals d = group + 2k; an item waits until, at
// power k-1, the chunks holding its columns are complete. Chunk positions,
// diagonal offsets and dependency ranges are derived on the fly from the
// group array, so nothing beyond the flags is stored.
#include <mutex>

#include "engine.h"

namespace race {

constexpr int kNoAllocScratchInts = 1 << 22;  // 16 MiB
constexpr int kNaThreads = 256;

// Layout: [0] ticket, [1] status, [2..3] reserved, [4 .. 4+G] chunk start
// per group, then diagonal starts (G + 2(p-1) + 1), then p * chunks flags.
static __device__ __align__(256) int gNoAllocScratch[kNoAllocScratchInts];

namespace {

__device__ __forceinline__ int ldAcq(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Single-block setup: chunk starts per group and item starts per diagonal.
// The device copy of the groups must describe the layout the host sized
// the scratch for: rows 0..n in non-decreasing offsets and hostChunks chunks
// in all. Otherwise the status word reports a bad schedule and no item is
// issued (all diagonals empty), so no flag beyond the checked region is
// touched.
__global__ void kNaSetup(int *scr, const int *__restrict__ groupPtr, int G, int power, int stride, int n,
                         long long hostChunks) {
    int *chunkStart = scr + 4;
    int *diagStart = chunkStart + G + 1;
    if (threadIdx.x == 0) {
        const int D = G + stride * (power - 1);
        bool ok = groupPtr[0] == 0 && groupPtr[G] == n;
        long long c = 0;
        for (int g = 0; g < G && ok; ++g) {
            if (groupPtr[g + 1] < groupPtr[g]) ok = false;
            chunkStart[g] = (int)c;
            c += (groupPtr[g + 1] - groupPtr[g] + 31) / 32;
        }
        if (!ok || c != hostChunks) {
            scr[1] = DEV_BAD_SCHEDULE;
            for (int g = 0; g <= G; ++g) chunkStart[g] = 0;
            for (int d = 0; d <= D; ++d) diagStart[d] = 0;
            return;
        }
        chunkStart[G] = (int)c;
        int it = 0;
        for (int d = 0; d < D; ++d) {
            diagStart[d] = it;
            for (int k = 0; k < power; ++k) {
                int g = d - stride * k;
                if (g >= 0 && g < G) it += chunkStart[g + 1] - chunkStart[g];
            }
        }
        diagStart[D] = it;
    }
}

// Group holding row r (binary search over groupPtr).
__device__ __forceinline__ int groupOf(const int *groupPtr, int G, int r) {
    int a = 0, b = G - 1;
    while (a < b) {
        int m = (a + b + 1) >> 1;
        if (groupPtr[m] <= r) a = m; else b = m - 1;
    }
    return a;
}

struct NaArgs {
    int n, G, power, stride;
    const int *rowPtr, *col;
    const double *val;
    double *x;
    const int *groupPtr;
    int *scr;
};

__global__ void __launch_bounds__(kNaThreads) kMpkNoAlloc(NaArgs a) {
    const int lane = threadIdx.x & 31;
    int *ticket = a.scr, *status = a.scr + 1;
    const int *chunkStart = a.scr + 4;
    const int *diagStart = chunkStart + a.G + 1;
    const int D = a.G + a.stride * (a.power - 1);
    const int numChunks = chunkStart[a.G];
    int *done = const_cast<int *>(diagStart) + D + 1;
    const int numItems = diagStart[D];
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(ticket, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= numItems) return;
        // item -> (diagonal, power, group, chunk)
        int lo = 0, hi = D - 1;
        while (lo < hi) {
            int m = (lo + hi + 1) >> 1;
            if (diagStart[m] <= it) lo = m; else hi = m - 1;
        }
        const int d = lo;
        int rem = it - diagStart[d], k = 0, g = 0;
        for (k = 0; k < a.power; ++k) {
            g = d - a.stride * k;
            if (g < 0 || g >= a.G) continue;
            int cnt = chunkStart[g + 1] - chunkStart[g];
            if (rem < cnt) break;
            rem -= cnt;
        }
        if (k == a.power) {  // cannot happen with consistent tables; never index with it
            if (lane == 0) atomicCAS(status, DEV_OK, DEV_BAD_SCHEDULE);
            return;
        }
        const int c = chunkStart[g] + rem;
        const int r0 = a.groupPtr[g] + 32 * rem;
        const int r1 = min(r0 + 32, a.groupPtr[g + 1]);
        const int r = r0 + lane;
        const bool live = r < r1;
        const int s = live ? a.rowPtr[r] : 0, e = live ? a.rowPtr[r + 1] : 0;
        if (k > 0) {
            // chunk ranges read in groups g-1, g, g+1 (columns elsewhere cannot
            // occur in a matrix permuted with the engine's MPK permutation;
            // they are reported through the status word)
            int cmin[3] = {INT_MAX, INT_MAX, INT_MAX}, cmax[3] = {-1, -1, -1};
            bool bad = false;
            for (int j = s; j < e; ++j) {
                const int cc = a.col[j];
                const int gg = groupOf(a.groupPtr, a.G, cc);
                const int dd = gg - g + 1;
                if (dd < 0 || dd > 2) {
                    bad = true;
                    continue;
                }
                const int ch = chunkStart[gg] + (cc - a.groupPtr[gg]) / 32;
                cmin[dd] = min(cmin[dd], ch);
                cmax[dd] = max(cmax[dd], ch);
            }
            if (__any_sync(0xffffffffu, bad)) {
                if (lane == 0) atomicCAS(status, DEV_OK, DEV_BAD_SCHEDULE);
                return;
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                for (int o = 16; o; o >>= 1) {
                    cmin[q] = min(cmin[q], __shfl_xor_sync(0xffffffffu, cmin[q], o));
                    cmax[q] = max(cmax[q], __shfl_xor_sync(0xffffffffu, cmax[q], o));
                }
                // an empty range becomes [0, -1]: the sentinel INT_MAX must
                // never enter the index arithmetic below (INT_MAX + lane
                // overflows to a negative index)
                if (cmax[q] < 0) cmin[q] = 0;
            }
            const int *dn = done + (size_t)(k - 1) * numChunks;
            long long spins = 0;
            for (;;) {
                bool ok = true;
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    for (int i = cmin[q] + lane; i <= cmax[q]; i += 32)
                        if (ldAcq(dn + i) == 0) ok = false;
                if (__all_sync(0xffffffffu, ok)) break;
                if (++spins > kSpinLimit || ldAcq(status) != DEV_OK) {
                    if (lane == 0) atomicCAS(status, DEV_OK, DEV_WAIT_TIMEOUT);
                    return;
                }
                __nanosleep(32);
            }
        }
        const double *xin = a.x + (size_t)k * a.n;
        if (live && e - s <= kMpkHubRowLen) {
            double t = 0.0;
            for (int j = s; j < e; ++j) t = fma(a.val[j], xin[a.col[j]], t);
            a.x[(size_t)(k + 1) * a.n + r] = t;
        }
        // rows longer than kMpkHubRowLen: the whole warp, in the registered
        // path's order (lane l: entries l, l+32, ...; then the xor butterfly)
        unsigned hubs = __ballot_sync(0xffffffffu, live && e - s > kMpkHubRowLen);
        while (hubs) {
            const int h = __ffs(hubs) - 1;
            hubs &= hubs - 1;
            const int hs = __shfl_sync(0xffffffffu, s, h), he = __shfl_sync(0xffffffffu, e, h);
            double t = 0.0;
            for (int j = hs + lane; j < he; j += 32) t = fma(a.val[j], xin[a.col[j]], t);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) a.x[(size_t)(k + 1) * a.n + r0 + h] = t;
        }
        __syncwarp();
        if (lane == 0)
            asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(done + (size_t)k * numChunks + c), "r"(1)
                         : "memory");
    }
}

std::mutex gNaMutex;
int *gNaAddr[64] = {};  // device address of the scratch array, per device

}  // namespace

}  // namespace race

extern "C" int race_mpk_noalloc(int n, const int *rowPtr, const int *col, const double *val, const int *groupPtr_dev,
                                const int *groupPtr_host, int numGroups, int power, double *x, void *stream) {
    using namespace race;
    if (n <= 0 || !rowPtr || !col || !val || !groupPtr_dev || !groupPtr_host || !x || numGroups < 1 || power < 1 ||
        power > 255)
        return RACE_ERR_INVALID_ARG;
    if (groupPtr_host[0] != 0 || groupPtr_host[numGroups] != n) {
        fprintf(stderr, "[RACE-GB300] race_mpk_noalloc: level groups must cover rows 0..n\n");
        return RACE_ERR_INVALID_ARG;
    }
    for (int g = 0; g < numGroups; ++g)
        if (groupPtr_host[g + 1] < groupPtr_host[g]) {
            fprintf(stderr, "[RACE-GB300] race_mpk_noalloc: level group offsets must not decrease\n");
            return RACE_ERR_INVALID_ARG;
        }
    // scratch needed: 4 + (G+1) + (G + 2(p-1) + 1) + p * chunks
    long long chunks = 0;
    for (int g = 0; g < numGroups; ++g) chunks += (groupPtr_host[g + 1] - groupPtr_host[g] + 31) / 32;
    const int stride = 2;
    const long long need = 4 + (numGroups + 1) + (numGroups + stride * (power - 1) + 1) + (long long)power * chunks;
    if (need > kNoAllocScratchInts) {
        fprintf(stderr,
                "[RACE-GB300] race_mpk_noalloc: problem needs %lld scratch ints, the built-in array holds %d "
                "(power * ceil(rows/32) must stay below about %d)\n",
                need, kNoAllocScratchInts, kNoAllocScratchInts);
        return RACE_ERR_INVALID_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RACE_ERR_CUDA;
    int *scr = nullptr;
    {
        std::lock_guard<std::mutex> lock(gNaMutex);
        if (!gNaAddr[dev]) {
            // first call on this device: resolve the array's device address
            // (with this device current); a host-side use of the symbol would
            // name host memory
            if (cudaGetSymbolAddress((void **)&gNaAddr[dev], gNoAllocScratch) != cudaSuccess) {
                gNaAddr[dev] = nullptr;
                return RACE_ERR_CUDA;
            }
        }
        scr = gNaAddr[dev];
    }
    // every call shares the array: clear the counters and the flags it uses
    const long long flagsOff = 4 + (numGroups + 1) + (numGroups + stride * (power - 1) + 1);
    if (cudaMemsetAsync(scr, 0, 4 * sizeof(int), s) != cudaSuccess) return RACE_ERR_CUDA;
    if (cudaMemsetAsync(scr + flagsOff, 0, sizeof(int) * (size_t)(power * chunks), s) != cudaSuccess)
        return RACE_ERR_CUDA;
    kNaSetup<<<1, 32, 0, s>>>(scr, groupPtr_dev, numGroups, power, stride, n, chunks);
    int sms = 0, occ = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return RACE_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kMpkNoAlloc, kNaThreads, 0) != cudaSuccess)
        return RACE_ERR_CUDA;
    NaArgs a{n, numGroups, power, stride, rowPtr, col, val, x, groupPtr_dev, scr};
    kMpkNoAlloc<<<sms * (occ > 0 ? occ : 1), kNaThreads, 0, s>>>(a);
    if (cudaGetLastError() != cudaSuccess) return RACE_ERR_CUDA;
    int st = 0;
    if (cudaMemcpyAsync(&st, scr + 1, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return RACE_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RACE_ERR_CUDA;
    if (st == DEV_BAD_SCHEDULE) return RACE_ERR_INVALID_ARG;
    if (st != DEV_OK) return RACE_ERR_TIMEOUT;
    return RACE_SUCCESS;
}
