// GPU graph set-up and level traversal.
//
// Graph (RACE::Graph, src/graph_SoA.cpp:437-477 with permute-on-fly): the
// CRS pattern stays in its original numbering; the running permutation
// totalPerm/totalInvPerm maps the current index space to original rows.
// A pattern that is not symmetric gets the missing transposed entries
// appended to their rows first (makeSymmetricGraph, src/graph.cpp:47-142).
//
// Traversal (Traverse::calculateDistance, src/traverse_GAP_graphSoA.cpp:
// 135-575): a level-synchronous top-down BFS over rows [lo,hi) of the
// current space from root lo. One warp expands one frontier vertex; a vertex
// is claimed with an atomic exchange on a per-traversal stamp, so every row
// is visited once and gets the level of the step that reached it first
// (levels do not depend on the order inside a frontier). Distance-2 mode
// lets out-of-range neighbours of in-range rows pass the front on once;
// islands restart from the lowest unvisited row. Then a histogram gives rows
// and non-zeros per level, a stable radix sort of (level, row) gives the
// level order, and the order is composed into totalPerm.
#include <cub/cub.cuh>

#include <algorithm>
#include <climits>
#include <numeric>

#include "engine.h"
#include "mpk_order.h"

namespace race {
namespace {

constexpr int kWarpsPerBlock = 8;

__global__ void kFill(int *a, int lo, int hi, int v) {
    int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < hi) a[i] = v;
}

__global__ void kSetRoot(int *dist, int *stamp, int *front, int root, int lvl, int stampVal) {
    dist[root] = lvl;
    stamp[root] = stampVal;
    front[0] = root;
}

// ctr[0]: size of the next frontier; ctr[1]: in-range rows newly reached.
template <int DMODE>
__global__ void kExpand(const int *__restrict__ rowPtr, const int *__restrict__ col, const int *__restrict__ perm,
                        const int *__restrict__ invPerm, int n, const int *__restrict__ front, int fsize,
                        int *__restrict__ next, int *__restrict__ ctr, int *__restrict__ dist, int *__restrict__ stamp,
                        int stampVal, int lvl, int lo, int hi) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int w = warp; w < fsize; w += nwarps) {
        const int u = front[w];
        const int pu = perm[u];
        const bool uIn = (u >= lo) && (u < hi);
        const int s = rowPtr[pu], e = rowPtr[pu + 1];
        for (int base = s; base < e; base += 32) {
            int j = base + lane;
            bool push = false, inRange = false;
            int c2 = -1;
            if (j < e) {
                int c = col[j];
                if (c >= 0 && c < n) {  // columns beyond the matrix are remote (traverse :172)
                    c2 = invPerm[c];
                    if (stamp[c2] != stampVal) {
                        inRange = (c2 >= lo) && (c2 < hi);
                        if (inRange || (DMODE == DIST_TWO && uIn)) {
                            if (atomicExch(&stamp[c2], stampVal) != stampVal) {
                                push = true;
                                if (inRange) dist[c2] = lvl;
                            }
                        }
                    }
                }
            }
            unsigned m = __ballot_sync(0xffffffffu, push);
            if (m) {
                int leader = __ffs(m) - 1;
                int basePos = 0;
                unsigned mi = __ballot_sync(0xffffffffu, push && inRange);
                if (lane == leader) {
                    basePos = atomicAdd(&ctr[0], __popc(m));
                    if (mi) atomicAdd(&ctr[1], __popc(mi));
                }
                basePos = __shfl_sync(0xffffffffu, basePos, leader);
                if (push) next[basePos + __popc(m & ((1u << lane) - 1))] = c2;
            }
        }
    }
}

// Lowest row of [from,hi) that has no level yet.
__global__ void kIsland(const int *dist, int from, int hi, int *out) {
    int i = from + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < hi && dist[i] == -1) atomicMin(out, i);
}

// Per-level row and nnz counts plus the (level, row) sort pairs. With few
// levels (a BFS from a corner of a grid gives ~100) a global atomic per row
// serialises on a handful of addresses, so each block first counts into
// shared memory (grid-stride loop) and adds its non-zero bins once. With
// more levels than fit, rows of a warp that share a level are combined
// (match.any) before one lane adds for all of them.
constexpr int kHistSmemLevels = 4096;
constexpr int kNumSmsHint = 152;  // GB300; only sizes the grid-stride histogram grid

__global__ void kLevelHist(const int *__restrict__ dist, const int *__restrict__ perm, const int *__restrict__ rowPtr,
                           int lo, int hi, int numLevels, int *levelRow, int *levelNnz, int *keys, int *vals) {
    extern __shared__ int sh[];
    const bool smem = numLevels <= kHistSmemLevels;
    int *shRow = sh, *shNnz = sh + numLevels;
    if (smem) {
        for (int l = threadIdx.x; l < 2 * numLevels; l += blockDim.x) sh[l] = 0;
        __syncthreads();
    }
    const int stride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (int base = lo + blockIdx.x * blockDim.x; base < hi; base += stride) {
        int i = base + threadIdx.x;
        bool valid = i < hi;
        int d = -1, len = 0;
        if (valid) {
            d = dist[i];
            int pr = perm[i];
            len = rowPtr[pr + 1] - rowPtr[pr];
            keys[i - lo] = d;
            vals[i - lo] = i;
        }
        if (smem) {
            if (valid) {
                atomicAdd(&shRow[d], 1);
                atomicAdd(&shNnz[d], len);
            }
        } else {
            const unsigned act = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                const unsigned peers = __match_any_sync(act, d);
                const int sumLen = __reduce_add_sync(peers, len);
                if (lane == __ffs(peers) - 1) {
                    atomicAdd(&levelRow[d], __popc(peers));
                    atomicAdd(&levelNnz[d], sumLen);
                }
            }
        }
    }
    if (smem) {
        __syncthreads();
        for (int l = threadIdx.x; l < numLevels; l += blockDim.x) {
            if (shRow[l]) {
                atomicAdd(&levelRow[l], shRow[l]);
                atomicAdd(&levelNnz[l], shNnz[l]);
            }
        }
    }
}

// totalPerm'[i] = totalPerm[order[i-lo]]; totalInvPerm'[totalPerm'[i]] = i.
__global__ void kComposeGather(const int *__restrict__ perm, const int *__restrict__ order, int lo, int hi,
                               int *__restrict__ tmp) {
    int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < hi) tmp[i - lo] = perm[order[i - lo]];
}
__global__ void kComposeScatter(const int *__restrict__ tmp, int lo, int hi, int *__restrict__ perm,
                                int *__restrict__ invPerm) {
    int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < hi) {
        int p = tmp[i - lo];
        perm[i] = p;
        invPerm[p] = i;
    }
}

// Symmetrisation: for every off-diagonal (r,c) look for (c,r) in row c; if
// absent, c gets r appended. Pass 0 counts, pass 1 writes.
__global__ void kSymCount(const int *__restrict__ rowPtr, const int *__restrict__ col, int n, int *__restrict__ extra) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) {
        int c = col[j];
        if (c == r || c < 0 || c >= n) continue;
        bool has = false;
        for (int k = rowPtr[c]; k < rowPtr[c + 1]; ++k)
            if (col[k] == r) {
                has = true;
                break;
            }
        if (!has) atomicAdd(&extra[c], 1);
    }
}
__global__ void kSymFill(const int *__restrict__ rowPtr, const int *__restrict__ col, int n,
                         const int *__restrict__ newRowPtr, int *__restrict__ fill, int *__restrict__ newCol) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int o = newRowPtr[r];
    for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) newCol[o + j - rowPtr[r]] = col[j];
    for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) {
        int c = col[j];
        if (c == r || c < 0 || c >= n) continue;
        bool has = false;
        for (int k = rowPtr[c]; k < rowPtr[c + 1]; ++k)
            if (col[k] == r) {
                has = true;
                break;
            }
        if (!has) {
            int slot = atomicAdd(&fill[c], 1);
            newCol[newRowPtr[c] + (rowPtr[c + 1] - rowPtr[c]) + slot] = r;
        }
    }
}

int blocksFor(long long n, int t) { return (int)std::max<long long>(1, (n + t - 1) / t); }

}  // namespace

Engine::Engine(int nrow, int nthreads, int dist_, const int *rowPtr, const int *col, bool symmHint,
               const int *initPerm, const int *initInvPerm, int d2_, int lbTarget_, const Params &params_)
    : n(nrow), dist(dist_), requested(nthreads), d2(d2_), lbTarget(lbTarget_), params(params_) {
    if (nrow <= 0 || !rowPtr || !col) throw Error(RACE_ERR_INVALID_ARG, "empty matrix");
    if (dist_ != DIST_ONE && dist_ != DIST_TWO && dist_ != DIST_POWER) throw Error(RACE_ERR_INVALID_ARG, "bad dist");
    if (nthreads < 1) throw Error(RACE_ERR_INVALID_ARG, "nthreads must be >= 1");
    long long onnz = rowPtr[nrow];
    hRowPtr.assign(rowPtr, rowPtr + nrow + 1);
    hCol.assign(col, col + onnz);
    dRowPtr.upload(hRowPtr.data(), nrow + 1, stream);
    dCol.upload(hCol.data(), onnz, stream);
    nnz = onnz;
    // Graph ctor (graph_SoA.cpp:437-468): symmetrise unless the caller says
    // the pattern is symmetric. For matrix power the reference keeps the
    // pattern when RACE_MAX_RECURSION_STAGES is 0 (no recursion).
    bool needSym = !symmHint;
    if (dist_ == DIST_POWER && params.maxRecStages == 0) needSym = false;
    if (needSym) {
        DevBuf<int> extra(nrow), fill(nrow), newRowPtr(nrow + 1);
        RACE_CUDA(cudaMemsetAsync(extra.p, 0, sizeof(int) * nrow, stream));
        kSymCount<<<blocksFor(nrow, 256), 256, 0, stream>>>(dRowPtr.p, dCol.p, nrow, extra.p);
        std::vector<int> hExtra(nrow);
        RACE_CUDA(cudaMemcpyAsync(hExtra.data(), extra.p, sizeof(int) * nrow, cudaMemcpyDeviceToHost, stream));
        RACE_CUDA(cudaStreamSynchronize(stream));
        long long add = 0;
        for (int v : hExtra) add += v;
        if (add > 0) {
            std::vector<int> nrp(nrow + 1, 0);
            for (int r = 0; r < nrow; ++r) nrp[r + 1] = nrp[r] + (hRowPtr[r + 1] - hRowPtr[r]) + hExtra[r];
            newRowPtr.upload(nrp.data(), nrow + 1, stream);
            DevBuf<int> newCol(nrp[nrow]);
            RACE_CUDA(cudaMemsetAsync(fill.p, 0, sizeof(int) * nrow, stream));
            kSymFill<<<blocksFor(nrow, 256), 256, 0, stream>>>(dRowPtr.p, dCol.p, nrow, newRowPtr.p, fill.p, newCol.p);
            hRowPtr = nrp;
            hCol.resize(nrp[nrow]);
            RACE_CUDA(cudaMemcpyAsync(hCol.data(), newCol.p, sizeof(int) * (size_t)nrp[nrow], cudaMemcpyDeviceToHost,
                                      stream));
            dRowPtr = std::move(newRowPtr);
            dCol = std::move(newCol);
            nnz = nrp[nrow];
            RACE_CUDA(cudaStreamSynchronize(stream));
        }
    }
    // totalPerm = initPerm or identity (graph_SoA.cpp:63-79)
    hPerm.resize(nrow);
    hInvPerm.resize(nrow);
    if (initPerm && initInvPerm) {
        std::copy(initPerm, initPerm + nrow, hPerm.begin());
        std::copy(initInvPerm, initInvPerm + nrow, hInvPerm.begin());
    } else {
        std::iota(hPerm.begin(), hPerm.end(), 0);
        std::iota(hInvPerm.begin(), hInvPerm.end(), 0);
    }
    dPerm.upload(hPerm.data(), nrow, stream);
    dInvPerm.upload(hInvPerm.data(), nrow, stream);
    dDist.alloc(nrow);
    dStamp.alloc(nrow);
    RACE_CUDA(cudaMemsetAsync(dStamp.p, 0, sizeof(int) * nrow, stream));
    dQ0.alloc(nrow + 1);
    dQ1.alloc(nrow + 1);
    dCtr.alloc(4);
    dTmp.alloc(nrow);
    dKeys.alloc(nrow);
    dVals.alloc(nrow);
    dKeysOut.alloc(nrow);
    dValsOut.alloc(nrow);
    dStatus.alloc(4);
    if (const char *st = getenv("RACE_GPU_MPK_STRIDE")) mpkStride = atoi(st) == 1 ? 1 : 2;
    if (const char *sp = getenv("RACE_GPU_MPK_SPLIT")) mpkSplit = std::max(0, atoi(sp));
    if (const char *o = getenv("RACE_GPU_MPK_ORDER")) mpkOrder = std::string(o) == "group" ? 1 : 0;
    if (const char *r = getenv("RACE_GPU_MPK_RUN")) mpkRun = std::min(std::max(1, atoi(r)), kMpkMaxRunLen);
    if (const char *l = getenv("RACE_GPU_MPK_LAG")) mpkLag = std::max(0, atoi(l));
    if (const char *d = getenv("RACE_GPU_MPK_DIES")) mpkDieQueues = atoi(d) != 1;
    if (const char *h = getenv("RACE_GPU_MPK_HINTS")) mpkHints = atoi(h) ? 1 : 0;
    if (const char *c16 = getenv("RACE_GPU_MPK_COL16")) mpkCol16 = atoi(c16) != 0;
    if (const char *mr = getenv("RACE_GPU_SWEEP_MIDROW")) sweepMidRow = std::max(-1, atoi(mr));
    if (const char *ss = getenv("RACE_GPU_SWEEP_SELL")) sweepSell = atoi(ss) != 0;
    if (const char *sc = getenv("RACE_GPU_MPK_SCHEDULE"))
        mpkSchedule = std::string(sc) == "wavefront" ? RACE_MPK_WAVEFRONT
                      : std::string(sc) == "sweeps"  ? RACE_MPK_SWEEPS
                                                     : RACE_MPK_AUTO;
    if (const char *w = getenv("RACE_GPU_MPK_COL_WINDOW")) mpkColWindow = std::min(std::max(1, atoi(w)), kMpkColWindow);
    if (const char *b = getenv("RACE_GPU_MPK_CTAS")) mpkCtasPerSm = std::max(0, atoi(b));
    // Coloring traversals (distance-1/-2) of ranges shorter than
    // hostTraverseBelow run on the host (direction-optimised BFS, a few
    // microseconds for the many short ranges of a level recursion, where a
    // GPU traversal pays launches and host round trips per level). On a
    // GB300 host a graph with hub rows colours fastest entirely on the host
    // (4.2M-row power-law graph, distance 2: 1.9 s against 24 s with GPU
    // traversals); without hubs the GPU takes ranges from 2^20 rows on.
    int maxRowLen = 0;
    for (int r = 0; r < nrow; ++r) maxRowLen = std::max(maxRowLen, hRowPtr[r + 1] - hRowPtr[r]);
    hostTraverseBelow = maxRowLen > 1024 ? INT_MAX : (1 << 20);
    if (const char *ht = getenv("RACE_GPU_HOST_TRAVERSE_BELOW")) hostTraverseBelow = std::max(0, atoi(ht));
    if (const char *sm = getenv("RACE_GPU_SWEEP_MODE")) {
        std::string m(sm);
        sweepMode = m == "leaf" ? SWEEP_LEAF : m == "wave" ? SWEEP_WAVE : m == "gather" ? SWEEP_GATHER : SWEEP_AUTO;
    }
    RACE_CUDA(cudaStreamSynchronize(stream));
}

Engine::~Engine() {}

long long Engine::rangeNnz(int lo, int hi) const {
    long long s = 0;
    for (int r = lo; r < hi; ++r) {
        int p = hPerm[r];
        s += hRowPtr[p + 1] - hRowPtr[p];
    }
    return s;
}

void Engine::syncDevicePerm() {
    if (!devPermStale) return;
    dPerm.upload(hPerm.data(), n, stream);
    dInvPerm.upload(hInvPerm.data(), n, stream);
    RACE_CUDA(cudaStreamSynchronize(stream));
    devPermStale = false;
}

LevelData Engine::traverse(int lo, int hi, int mode, const std::string &mtxType) {
    LevelData ld;
    if (hi <= lo) return ld;
    const int len = hi - lo;
    cudaStream_t s = stream;
    // A short coloring range costs the GPU a few launches and host round
    // trips per level for little work: traverse it on the host instead.
    if (mtxType == "N" && (mode == DIST_ONE || mode == DIST_TWO) && len < hostTraverseBelow) {
        if (!traverseRangeHost(n, hRowPtr.data(), hCol.data(), hPerm, hInvPerm, lo, hi, mode, hostScratch, ld))
            throw Error(RACE_ERR_GRAPH_TRAVERSAL, "some rows went missing in BFS");
        devPermStale = true;
        return ld;
    }
    syncDevicePerm();
    int totalLevel = 0;
    if (mtxType == "N") {
        ++stamp;
        kFill<<<blocksFor(len, 256), 256, 0, s>>>(dDist.p, lo, hi, -1);
        kSetRoot<<<1, 1, 0, s>>>(dDist.p, dStamp.p, dQ0.p, lo, 0, stamp);
        int *front = dQ0.p, *next = dQ1.p;
        int fsize = 1;
        long long counter = 1;
        int currLvl = 0;
        int prevIslandStop = lo;
        int hctr[2];
        while (fsize > 0) {
            currLvl += 1;
            RACE_CUDA(cudaMemsetAsync(dCtr.p, 0, 2 * sizeof(int), s));
            int blocks = std::min(blocksFor((long long)fsize * 32, kWarpsPerBlock * 32), 152 * 16);
            if (mode == DIST_TWO)
                kExpand<DIST_TWO><<<blocks, kWarpsPerBlock * 32, 0, s>>>(dRowPtr.p, dCol.p, dPerm.p, dInvPerm.p, n,
                                                                          front, fsize, next, dCtr.p, dDist.p,
                                                                          dStamp.p, stamp, currLvl, lo, hi);
            else
                kExpand<DIST_ONE><<<blocks, kWarpsPerBlock * 32, 0, s>>>(dRowPtr.p, dCol.p, dPerm.p, dInvPerm.p, n,
                                                                          front, fsize, next, dCtr.p, dDist.p,
                                                                          dStamp.p, stamp, currLvl, lo, hi);
            RACE_CUDA(cudaMemcpyAsync(hctr, dCtr.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
            RACE_CUDA(cudaStreamSynchronize(s));
            fsize = hctr[0];
            counter += hctr[1];
            std::swap(front, next);
            if (fsize == 0 && counter != len) {
                // island restart (traverse_GAP_graphSoA.cpp:282-306)
                int big = INT32_MAX;
                RACE_CUDA(cudaMemcpyAsync(dCtr.p + 2, &big, sizeof(int), cudaMemcpyHostToDevice, s));
                kIsland<<<blocksFor(hi - prevIslandStop, 256), 256, 0, s>>>(dDist.p, prevIslandStop, hi, dCtr.p + 2);
                int isl;
                RACE_CUDA(cudaMemcpyAsync(&isl, dCtr.p + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
                RACE_CUDA(cudaStreamSynchronize(s));
                if (isl == INT32_MAX) throw Error(RACE_ERR_GRAPH_TRAVERSAL, "some rows went missing in BFS");
                if (mode != DIST_POWER) currLvl += 1;
                kSetRoot<<<1, 1, 0, s>>>(dDist.p, dStamp.p, front, isl, currLvl, stamp);
                fsize = 1;
                counter += 1;
                prevIslandStop = isl;
            }
        }
        totalLevel = currLvl;
    } else {
        // mtxType L/U: one row per level, forward or backward
        // (traverse_GAP_graphSoA.cpp:316-335), over the whole matrix.
        if (lo != 0 || hi != n) throw Error(RACE_ERR_NOT_IMPLEMENTED, "triangular MPK on a sub-range");
        std::vector<int> d(n);
        for (int i = 0; i < n; ++i) d[i] = (mtxType == "L") ? i : (n - 1) - i;
        RACE_CUDA(cudaMemcpyAsync(dDist.p, d.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        totalLevel = n;
    }

    ld.totalLevel = totalLevel;
    DevBuf<int> lr(std::max(totalLevel, 1)), ln(std::max(totalLevel, 1));
    RACE_CUDA(cudaMemsetAsync(lr.p, 0, sizeof(int) * lr.n, s));
    RACE_CUDA(cudaMemsetAsync(ln.p, 0, sizeof(int) * ln.n, s));
    {
        const size_t smem = totalLevel <= kHistSmemLevels ? sizeof(int) * 2 * totalLevel : 0;
        const int blocks = std::min(blocksFor(len, 256), smem ? 2 * kNumSmsHint : 1 << 30);
        kLevelHist<<<blocks, 256, smem, s>>>(dDist.p, dPerm.p, dRowPtr.p, lo, hi, totalLevel, lr.p, ln.p, dKeys.p,
                                             dVals.p);
    }
    ld.levelRow.resize(totalLevel);
    ld.levelNnz.resize(totalLevel);
    RACE_CUDA(cudaMemcpyAsync(ld.levelRow.data(), lr.p, sizeof(int) * totalLevel, cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaMemcpyAsync(ld.levelNnz.data(), ln.p, sizeof(int) * totalLevel, cudaMemcpyDeviceToHost, s));

    // stable sort by level (std::stable_sort in sortPerm_parallel, utility.h:60-68)
    int endBit = 1;
    while ((1LL << endBit) < (long long)totalLevel + 1 && endBit < 32) ++endBit;
    size_t tempBytes = 0;
    RACE_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, dKeys.p, dKeysOut.p, dVals.p, dValsOut.p, len, 0,
                                              endBit, s));
    dCubTemp.ensure(tempBytes);
    RACE_CUDA(cub::DeviceRadixSort::SortPairs(dCubTemp.p, tempBytes, dKeys.p, dKeysOut.p, dVals.p, dValsOut.p, len, 0,
                                              endBit, s));
    kComposeGather<<<blocksFor(len, 256), 256, 0, s>>>(dPerm.p, dValsOut.p, lo, hi, dTmp.p);
    kComposeScatter<<<blocksFor(len, 256), 256, 0, s>>>(dTmp.p, lo, hi, dPerm.p, dInvPerm.p);
    RACE_CUDA(cudaMemcpyAsync(hPerm.data() + lo, dPerm.p + lo, sizeof(int) * len, cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    for (int i = lo; i < hi; ++i) hInvPerm[hPerm[i]] = i;
    for (int l = 0; l < totalLevel; ++l) {
        ld.nrow += ld.levelRow[l];
        ld.nnz += ld.levelNnz[l];
    }
    return ld;
}

}  // namespace race
