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
//   runs with the kernel body's own operation order
//   (examples/src/helpers/kernels.cpp) — one thread per row up to 32
//   entries, one warp folding gathered entries in order up to 512 — so FP64
//   results are identical bit for bit to RACE's sequential walk, and rows
//   that RACE keeps in one long leaf still run in parallel when they do not
//   conflict. Rows above 512 entries get waves of their own, shared by all
//   warps of the grid (reassociated, within 1e-12).
// * Leaf mode (RACE_GPU_SWEEP_MODE=leaf). The flattened phases run with a
//   grid barrier between phases; one warp owns one leaf and walks its rows in
//   order, lanes splitting a row's non-zeros with warp-shuffle reductions.
//   Sums are reassociated (within 1e-12 relative of the sequential result).
//
// Neither mode needs atomics on the transpose scatter: the coloring (leaf
// mode) or the wave plan (wave mode) gives every written entry one writer.
#include <algorithm>
#include <cstdlib>

#include <cuda_bf16.h>

#include "engine.h"

namespace race {
namespace {

constexpr int kSweepThreads = 256;
constexpr int kWarps = kSweepThreads / 32;
// Wave mode: one block per SM; the grid barrier costs one arrival per block,
// so the threads a wave can use grow with the block size at no barrier cost.
constexpr int kWaveThreads = 256;
constexpr int kWaveBlocksPerSm = 1;

__device__ __forceinline__ unsigned ldAcquireU(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier on a monotonic arrival counter (bar[0], zeroed at launch).
// Every block arrives once per barrier and no block can arrive at the next
// barrier before all have arrived at this one, so the arrivals of barrier k
// are k*G+1 .. (k+1)*G (G = gridDim.x): a block's own arrival number gives
// the count to wait for, with no reset or generation word (one atomic and
// the polling, instead of three dependent round trips). Returns false (and
// sets *status) if the wait exceeded the spin limit.
__device__ bool gridBarrier(unsigned *bar, int *status) {
    __shared__ int sOk;
    __syncthreads();
    if (threadIdx.x == 0) {
        sOk = 1;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u) + 1;
        const unsigned target = ((arrived - 1) / gridDim.x + 1) * gridDim.x;
        long long spins = 0;
        while (ldAcquireU(bar) < target) {
            if (++spins > kSpinLimit) {
                atomicCAS(status, DEV_OK, DEV_WAIT_TIMEOUT);
                sOk = 0;
                break;
            }
            __nanosleep(32);
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
    // wave mode, rows above kHugeRow (see DevWaves)
    const unsigned char *waveHuge;
    const int *segFirst, *segPos, *segBeg, *segEnd;
    double *segScratch;
    int numSegs;
    int midRow;  // wave mode: rows of up to midRow entries run one thread each, longer ones a warp
    // wave mode: SELL copy of the thread rows (DevWaves), or null
    const int *waveChunk;
    const long long *chunkOff;
    const void *sellVal;
    const int *sellCol;
};

// Entries [jb, e) of a row in order, one thread: columns and values in
// batches of 8, then the batch's gathers of x, then f(value, x[col]) in the
// row's order (the loads of a batch are in flight together; the chain of f
// is the sequential one).
template <typename VT, typename XT, typename F>
__device__ __forceinline__ void serialRow(const SweepArgs &a, int jb, int e, F &&f) {
    const VT *val = (const VT *)a.val;
    const XT *x = (const XT *)a.x;
    int j = jb;
    for (; j + 8 <= e; j += 8) {
        int c[8];
        XT v[8], xv[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            c[k] = a.col[j + k];
            v[k] = ld<VT, XT>(val, j + k);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) xv[k] = x[c[k]];
#pragma unroll
        for (int k = 0; k < 8; ++k) f(v[k], xv[k]);
    }
    for (; j < e; ++j) f(ld<VT, XT>(val, j), x[a.col[j]]);
}

// The four values of an entry group of the SELL copy (16-byte aligned).
__device__ __forceinline__ void groupVals(const double *v, double out[4]) {
    const double2 a = *(const double2 *)v, b = *(const double2 *)(v + 2);
    out[0] = a.x;
    out[1] = a.y;
    out[2] = b.x;
    out[3] = b.y;
}
__device__ __forceinline__ void groupVals(const float *v, float out[4]) {
    const float4 a = *(const float4 *)v;
    out[0] = a.x;
    out[1] = a.y;
    out[2] = a.z;
    out[3] = a.w;
}
__device__ __forceinline__ void groupVals(const __nv_bfloat16 *v, float out[4]) {
    const uint2 a = *(const uint2 *)v;
    out[0] = __uint_as_float(a.x << 16);
    out[1] = __uint_as_float(a.x & 0xffff0000u);
    out[2] = __uint_as_float(a.y << 16);
    out[3] = __uint_as_float(a.y & 0xffff0000u);
}
__device__ __forceinline__ int comp(const int4 &c, int q) { return q == 0 ? c.x : q == 1 ? c.y : q == 2 ? c.z : c.w; }

// The entries of one row, as the row bodies below see them: entry k
// (0-based, CRS order) and an in-order walk sum(x, k0, f) calling
// f(value, x[col]) for entries k0..len-1. CrsRow reads the caller's CRS
// (loads in batches of 8, serialRow); SellRow reads the SELL copy, one
// group of four entries per vector load of values and columns.
template <typename VT, typename XT>
struct CrsRow {
    const int *col;
    const VT *val;
    int s, len;
    __device__ XT v(int k) const { return ld<VT, XT>(val, s + k); }
    __device__ int c(int k) const { return col[s + k]; }
    template <typename F>
    __device__ void sum(const SweepArgs &a, int k0, F &&f) const {
        serialRow<VT, XT>(a, s + k0, s + len, f);
    }
};

template <typename VT, typename XT>
struct SellRow {
    const int *col;
    const VT *val;
    long long off;  // the chunk's first slot
    int lane, len;
    __device__ long long slot(int k) const { return off + 32LL * (k & ~3) + 4 * lane + (k & 3); }
    __device__ XT v(int k) const { return ld<VT, XT>(val, slot(k)); }
    __device__ int c(int k) const { return col[slot(k)]; }
    template <typename F>
    __device__ void sum(const SweepArgs &a, int k0, F &&f) const {
        const XT *x = (const XT *)a.x;
        for (int g = k0 & ~3; g < len; g += 4) {
            const long long o = off + 32LL * g + 4 * lane;
            const int4 cc = *(const int4 *)(col + o);
            XT vv[4], xv[4];
            groupVals(val + o, vv);
            const int lo = max(g, k0) - g, hi = min(len - g, 4);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (q >= lo && q < hi) xv[q] = x[comp(cc, q)];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (q >= lo && q < hi) f(vv[q], xv[q]);
        }
    }
};

// One row with the kernel body's own operation order (thread per row).
template <typename VT, typename XT, typename Row>
__device__ __forceinline__ void rowSerial(const SweepArgs &a, int r, const Row &row) {
    XT *x = (XT *)a.x;
    XT *b = (XT *)a.b;
    const int len = row.len;
    switch (a.kernel) {
    case RACE_K_SPMV: {  // kernels.cpp:5-15
        XT t = XT(0);
        row.sum(a, 0, [&](XT v, XT xv) { t = mac(v, xv, t); });
        b[r] = t;
        break;
    }
    case RACE_K_SPMTV: {  // kernels.cpp:107-115
        const XT xr = x[r];
        for (int k = 0; k < len; ++k) {
            const int c = row.c(k);
            b[c] = mac(row.v(k), xr, b[c]);
        }
        break;
    }
    case RACE_K_SYMMSPMV: {  // kernels.cpp:403-417
        if (len == 0) break;  // no diagonal entry to read (the bodies assume one)
        const XT xr = x[r];
        b[r] = mac(row.v(0), xr, b[r]);
        XT t = XT(0);
        for (int k = 1; k < len; ++k) {
            const int c = row.c(k);
            const XT v = row.v(k);
            t = mac(v, x[c], t);
            b[c] = mac(v, xr, b[c]);
        }
        b[r] += t;
        break;
    }
    case RACE_K_GS: {  // kernels.cpp:174-186
        if (len == 0) break;  // no diagonal entry to divide by
        XT t = b[r];
        row.sum(a, 1, [&](XT v, XT xv) { t = mac(-v, xv, t); });
        x[r] = t / row.v(0);
        break;
    }
    case RACE_K_KACZ: {  // kernels.cpp:285-302
        XT nrm = XT(0), sc = -b[r];
        row.sum(a, 0, [&](XT v, XT xv) {
            sc = mac(v, xv, sc);
            nrm = mac(v, v, nrm);
        });
        sc /= nrm;
        for (int k = 0; k < len; ++k) {
            const int c = row.c(k);
            x[c] = mac(-sc, row.v(k), x[c]);
        }
        break;
    }
    default: break;
    }
}

// Wave mode keeps the sequential order (bit-exact) for rows of up to
// kHugeRow entries: up to SweepArgs::midRow (the engine's sweepMidRow) one
// thread, above that one warp (rowWarpExact): one thread walking a few
// hundred entries would pay a dependent gather per few entries and make its
// row the wave's critical path. Longer rows are reassociated (hugeWave).

template <typename VT, typename XT>
__device__ __forceinline__ void rowWarp(const SweepArgs &a, int row, int lane);

// Rows above this many entries (one reaches a quarter of a million in a
// power-law graph) get waves of their own in which all warps of the grid
// share them: segments of kHugeSeg entries are summed by one warp each, a
// grid barrier, then one warp per row combines its segments in order and
// applies the kernel's row update (Kaczmarz: a second barrier, then the
// scatter with the row's scale). Sums are reassociated, deterministically.
constexpr int kHugeRow = 512;
constexpr int kHugeSeg = 256;

template <typename VT, typename XT>
__device__ bool hugeWave(const SweepArgs &a, int r0, int r1, int gw, int nw, int lane);

// Entries [jb, e) of a row, folded in order by every lane of a warp: each
// round gathers up to kFoldBlocks x 32 entries at once (all loads in
// flight), stages the (value, x) pairs in the warp's shared memory, then
// every lane applies f(value, x[col]) to them in the row's order, reading
// the pairs as broadcasts (the reads do not depend on the running sum, so
// they pipeline), so every lane runs the same sequential chain. Called by
// whole warps of kWaveSweep only.
constexpr int kFoldBlocks = 8;

template <typename XT>
struct FoldStage {
    XT v[kWaveThreads / 32][32 * kFoldBlocks];
    XT x[kWaveThreads / 32][32 * kFoldBlocks];
};

// One stage per block and accumulation type, shared by every fold body.
template <typename XT>
__device__ __forceinline__ FoldStage<XT> &foldStage() {
    __shared__ FoldStage<XT> st;
    return st;
}

template <typename VT, typename XT, typename F>
__device__ __forceinline__ void foldRow(const SweepArgs &a, int jb, int e, int lane, F &&f) {
    FoldStage<XT> &st = foldStage<XT>();
    const VT *val = (const VT *)a.val;
    const XT *x = (const XT *)a.x;
    const int w = threadIdx.x >> 5;
    for (int jr = jb; jr < e; jr += 32 * kFoldBlocks) {
        XT v[kFoldBlocks], xv[kFoldBlocks];
#pragma unroll
        for (int k = 0; k < kFoldBlocks; ++k) {
            const int j = jr + 32 * k + lane;
            const bool ok = j < e;
            v[k] = ok ? ld<VT, XT>(val, j) : XT(0);
            xv[k] = ok ? x[a.col[j]] : XT(0);
        }
        __syncwarp();  // the previous round's reads are done
#pragma unroll
        for (int k = 0; k < kFoldBlocks; ++k) {
            st.v[w][32 * k + lane] = v[k];
            st.x[w][32 * k + lane] = xv[k];
        }
        __syncwarp();
        const int m = min(32 * kFoldBlocks, e - jr);
#pragma unroll 8
        for (int q = 0; q < m; ++q) f(st.v[w][q], st.x[w][q]);
    }
}

// A row with the kernel body's own operation order, run by a warp (rows of
// midRow+1..kHugeRow entries): sums through foldRow, identical bit for bit
// to rowSerial; scatters (one distinct column per entry) run lane-parallel
// with the same per-entry arithmetic.
template <typename VT, typename XT>
__device__ __forceinline__ void rowWarpExact(const SweepArgs &a, int r, int lane) {
    const VT *val = (const VT *)a.val;
    XT *x = (XT *)a.x;
    XT *b = (XT *)a.b;
    const int s = a.rowPtr[r], e = a.rowPtr[r + 1];
    switch (a.kernel) {
    case RACE_K_SPMV: {
        XT t = XT(0);
        foldRow<VT, XT>(a, s, e, lane, [&](XT v, XT xv) { t = mac(v, xv, t); });
        if (lane == 0) b[r] = t;
        break;
    }
    case RACE_K_SPMTV: {
        const XT xr = x[r];
        for (int j = s + lane; j < e; j += 32) {
            const int c = a.col[j];
            b[c] = mac(ld<VT, XT>(val, j), xr, b[c]);
        }
        break;
    }
    case RACE_K_SYMMSPMV: {
        // the diagonal update and the final b[r] += t touch only b[r]; the
        // scatter only columns above r, so lane 0 does both at the end
        const XT xr = x[r];
        XT t = XT(0);
        foldRow<VT, XT>(a, s + 1, e, lane, [&](XT v, XT xv) { t = mac(v, xv, t); });
        for (int j = s + 1 + lane; j < e; j += 32) {
            const int c = a.col[j];
            b[c] = mac(ld<VT, XT>(val, j), xr, b[c]);
        }
        if (lane == 0) {
            b[r] = mac(ld<VT, XT>(val, s), xr, b[r]);
            b[r] += t;
        }
        break;
    }
    case RACE_K_GS: {
        XT t = b[r];
        foldRow<VT, XT>(a, s + 1, e, lane, [&](XT v, XT xv) { t = mac(-v, xv, t); });
        if (lane == 0) x[r] = t / ld<VT, XT>(val, s);
        break;
    }
    case RACE_K_KACZ: {
        XT nrm = XT(0), sc = -b[r];
        foldRow<VT, XT>(a, s, e, lane, [&](XT v, XT xv) {
            sc = mac(v, xv, sc);
            nrm = mac(v, v, nrm);
        });
        sc /= nrm;
        __syncwarp();  // every lane's reads of x precede the scatter
        for (int j = s + lane; j < e; j += 32) {
            const int c = a.col[j];
            x[c] = mac(-sc, ld<VT, XT>(val, j), x[c]);
        }
        break;
    }
    default: break;
    }
}

template <typename VT, typename XT>
__global__ void __launch_bounds__(kWaveThreads, 1) kWaveSweep(SweepArgs a) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nt = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = tid >> 5, nw = nt >> 5;
    for (int w = 0; w < a.num; ++w) {
        const int r0 = a.ptr[w], r1 = a.ptr[w + 1];
        if (a.waveHuge && a.waveHuge[w]) {
            if (!hugeWave<VT, XT>(a, r0, r1, gw, nw, lane)) return;
            if (w + 1 < a.num && !gridBarrier(a.bar, a.status)) return;
            continue;
        }
        for (int i = r0 + tid; i < r1; i += nt) {
            const int r = a.rows[i];
            const int rs = a.rowPtr[r], len = a.rowPtr[r + 1] - rs;
            if (len > a.midRow) continue;
            if (a.sellCol)  // position i - r0 of the wave: chunk (i - r0) / 32, lane (i - r0) % 32
                rowSerial<VT, XT>(a, r,
                                  SellRow<VT, XT>{a.sellCol, (const VT *)a.sellVal,
                                                  a.chunkOff[a.waveChunk[w] + ((i - r0) >> 5)], (i - r0) & 31, len});
            else
                rowSerial<VT, XT>(a, r, CrsRow<VT, XT>{a.col, (const VT *)a.val, rs, len});
        }
        // longer rows of this wave: one warp each, distributed over all warps
        // of the grid (rows of a wave are independent, so the passes may
        // interleave)
        for (int i = r0 + gw; i < r1; i += nw) {
            const int r = a.rows[i];
            const int len = a.rowPtr[r + 1] - a.rowPtr[r];
            if (len > kHugeRow)
                rowWarp<VT, XT>(a, r, lane);  // not reached: the plan gives such rows huge waves
            else if (len > a.midRow)
                rowWarpExact<VT, XT>(a, r, lane);
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
__device__ bool hugeWave(const SweepArgs &a, int r0, int r1, int gw, int nw, int lane) {
    const VT *val = (const VT *)a.val;
    XT *x = (XT *)a.x;
    XT *b = (XT *)a.b;
    double *dot = a.segScratch, *nrm = a.segScratch + a.numSegs, *scl = a.segScratch + 2 * a.numSegs;
    const int g0 = a.segFirst[r0], g1 = a.segFirst[r1];
    // 1. segment sums, and the scatters that need no row result
    for (int g = g0 + gw; g < g1; g += nw) {
        const int r = a.rows[a.segPos[g]];
        const int s = a.rowPtr[r], jb = a.segBeg[g], je = a.segEnd[g];
        XT t = XT(0), q = XT(0);
        switch (a.kernel) {
        case RACE_K_SPMV:
        case RACE_K_GS:
        case RACE_K_KACZ: {
            // a segment holds at most 8 entries per lane: gather all, then sum
            constexpr int kPer = kHugeSeg / 32;
            XT v[kPer], xv[kPer];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int j = jb + lane + 32 * k;
                const bool ok = j < je && !(a.kernel == RACE_K_GS && j == s);
                v[k] = ok ? ld<VT, XT>(val, j) : XT(0);
                xv[k] = ok ? x[a.col[j]] : XT(0);
            }
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                t = mac(v[k], xv[k], t);
                q = mac(v[k], v[k], q);
            }
            break;
        }
        case RACE_K_SYMMSPMV: {
            const XT xr = x[r];
            for (int j = jb + lane; j < je; j += 32)
                if (j != s) {
                    const int c = a.col[j];
                    const XT v = ld<VT, XT>(val, j);
                    t = mac(v, x[c], t);
                    b[c] = mac(v, xr, b[c]);
                }
            break;
        }
        case RACE_K_SPMTV: {
            const XT xr = x[r];
            for (int j = jb + lane; j < je; j += 32) {
                const int c = a.col[j];
                b[c] = mac(ld<VT, XT>(val, j), xr, b[c]);
            }
            break;
        }
        default: break;
        }
        t = warpSum(t);
        q = warpSum(q);
        if (lane == 0) {
            dot[g] = (double)t;
            nrm[g] = (double)q;
        }
    }
    if (a.kernel == RACE_K_SPMTV) return true;
    if (!gridBarrier(a.bar, a.status)) return false;
    // 2. one warp per row: its segments in order, then the row update
    for (int i = r0 + gw; i < r1; i += nw) {
        const int r = a.rows[i];
        XT S = XT(0), Q = XT(0);
        for (int g = a.segFirst[i] + lane; g < a.segFirst[i + 1]; g += 32) {
            S += (XT)dot[g];
            Q += (XT)nrm[g];
        }
        S = warpSum(S);
        Q = warpSum(Q);
        if (lane == 0) {
            const int s = a.rowPtr[r];
            switch (a.kernel) {
            case RACE_K_SPMV: b[r] = S; break;
            case RACE_K_GS: x[r] = (b[r] - S) / ld<VT, XT>(val, s); break;
            case RACE_K_SYMMSPMV: b[r] = mac(ld<VT, XT>(val, s), x[r], b[r]) + S; break;
            case RACE_K_KACZ: scl[a.segFirst[i]] = (double)((S - b[r]) / Q); break;
            default: break;
            }
        }
    }
    if (a.kernel != RACE_K_KACZ) return true;
    if (!gridBarrier(a.bar, a.status)) return false;
    // 3. Kaczmarz scatter with the row's scale
    for (int g = g0 + gw; g < g1; g += nw) {
        const XT sc = (XT)scl[a.segFirst[a.segPos[g]]];
        for (int j = a.segBeg[g] + lane; j < a.segEnd[g]; j += 32) {
            const int c = a.col[j];
            x[c] = mac(-sc, ld<VT, XT>(val, j), x[c]);
        }
    }
    return true;
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
        if (e == s) break;  // no diagonal entry to read
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
        if (e == s) break;  // no diagonal entry to divide by
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
int coopBlocks(K kernel, int want, int capPerSm = 0, int threads = kSweepThreads) {
    int dev = 0, sms = 0, occ = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, 0));
    occ = std::max(occ, 1);
    if (capPerSm > 0) occ = std::min(occ, capPerSm);
    return std::max(1, std::min(sms * occ, want));
}

// CRS -> SELL copy of the thread rows of a wave plan (DevWaves): one warp
// per chunk, lane l the chunk's l-th position; rows above midRow entries
// (run by a warp from the CRS) and positions past the wave are padding
// (value 0, column the row itself or 0).
template <typename VT>
__global__ void kWaveToSell(const int *__restrict__ rowPtr, const int *__restrict__ col, const VT *__restrict__ val,
                            const int *__restrict__ rows, const int *__restrict__ chunkPos,
                            const int *__restrict__ chunkEnd, const int *__restrict__ chunkLen,
                            const long long *__restrict__ chunkOff, int numChunks, int midRow, VT *__restrict__ sval,
                            int *__restrict__ scol) {
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= numChunks) return;
    const int lane = threadIdx.x & 31;
    const int p = chunkPos[c] + lane;
    const bool live = p < chunkEnd[c];
    const int r = live ? rows[p] : 0;
    const int s = live ? rowPtr[r] : 0;
    int len = live ? rowPtr[r + 1] - s : 0;
    if (len > midRow) len = 0;
    for (int k = 0; k < chunkLen[c]; ++k) {
        const long long o = chunkOff[c] + 32LL * (k & ~3) + 4 * lane + (k & 3);
        sval[o] = k < len ? val[s + k] : VT(0);
        scol[o] = k < len ? col[s + k] : r;
    }
}

// Blocks per SM of the wave-mode grid. Every wave ends with a grid barrier
// whose cost grows with the number of blocks, while a wave rarely holds more
// rows than a few blocks per SM cover (256 threads each, grid-stride loops
// take the rest). RACE_GPU_SWEEP_BLOCKS_PER_SM overrides it (0: occupancy).
int waveBlocksPerSm() {
    static const int v = [] {
        const char *s = getenv("RACE_GPU_SWEEP_BLOCKS_PER_SM");
        return s ? atoi(s) : kWaveBlocksPerSm;
    }();
    return v;
}

template <typename VT, typename XT>
void launch(bool waveMode, SweepArgs &a, int maxWork, cudaStream_t s) {
    void *args[] = {&a};
    if (waveMode) {
        int blocks = coopBlocks(kWaveSweep<VT, XT>, ceilDiv(maxWork, kWaveThreads), waveBlocksPerSm(), kWaveThreads);
        RACE_CUDA(cudaLaunchCooperativeKernel((void *)kWaveSweep<VT, XT>, blocks, kWaveThreads, args, 0, s));
    } else {
        int blocks = coopBlocks(kLeafSweep<VT, XT>, ceilDiv(maxWork, kWarps));
        RACE_CUDA(cudaLaunchCooperativeKernel((void *)kLeafSweep<VT, XT>, blocks, kSweepThreads, args, 0, s));
    }
}

// Gather execution (RACE_SWEEP_GATHER): one thread per entry of b, which
// replays the updates RACE's sequential walk makes to it, in that walk's
// order (GatherPlan, waves.h), with the kernel bodies' own operations, so
// the results equal the wave executor's bit for bit; no phases, no grid
// barriers. SpMV needs no plan: its rows are independent.
template <typename VT, typename XT>
__global__ void kGather(int kernel, int n, const int *__restrict__ ptr, const int *__restrict__ entry,
                        const int *__restrict__ src, const int *__restrict__ rowPtr, const int *__restrict__ col,
                        const void *val_, const XT *__restrict__ x, XT *__restrict__ b) {
    const VT *val = (const VT *)val_;
    for (int y = blockIdx.x * blockDim.x + threadIdx.x; y < n; y += gridDim.x * blockDim.x) {
        if (kernel == RACE_K_SPMV) {  // kernels.cpp:5-15
            XT t = XT(0);
            for (int j = rowPtr[y]; j < rowPtr[y + 1]; ++j) t = mac(ld<VT, XT>(val, j), x[col[j]], t);
            b[y] = t;
            continue;
        }
        XT acc = b[y];
        for (int k = ptr[y]; k < ptr[y + 1]; ++k) {
            const int e = entry[k];
            if (e >= 0) {  // b[y] += a x[src] of another row (SpMTV :107-115, SymmSpMV :403-417)
                acc = mac(ld<VT, XT>(val, e), x[src[k]], acc);
            } else {  // row y's own SymmSpMV update: diagonal, then its off-diagonal dot product
                const int s = rowPtr[y], end = rowPtr[y + 1];
                if (end == s) continue;  // no diagonal entry to read
                acc = mac(ld<VT, XT>(val, s), x[y], acc);
                XT t = XT(0);
                for (int j = s + 1; j < end; ++j) t = mac(ld<VT, XT>(val, j), x[col[j]], t);
                acc += t;
            }
        }
        b[y] = acc;
    }
}

template <typename VT, typename XT>
void launchGather(const FuncEntry &f, const DevGather &g, cudaStream_t s) {
    const race_operands &o = f.ops;
    const int n = o.n;
    if (n == 0) return;
    const int blocks = std::min(ceilDiv(n, 256), 152 * 16);
    kGather<VT, XT><<<blocks, 256, 0, s>>>(f.kernel, n, g.ptr.p, g.entry.p, g.row.p, o.rowPtr, o.col, o.val,
                                            (const XT *)o.x, (XT *)o.b);
    RACE_CUDA(cudaGetLastError());
}

void runGather(Engine &e, FuncEntry &f, int dir) {
    const race_operands &ops = f.ops;
    DevGather &g = f.gather[dir];
    if (!g.built && f.kernel != RACE_K_SPMV) {
        const int n = ops.n;
        std::vector<int> rp(n + 1);
        RACE_CUDA(cudaMemcpyAsync(rp.data(), ops.rowPtr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, e.stream));
        RACE_CUDA(cudaStreamSynchronize(e.stream));
        std::vector<int> cl(std::max(rp[n], 1));
        RACE_CUDA(cudaMemcpyAsync(cl.data(), ops.col, sizeof(int) * (size_t)rp[n], cudaMemcpyDeviceToHost, e.stream));
        RACE_CUDA(cudaStreamSynchronize(e.stream));
        const GatherPlan gp = buildGatherPlan(f.kernel, n, rp.data(), cl.data(), e.phases[dir]);
        g.ptr.upload(gp.ptr.data(), gp.ptr.size(), e.stream);
        g.entry.upload(gp.entry.empty() ? nullptr : gp.entry.data(), std::max<size_t>(gp.entry.size(), 1), e.stream);
        g.row.upload(gp.row.empty() ? nullptr : gp.row.data(), std::max<size_t>(gp.row.size(), 1), e.stream);
        RACE_CUDA(cudaStreamSynchronize(e.stream));
        g.built = true;
    }
    if (ops.vec_type == RACE_VAL_F64) {
        if (ops.val_type != RACE_VAL_F64) throw Error(RACE_ERR_INVALID_ARG, "FP64 vectors need FP64 values");
        launchGather<double, double>(f, g, e.stream);
    } else if (ops.vec_type == RACE_VAL_F32) {
        if (ops.val_type == RACE_VAL_F32)
            launchGather<float, float>(f, g, e.stream);
        else if (ops.val_type == RACE_VAL_BF16)
            launchGather<__nv_bfloat16, float>(f, g, e.stream);
        else
            throw Error(RACE_ERR_INVALID_ARG, "FP32 vectors need FP32 or BF16 values");
    } else {
        throw Error(RACE_ERR_INVALID_ARG, "unknown vector type");
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

// Thread-row limit of a sweep function (Engine::sweepMidRow).
static int midRowOf(const Engine &e, const FuncEntry &f) {
    const int m = e.sweepMidRow >= 0 ? e.sweepMidRow : (f.ops.vec_type == RACE_VAL_F64 ? 16 : 8);
    return std::min(m, kHugeRow);
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
        // Rows above kHugeRow leave their wave for a wave of their own just
        // before it (rows of a wave are independent, so any split keeps the
        // order valid); their segments are listed per plan position.
        std::vector<int> ptr{0}, rows, segFirst{0}, segPos, segBeg, segEnd;
        std::vector<unsigned char> huge;
        std::vector<int> normal;
        for (int w = 0; w < wp.numWaves(); ++w) {
            normal.clear();
            const size_t hugeStart = rows.size();
            for (int i = wp.wavePtr[w]; i < wp.wavePtr[w + 1]; ++i) {
                const int r = wp.rows[i];
                if (rp[r + 1] - rp[r] <= kHugeRow) {
                    normal.push_back(r);
                    continue;
                }
                const int pos = (int)rows.size();
                rows.push_back(r);
                for (int j = rp[r]; j < rp[r + 1]; j += kHugeSeg) {
                    segPos.push_back(pos);
                    segBeg.push_back(j);
                    segEnd.push_back(std::min(rp[r + 1], j + kHugeSeg));
                }
                segFirst.push_back((int)segPos.size());
            }
            if (rows.size() > hugeStart) {
                ptr.push_back((int)rows.size());
                huge.push_back(1);
            }
            if (!normal.empty()) {
                for (int r : normal) {
                    rows.push_back(r);
                    segFirst.push_back((int)segPos.size());
                }
                ptr.push_back((int)rows.size());
                huge.push_back(0);
            }
        }
        DevWaves &w = f.waves[dir];
        // SELL copy of the thread rows: a wave's rows are independent, so
        // they are sorted by length (longest first, then by row) and cut
        // into chunks of 32 positions whose width is their longest thread
        // row (SELL-C-sigma with sigma = the wave)
        const int mid = midRowOf(e, f);
        std::vector<int> waveChunk{0}, cPos, cEnd, cLen;
        std::vector<long long> cOff;
        long long slots = 0;
        if (e.sweepSell) {
            auto rowLen = [&](int r) { return rp[r + 1] - rp[r]; };
            for (size_t wi = 0; wi < huge.size(); ++wi) {
                if (!huge[wi]) {
                    std::sort(rows.begin() + ptr[wi], rows.begin() + ptr[wi + 1], [&](int x, int y) {
                        return rowLen(x) != rowLen(y) ? rowLen(x) > rowLen(y) : x < y;
                    });
                    for (int p0 = ptr[wi]; p0 < ptr[wi + 1]; p0 += 32) {
                        const int p1 = std::min(p0 + 32, ptr[wi + 1]);
                        int L = 0;
                        for (int q = p0; q < p1; ++q)
                            if (rowLen(rows[q]) <= mid) L = std::max(L, rowLen(rows[q]));
                        L = (L + 3) & ~3;
                        cPos.push_back(p0);
                        cEnd.push_back(p1);
                        cLen.push_back(L);
                        cOff.push_back(slots);
                        slots += 32LL * L;
                    }
                }
                waveChunk.push_back((int)cPos.size());
            }
        }
        w.numWaves = (int)huge.size();
        w.maxRows = 0;
        for (int i = 0; i < w.numWaves; ++i) w.maxRows = std::max(w.maxRows, ptr[i + 1] - ptr[i]);
        w.numSegs = (int)segPos.size();
        w.wavePtr.upload(ptr.data(), ptr.size(), e.stream);
        w.rows.upload(rows.empty() ? nullptr : rows.data(), std::max<size_t>(rows.size(), 1), e.stream);
        w.waveHuge.upload(huge.empty() ? nullptr : huge.data(), std::max<size_t>(huge.size(), 1), e.stream);
        w.segFirst.upload(segFirst.data(), segFirst.size(), e.stream);
        w.segPos.upload(segPos.empty() ? nullptr : segPos.data(), std::max<size_t>(segPos.size(), 1), e.stream);
        w.segBeg.upload(segBeg.empty() ? nullptr : segBeg.data(), std::max<size_t>(segBeg.size(), 1), e.stream);
        w.segEnd.upload(segEnd.empty() ? nullptr : segEnd.data(), std::max<size_t>(segEnd.size(), 1), e.stream);
        w.segScratch.alloc(std::max<size_t>(3 * segPos.size(), 1));
        w.sell = e.sweepSell;
        w.sellMidRow = mid;
        w.sellSlots = slots;
        if (w.sell) {
            const int C = (int)cPos.size();
            w.waveChunk.upload(waveChunk.data(), waveChunk.size(), e.stream);
            w.chunkOff.upload(cOff.empty() ? nullptr : cOff.data(), std::max(C, 1), e.stream);
            DevBuf<int> dPos, dEnd, dLen;
            dPos.upload(cPos.empty() ? nullptr : cPos.data(), std::max(C, 1), e.stream);
            dEnd.upload(cEnd.empty() ? nullptr : cEnd.data(), std::max(C, 1), e.stream);
            dLen.upload(cLen.empty() ? nullptr : cLen.data(), std::max(C, 1), e.stream);
            const size_t vb = f.ops.val_type == RACE_VAL_F64 ? 8 : f.ops.val_type == RACE_VAL_F32 ? 4 : 2;
            w.sellVal.alloc(std::max<long long>(slots, 4) * vb);
            w.sellCol.alloc(std::max<long long>(slots, 4));
            if (C > 0) {
                const int blocks = ceilDiv(C, 8);
                switch (f.ops.val_type) {
                case RACE_VAL_F64:
                    kWaveToSell<double><<<blocks, 256, 0, e.stream>>>(f.ops.rowPtr, f.ops.col, (const double *)f.ops.val,
                                                                     w.rows.p, dPos.p, dEnd.p, dLen.p, w.chunkOff.p, C,
                                                                     mid, (double *)w.sellVal.p, w.sellCol.p);
                    break;
                case RACE_VAL_F32:
                    kWaveToSell<float><<<blocks, 256, 0, e.stream>>>(f.ops.rowPtr, f.ops.col, (const float *)f.ops.val,
                                                                    w.rows.p, dPos.p, dEnd.p, dLen.p, w.chunkOff.p, C,
                                                                    mid, (float *)w.sellVal.p, w.sellCol.p);
                    break;
                case RACE_VAL_BF16:
                    kWaveToSell<__nv_bfloat16><<<blocks, 256, 0, e.stream>>>(
                        f.ops.rowPtr, f.ops.col, (const __nv_bfloat16 *)f.ops.val, w.rows.p, dPos.p, dEnd.p, dLen.p,
                        w.chunkOff.p, C, mid, (__nv_bfloat16 *)w.sellVal.p, w.sellCol.p);
                    break;
                default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
                }
                RACE_CUDA(cudaGetLastError());
            }
            RACE_CUDA(cudaStreamSynchronize(e.stream));  // the temporaries go out of scope
        }
    }
    RACE_CUDA(cudaStreamSynchronize(e.stream));
}

bool usesGather(const Engine &e, const FuncEntry &f) {
    return (e.sweepMode == SWEEP_GATHER || e.sweepMode == SWEEP_AUTO) &&
           (f.kernel == RACE_K_SPMV || f.kernel == RACE_K_SPMTV || f.kernel == RACE_K_SYMMSPMV);
}

void runSweep(Engine &e, FuncEntry &f, bool rev) {
    const race_operands &ops = f.ops;
    const int dir = rev ? 1 : 0;
    RACE_CUDA(cudaMemsetAsync(e.dStatus.p, 0, sizeof(int) * 4, e.stream));
    // SpMV, SpMTV and SymmSpMV have no data dependencies between rows: by
    // default (and in gather mode) they run as one gather launch, which on
    // GB300 beats the phase-by-phase executors by 9-37x on the 32^3 D2
    // SymmSpMV (0.010 ms against 0.089-0.77 ms per call)
    if (usesGather(e, f)) {
        runGather(e, f, dir);
        return;
    }
    const bool waveMode = useWaveMode(e, f, dir);
    SweepArgs a{f.kernel, ops.rowPtr, ops.col, ops.val, ops.x, ops.b, nullptr, nullptr, nullptr, 0,
                (unsigned *)(e.dStatus.p + 2), e.dStatus.p};
    a.midRow = midRowOf(e, f);
    int maxWork = 0;
    if (waveMode) {
        DevWaves &w = f.waves[dir];
        a.ptr = w.wavePtr.p;
        a.rows = w.rows.p;
        a.num = w.numWaves;
        a.waveHuge = w.numSegs > 0 ? w.waveHuge.p : nullptr;
        a.segFirst = w.segFirst.p;
        a.segPos = w.segPos.p;
        a.segBeg = w.segBeg.p;
        a.segEnd = w.segEnd.p;
        a.segScratch = w.segScratch.p;
        a.numSegs = w.numSegs;
        if (w.sell && w.sellMidRow == a.midRow) {
            a.waveChunk = w.waveChunk.p;
            a.chunkOff = w.chunkOff.p;
            a.sellVal = w.sellVal.p;
            a.sellCol = w.sellCol.p;
        }
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
