// Level-blocked matrix-power kernel (MPK): x_k = A x_{k-1}, k = 1..p.
//
// RACE's schedule (src/matrixPower.cpp consolidatePartition; executor
// src/functionManager.cpp:618-823) groups BFS levels so that p+1 powers of
// one group fit the cache, and runs a diagonal wavefront over (group,
// power). BFS levels only couple neighbouring levels, so power k of a group
// needs power k-1 of the group itself and of its two neighbours.
//
// Layout. At registration the permuted CRS is copied into SELL-32: rows are
// cut into chunks of at most 32 consecutive rows that never cross a level
// group; each lane owns one row and its entries sit in groups of four
// consecutive slots (entry j at off + 32 (j - j % 4) + 4 lane + j % 4), so a
// lane fetches four values and four columns with one or two vector loads
// and a warp's load covers 256-1024 contiguous bytes. Columns are stored in
// 16 bits where a chunk's columns fit four windows of 2^14 rows (a 2-bit
// window and the offset from that window's per-chunk base; the other
// chunks keep 32-bit columns). Each lane walks its row as a sequential fma
// chain in CRS order (MAT_SPMV_KERNEL's order,
// examples/src/helpers/kernels.cpp:749-777): FP64 output is bit-identical
// to p sequential SpMVs with fused multiply-adds. Padding slots are loaded
// as part of a last partial group but never computed. One lane per row
// keeps GB300's FP64 pipe (1/64 of the FP32 rate) busy with useful fmas
// only. Rows of more than kHubRowLen entries (hubs of power-law graphs)
// would stall their lane and pad their whole chunk: they are kept out of
// the SELL width, copied contiguously and summed by the whole warp (32
// ordered partial chains and a fixed butterfly), which matches the
// sequential sum to rounding rather than bit for bit.
//
// Schedule (RACE_MPK_WAVEFRONT). A work item is (power, chunk). Items are
// listed in the chunk-level wavefront order (mpk_order.cpp), grouped into
// runs of consecutive chunks, one queue per L2 die, and taken by persistent
// warps from per-queue tickets; each warp is an independent worker (no CTA
// barriers). A run waits until, at the previous power, the chunks holding
// its columns are complete: per chunk the engine records one chunk range in
// each of the previous, own and next group (narrow: a row's neighbours sit
// near the same position of the adjacent levels), widened to blocks of at
// most 16 chunks whose completions are counted, and the warp checks those
// counters in parallel. Runs wait only on earlier runs, held by running
// warps, so the schedule cannot deadlock; every wait is bounded anyway and
// reports a timeout through the status word. RACE_MPK_SWEEPS runs p plain
// SpMV launches on the same layout instead; RACE_MPK_AUTO keeps the faster.
//
// Reduced precision (FP32/BF16 values): the powers are kept in an internal
// FP32 copy of x and accumulated in FP32; each result is also written to the
// caller's FP64 x through an exact float->double bit conversion, so the FP32
// path issues no FP64 instructions in its inner loop.
#include <algorithm>
#include <numeric>

#include <cuda_bf16.h>

#include "dies.h"
#include "engine.h"
#include "mpk_order.h"

namespace race {

constexpr int kWarpThreads = 256;
// Rows longer than this are summed by a whole warp from a contiguous copy.
constexpr int kHubRowLen = kMpkHubRowLen;

namespace {

__device__ __forceinline__ int ldAcquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ldRelaxed(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned smIndex() {
    unsigned r;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
    return r;
}

// L2 eviction priorities (createpolicy): kind 1 evict_last, 2 evict_first,
// otherwise evict_normal.
__device__ __forceinline__ unsigned long long l2Policy(int kind) {
    unsigned long long p;
    if (kind == 1)
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    else if (kind == 2)
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    else
        asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}

template <typename VT>
__device__ __forceinline__ float toF(VT v);
template <>
__device__ __forceinline__ float toF<float>(float v) { return v; }
template <>
__device__ __forceinline__ float toF<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

// Exact binary32 -> binary64 conversion with integer operations (the IEEE
// 754 formats: re-bias the exponent, widen the significand; subnormal
// floats are normalised). Keeps the FP32 path off the FP64 pipe.
__device__ __forceinline__ double floatToDoubleExact(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned long long bits;
    if (e == 0xffu) {
        bits = sign | (0x7ffULL << 52) | ((unsigned long long)m << 29);
    } else if (e != 0) {
        bits = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (m == 0) {
        bits = sign;
    } else {
        const int p = 31 - __clz(m);  // value = m * 2^-149, leading bit at position p
        bits = sign | ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xfffffffffffffULL);
    }
    return __longlong_as_double((long long)bits);
}

struct SellView {
    const void *val;
    const int *col;             // 32-bit layout: sellSlots column indices
    const long long *chunkOff;  // numChunks: element offset of each chunk
    const int *chunkRow;        // numChunks+1: first row of each chunk
    const int *rowLen;          // n (-1: hub row)
    const int *hubChunkStart;   // numChunks+1
    const int *hubRow, *hubPtr;
    const void *hubVal;
    const int *hubCol;
    // 16-bit layout: per chunk four window bases (x < 0: the chunk keeps
    // 32-bit columns in wideCol from slot y on), per slot the window in bits
    // 14-15 and the offset from its base in bits 0-13
    const int4 *chunkBase;
    const unsigned short *col16;
    const int *wideCol;
};

// Vector loads of one entry group (four consecutive entries of a lane's
// row), with an L2 policy (POL) or plain.
template <bool POL>
__device__ __forceinline__ double2 ldVec(const double2 *a, unsigned long long pol) {
    double2 v;
    if constexpr (POL)
        asm("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(a), "l"(pol));
    else
        v = *a;
    return v;
}
template <bool POL>
__device__ __forceinline__ float4 ldVec(const float4 *a, unsigned long long pol) {
    float4 v;
    if constexpr (POL)
        asm("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
            : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
            : "l"(a), "l"(pol));
    else
        v = *a;
    return v;
}
template <bool POL>
__device__ __forceinline__ uint2 ldVec(const uint2 *a, unsigned long long pol) {
    uint2 v;
    if constexpr (POL)
        asm("ld.global.L2::cache_hint.v2.b32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(a), "l"(pol));
    else
        v = *a;
    return v;
}
template <bool POL>
__device__ __forceinline__ int4 ldVec(const int4 *a, unsigned long long pol) {
    int4 v;
    if constexpr (POL)
        asm("ld.global.L2::cache_hint.v4.b32 {%0, %1, %2, %3}, [%4], %5;"
            : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
            : "l"(a), "l"(pol));
    else
        v = *a;
    return v;
}

// Column of a stored 16-bit entry v: the base of window v >> 14 plus the
// low 14 bits.
__device__ __forceinline__ int col16Of(unsigned v, int4 b) {
    const int base = (v & 0x8000u) ? ((v & 0x4000u) ? b.w : b.z) : ((v & 0x4000u) ? b.y : b.x);
    return base + (int)(v & 0x3fffu);
}

// The four columns of an entry group at element offset o: one 8-byte load
// of 16-bit entries (C16) or one 16-byte load of 32-bit indices.
template <bool C16, bool POL>
__device__ __forceinline__ int4 groupCols(const void *col, long long o, int4 b, unsigned long long pol) {
    if constexpr (C16) {
        const uint2 w = ldVec<POL>((const uint2 *)((const unsigned short *)col + o), pol);
        return make_int4(col16Of(w.x & 0xffffu, b), col16Of(w.x >> 16, b), col16Of(w.y & 0xffffu, b),
                         col16Of(w.y >> 16, b));
    } else {
        return ldVec<POL>((const int4 *)((const int *)col + o), pol);
    }
}

// The four values of an entry group at element offset o (FP32/BF16 as
// floats).
template <bool POL>
__device__ __forceinline__ void groupVals(const double *val, long long o, double v[4], unsigned long long pol) {
    const double2 a = ldVec<POL>((const double2 *)(val + o), pol), c = ldVec<POL>((const double2 *)(val + o + 2), pol);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = c.x;
    v[3] = c.y;
}
template <bool POL>
__device__ __forceinline__ void groupVals(const float *val, long long o, float v[4], unsigned long long pol) {
    const float4 a = ldVec<POL>((const float4 *)(val + o), pol);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = a.z;
    v[3] = a.w;
}
template <bool POL>
__device__ __forceinline__ void groupVals(const __nv_bfloat16 *val, long long o, float v[4],
                                          unsigned long long pol) {
    const uint2 a = ldVec<POL>((const uint2 *)(val + o), pol);
    v[0] = __uint_as_float(a.x << 16);
    v[1] = __uint_as_float(a.x & 0xffff0000u);
    v[2] = __uint_as_float(a.y << 16);
    v[3] = __uint_as_float(a.y & 0xffff0000u);
}

// One row of a SELL-32 chunk: the lane's fma chain over its entries in CRS
// order. Entry j of the lane sits at element voff + 32 (j - j % 4) + j % 4
// (voff = the chunk's offset + 4 lane), its column at the same place from
// coff: every group of four entries is one or two vector loads of values
// and one of columns. A last partial group computes only the row's entries
// (its padding slots are loaded, never used). AT is the accumulation type:
// FP64 for FP64 values, FP32 otherwise.
template <typename VT, typename AT, bool C16, bool POL>
__device__ __forceinline__ AT sellRowAcc(const VT *__restrict__ val, long long voff, const void *col, long long coff,
                                         int4 b, int len, const AT *x, unsigned long long pol) {
    AT t = AT(0);
    for (int j = 0; j < len; j += 4) {
        AT v[4];
        groupVals<POL>(val, voff + 32LL * j, v, pol);
        const int4 c = groupCols<C16, POL>(col, coff + 32LL * j, b, pol);
        if (len - j >= 4) {
            const AT x0 = x[c.x], x1 = x[c.y], x2 = x[c.z], x3 = x[c.w];
            t = fma(v[0], x0, t);
            t = fma(v[1], x1, t);
            t = fma(v[2], x2, t);
            t = fma(v[3], x3, t);
        } else {
            t = fma(v[0], x[c.x], t);
            if (len - j > 1) t = fma(v[1], x[c.y], t);
            if (len - j > 2) t = fma(v[2], x[c.z], t);
        }
    }
    return t;
}

// Row r at power k -> k+1 from its SELL entries; FP32/BF16 results also go
// to the FP64 powers through the exact conversion.
template <typename VT, bool C16, bool POL>
__device__ __forceinline__ void sellRow(const SellView &m, const void *col, long long voff, long long coff, int4 b,
                                        int len, int r, int k, int n, double *x, float *xf,
                                        unsigned long long pol) {
    if constexpr (sizeof(VT) == 8) {
        x[(size_t)(k + 1) * n + r] = sellRowAcc<double, double, C16, POL>((const double *)m.val, voff, col, coff, b,
                                                                          len, x + (size_t)k * n, pol);
    } else {
        const float v =
            sellRowAcc<VT, float, C16, POL>((const VT *)m.val, voff, col, coff, b, len, xf + (size_t)k * n, pol);
        xf[(size_t)(k + 1) * n + r] = v;
        x[(size_t)(k + 1) * n + r] = floatToDoubleExact(v);
    }
}

// A hub row summed by the whole warp: lane l takes entries l, l+32, ... in
// order (one fma chain per lane, coalesced reads of the contiguous copy),
// then a fixed butterfly combines the 32 partial sums. Deterministic, but
// not the sequential order of the short rows: results agree with the
// single-chain sum to rounding (relative 1e-15 scale), not bit for bit.
template <typename VT, typename AT>
__device__ __forceinline__ AT hubSum(const SellView &m, int h, const AT *x) {
    const int lane = threadIdx.x & 31;
    const VT *__restrict__ val = (const VT *)m.hubVal;
    AT t = AT(0);
    for (int e = m.hubPtr[h] + lane; e < m.hubPtr[h + 1]; e += 32) {
        if constexpr (sizeof(VT) == 8)
            t = fma(val[e], x[m.hubCol[e]], t);
        else
            t = fmaf(toF<VT>(val[e]), x[m.hubCol[e]], t);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// Chunk c at power k -> k+1: the lane's row (unless it is a hub row), then
// the chunk's hub rows one at a time with the whole warp. Called by all 32
// lanes of a warp. HUBS = false compiles the plain SELL row only (plans
// without hub rows keep the register count, hence the occupancy, of that);
// C16 reads the 16-bit column layout.
template <typename VT, bool HUBS, bool C16, bool POL = false>
__device__ __forceinline__ void chunkRow(const SellView &m, int c, int k, int n, double *x, float *xf,
                                         unsigned long long pol) {
    const int lane = threadIdx.x & 31;
    const int r = m.chunkRow[c] + lane;
    if (r < m.chunkRow[c + 1]) {
        const int len = m.rowLen[r];
        const long long off = m.chunkOff[c] + 4 * lane;
        if (len >= 0) {
            if constexpr (C16) {
                const int4 b = m.chunkBase[c];
                if (b.x >= 0)
                    sellRow<VT, true, POL>(m, m.col16, off, off, b, len, r, k, n, x, xf, pol);
                else
                    sellRow<VT, false, POL>(m, m.wideCol, off, (long long)b.y + 4 * lane, b, len, r, k, n, x, xf, pol);
            } else {
                sellRow<VT, false, POL>(m, m.col, off, off, make_int4(0, 0, 0, 0), len, r, k, n, x, xf, pol);
            }
        }
    }
    if constexpr (HUBS)
    for (int h = m.hubChunkStart[c]; h < m.hubChunkStart[c + 1]; ++h) {
        const int hr = m.hubRow[h];
        if constexpr (sizeof(VT) == 8) {
            const double v = hubSum<VT, double>(m, h, x + (size_t)k * n);
            if (lane == 0) x[(size_t)(k + 1) * n + hr] = v;
        } else {
            const float v = hubSum<VT, float>(m, h, xf + (size_t)k * n);
            if (lane == 0) {
                xf[(size_t)(k + 1) * n + hr] = v;
                x[(size_t)(k + 1) * n + hr] = floatToDoubleExact(v);
            }
        }
    }
}

struct MpkArgs {
    SellView m;
    double *x;      // caller's (p+1)*n powers
    float *xf;      // internal FP32 powers (reduced-precision storage only)
    int n;
    // numRuns: first chunk, end chunk, power k, flags (bit 0: last power of
    // the segment; bits 1-31: the completion block of the first chunk)
    const int4 *runHead;
    const int4 *runDep;        // 2 per run: four block intervals [lo,hi] read at power k-1
    int numBlocks;
    const int *blockStart;     // numBlocks+1: first chunk of each completion block
    int *done;                 // power * numBlocks: chunks complete per block
    int *ticket;               // one per die queue
    int *status;
    int hints;                 // L2 eviction hints on the matrix
    const int *smDie;          // die of every SM (numDies > 1)
    int numDies;
    int dieStart[3];           // die d's queue: runs dieStart[d] .. dieStart[d+1]-1
};

// Persistent warps: one run (up to 32 consecutive chunks at one power) per
// ticket. A run waits until every completion block in its intervals is
// complete at the previous power (its counter equals its chunk count);
// those chunks belong to runs earlier in the global order (the order is
// built from dependency ranges widened to whole blocks), taken by running
// warps, so the wait always ends (bounded anyway: a timeout goes to the
// status word). The polls are relaxed loads and one acquire fence follows
// the successful poll (a counter read by a relaxed load and a later
// fence.acq_rel form an acquire of the writers' releases). A warp takes the
// runs of its own die's queue, so each chunk's matrix block is cached by
// one die's L2 only; an empty queue sends it to the other one. A warp adds
// its previous run's chunks to their block counters (release reductions)
// only after fetching the next run, when the stores they publish have
// drained; that comes before any wait, so a warp never waits on itself.
// At least 6 resident blocks per SM (up to 40 registers a thread).
constexpr int kMpkMinBlocks = 6;

template <typename VT, bool HUBS, bool C16>
__global__ void __launch_bounds__(kWarpThreads, kMpkMinBlocks) kMpk(MpkArgs a) {
    const int lane = threadIdx.x & 31;
    const unsigned long long polKeep = l2Policy(a.hints ? 1 : 0), polDrop = l2Policy(a.hints ? 2 : 0);
    const int myDie = a.numDies > 1 ? a.smDie[smIndex()] : 0;
    int q = myDie;
    int pc0 = 0, pc1 = 0, pk = 0, pb = 0;  // run still to be counted, its first block
    int it = 0;
    for (;;) {
        if (lane == 0) it = atomicAdd(a.ticket + q, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        const int qStart = q == 0 ? a.dieStart[0] : a.dieStart[1];
        const int qCount = q == 0 ? a.dieStart[1] - a.dieStart[0] : a.dieStart[2] - a.dieStart[1];
        const bool have = it < qCount;
        int4 h = make_int4(0, 0, 0, 0), d0 = h, d1 = h;
        if (have) {
            h = a.runHead[qStart + it];
            d0 = a.runDep[2 * (qStart + it)];
            d1 = a.runDep[2 * (qStart + it) + 1];
        }
        // count the previous run; __syncwarp orders all lanes' stores before
        // the release reductions (lane i: the run's i-th block)
        __syncwarp();
        if (pc1 > pc0 && pb + lane < a.numBlocks) {
            const int bs = a.blockStart[pb + lane];
            if (bs < pc1) {
                const int cnt = min(pc1, a.blockStart[pb + lane + 1]) - max(pc0, bs);
                asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(a.done + (size_t)pk * a.numBlocks + pb +
                                                                              lane),
                             "r"(cnt)
                             : "memory");
            }
        }
        pc0 = pc1 = 0;
        if (!have) {
            if (a.numDies > 1 && q == myDie) {
                q = 1 - myDie;
                continue;
            }
            return;
        }
        const int k = h.z;  // computes x_{k+1} from x_k
        if (k > 0) {
            const int *done = a.done + (size_t)(k - 1) * a.numBlocks;
            const int *bs = a.blockStart;
            long long spins = 0;
            for (;;) {
                bool ok = true;
                for (int i = d0.x + lane; i <= d0.y; i += 32) ok &= ldRelaxed(done + i) == bs[i + 1] - bs[i];
                for (int i = d0.z + lane; i <= d0.w; i += 32) ok &= ldRelaxed(done + i) == bs[i + 1] - bs[i];
                for (int i = d1.x + lane; i <= d1.y; i += 32) ok &= ldRelaxed(done + i) == bs[i + 1] - bs[i];
                for (int i = d1.z + lane; i <= d1.w; i += 32) ok &= ldRelaxed(done + i) == bs[i + 1] - bs[i];
                if (__all_sync(0xffffffffu, ok)) break;
                if (++spins > kSpinLimit || ldAcquire(a.status) != DEV_OK) {
                    if (lane == 0) atomicCAS(a.status, DEV_OK, DEV_WAIT_TIMEOUT);
                    return;
                }
                __nanosleep(32);
            }
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
        }
        const unsigned long long pol = (h.w & 1) ? polDrop : polKeep;
        for (int c = h.x; c < h.y; ++c) chunkRow<VT, HUBS, C16, true>(a.m, c, k, a.n, a.x, a.xf, pol);
        pc0 = h.x;
        pc1 = h.y;
        pk = k;
        pb = h.w >> 1;
    }
}

// Plain y = A x on the SELL layout, no schedule: one warp per chunk.
template <typename VT, bool HUBS, bool C16>
__global__ void __launch_bounds__(kWarpThreads) kSpmvSell(SellView m, int numChunks, int n, int k, double *x,
                                                          float *xf) {
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < numChunks; c += nw)
        chunkRow<VT, HUBS, C16>(m, c, k, n, x, xf, 0);
}

// One wavefront step of a triangular partition: one warp per (chunk,
// power) item of the step. Every item's inputs were written by earlier
// launches, so nothing waits.
template <typename VT, bool HUBS, bool C16>
__global__ void __launch_bounds__(kWarpThreads) kMpkStep(SellView m, const int *__restrict__ itemChunk,
                                                         const unsigned char *__restrict__ itemPow, int count, int n,
                                                         double *x, float *xf) {
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < count; i += nw)
        chunkRow<VT, HUBS, C16>(m, itemChunk[i], itemPow[i], n, x, xf, 0);
}

// x0 -> FP32 copy (rounding to nearest) for the reduced-precision path.
__global__ void kToFloat(const double *__restrict__ x, float *__restrict__ xf, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xf[i] = (float)x[i];
}

// CRS thread-per-row SpMV (for raw pointers without a registered layout).
__global__ void kSpmvCrs(int n, const int *__restrict__ rowPtr, const int *__restrict__ col,
                         const double *__restrict__ val, const double *__restrict__ x, double *__restrict__ b) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double t = 0.0;
#pragma unroll 4
    for (int j = rowPtr[r]; j < rowPtr[r + 1]; ++j) t = fma(val[j], x[col[j]], t);
    b[r] = t;
}

// Contiguous copies of the hub rows, one warp per hub.
template <typename VT>
__global__ void kGatherHubs(const int *__restrict__ rowPtr, const int *__restrict__ col, const VT *__restrict__ val,
                            const int *__restrict__ hubRow, const int *__restrict__ hubPtr, int numHubs,
                            VT *__restrict__ hval, int *__restrict__ hcol) {
    const int h = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (h >= numHubs) return;
    const int s = rowPtr[hubRow[h]], len = hubPtr[h + 1] - hubPtr[h];
    for (int j = threadIdx.x & 31; j < len; j += 32) {
        hval[hubPtr[h] + j] = val[s + j];
        hcol[hubPtr[h] + j] = col[s + j];
    }
}

// Element offset of entry j of a lane's row inside its chunk: entries in
// groups of four consecutive slots per lane (SELL-32 with 4-entry groups).
__device__ __forceinline__ long long sellSlot(int j, int lane) {
    return 32LL * (j & ~3) + 4 * lane + (j & 3);
}

// CRS -> SELL-32 copy; padding slots get value 0 and the row's own column.
// Hub rows are longer than the chunk width L: their first L entries are
// copied and never read.
template <typename VT>
__global__ void kToSell(const int *__restrict__ rowPtr, const int *__restrict__ col, const VT *__restrict__ val,
                        const long long *__restrict__ chunkOff, const int *__restrict__ chunkRowP,
                        const int *__restrict__ chunkLen, int numChunks, VT *__restrict__ sval, int *__restrict__ scol) {
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= numChunks) return;
    const int lane = threadIdx.x & 31;
    const int r = chunkRowP[c] + lane;
    const bool live = r < chunkRowP[c + 1];
    const int s = live ? rowPtr[r] : 0, len = live ? rowPtr[r + 1] - s : 0;
    const int L = chunkLen[c];
    for (int j = 0; j < L; ++j) {
        const long long o = chunkOff[c] + sellSlot(j, lane);
        if (j < len) {
            sval[o] = val[s + j];
            scol[o] = col[s + j];
        } else {
            sval[o] = VT(0);
            scol[o] = live ? r : chunkRowP[c];
        }
    }
}

// 16-bit column layout. Every chunk's columns (hub rows excluded) are
// covered by at most four windows of `window` rows (at most 2^14, the
// offset field): the first starts at the smallest column, each next one at
// the smallest column at least `window` beyond the previous start (the
// greedy cover, which uses the fewest windows). A chunk that needs more
// gets x = -1 and keeps 32-bit columns; unused windows get INT_MAX. One
// block of 128 threads per chunk, a warp per row.
__global__ void kChunkWindows(const int *__restrict__ rowPtr, const int *__restrict__ col,
                              const int *__restrict__ chunkRowP, const int *__restrict__ rowLen, int numChunks,
                              int window, int4 *__restrict__ base) {
    const int c = blockIdx.x;
    if (c >= numChunks) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ int wmin[4];
    const int r0 = chunkRowP[c], r1 = chunkRowP[c + 1];
    int b[5] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX, INT_MAX};
    for (int w = 0; w < 5; ++w) {
        const int prev = w > 0 ? b[w - 1] : 0;
        int m = INT_MAX;
        for (int r = r0 + warp; r < r1; r += 4) {
            if (rowLen[r] < 0) continue;
            for (int j = rowPtr[r] + lane; j < rowPtr[r + 1]; j += 32) {
                const int cc = col[j];
                if (w == 0 || cc - prev >= window) m = min(m, cc);
            }
        }
        m = __reduce_min_sync(0xffffffffu, m);
        if (lane == 0) wmin[warp] = m;
        __syncthreads();
        b[w] = min(min(wmin[0], wmin[1]), min(wmin[2], wmin[3]));
        __syncthreads();
        if (b[w] == INT_MAX) break;
    }
    if (threadIdx.x == 0) base[c] = b[4] != INT_MAX ? make_int4(-1, 0, 0, 0) : make_int4(b[0], b[1], b[2], b[3]);
}

// CRS -> SELL-32 copy with 16-bit columns (kChunkWindows' bases; chunks
// with x = -1 write 32-bit columns to wideCol from slot y on). Padding
// slots get value 0 and column entry 0 (wide chunks: the row's own
// column); hub rows are padding here, their entries live in the hub copy.
template <typename VT>
__global__ void kToSell16(const int *__restrict__ rowPtr, const int *__restrict__ col, const VT *__restrict__ val,
                          const long long *__restrict__ chunkOff, const int *__restrict__ chunkRowP,
                          const int *__restrict__ chunkLen, const int4 *__restrict__ chunkBase, int numChunks,
                          VT *__restrict__ sval, unsigned short *__restrict__ col16, int *__restrict__ wideCol) {
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= numChunks) return;
    const int lane = threadIdx.x & 31;
    const int r = chunkRowP[c] + lane;
    const bool live = r < chunkRowP[c + 1];
    const int s = live ? rowPtr[r] : 0;
    int len = live ? rowPtr[r + 1] - s : 0;
    if (len > kMpkHubRowLen) len = 0;
    const int L = chunkLen[c];
    const int4 b = chunkBase[c];
    for (int j = 0; j < L; ++j) {
        const long long o = chunkOff[c] + sellSlot(j, lane);
        unsigned short v = 0;
        if (j < len) {
            sval[o] = val[s + j];
            const int cc = col[s + j];
            if (b.x >= 0) {
                const int sel = (cc >= b.y) + (cc >= b.z) + (cc >= b.w);
                const int bs = sel == 0 ? b.x : sel == 1 ? b.y : sel == 2 ? b.z : b.w;
                v = (unsigned short)((sel << 14) | (cc - bs));
            } else {
                wideCol[b.y + sellSlot(j, lane)] = cc;
            }
        } else {
            sval[o] = VT(0);
            if (b.x < 0) wideCol[b.y + sellSlot(j, lane)] = live ? r : chunkRowP[c];
        }
        col16[o] = v;
    }
}

// For every chunk, the range of chunks its columns fall in, separately for
// the previous, the own and the next level group. Columns outside those
// three groups mark the plan invalid (*bad = 1): BFS levels only couple
// neighbouring levels, so a RACE-permuted matrix never has them. With
// earlierOk (triangular partitions, run step by step) columns in any
// earlier group are allowed and left out of the ranges.
__global__ void kChunkRanges(const int *__restrict__ rowPtr, const int *__restrict__ col,
                             const int *__restrict__ chunkRowP, const int *__restrict__ chunkGroup, int numChunks,
                             int *__restrict__ range, int *__restrict__ bad, int earlierOk) {
    const int t = blockIdx.x;
    if (t >= numChunks) return;
    __shared__ int lo[3], hi[3];
    if (threadIdx.x < 3) {
        lo[threadIdx.x] = INT_MAX;
        hi[threadIdx.x] = -1;
    }
    __syncthreads();
    const int g = chunkGroup[t];
    for (int j = rowPtr[chunkRowP[t]] + threadIdx.x; j < rowPtr[chunkRowP[t + 1]]; j += blockDim.x) {
        const int c = col[j];
        int a = 0, b = numChunks - 1;
        while (a < b) {
            int mid = (a + b + 1) >> 1;
            if (chunkRowP[mid] <= c) a = mid; else b = mid - 1;
        }
        const int d = chunkGroup[a] - g + 1;
        if (d < 0 && earlierOk) continue;
        if (d < 0 || d > 2) {
            atomicExch(bad, 1);
            continue;
        }
        atomicMin(&lo[d], a);
        atomicMax(&hi[d], a);
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        range[6 * t + 2 * threadIdx.x] = (hi[threadIdx.x] < 0) ? 0 : lo[threadIdx.x];
        range[6 * t + 2 * threadIdx.x + 1] = hi[threadIdx.x];  // empty range: hi = -1 < lo
    }
}

int gDevSms = 0;
int devSms() {
    if (!gDevSms) {
        int dev = 0;
        RACE_CUDA(cudaGetDevice(&dev));
        RACE_CUDA(cudaDeviceGetAttribute(&gDevSms, cudaDevAttrMultiProcessorCount, dev));
    }
    return gDevSms;
}

template <typename K>
int residentBlocks(K kernel, int threads) {
    int occ = 0;
    RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, 0));
    return devSms() * std::max(occ, 1);
}

size_t valBytes(int vt) { return vt == RACE_VAL_F64 ? 8 : vt == RACE_VAL_F32 ? 4 : 2; }

// The SELL copy of the plan's chunks (32- or 16-bit columns) and the
// contiguous hub copies.
template <typename VT>
void copySell(const race_operands &ops, MpkPlan &p, const int *chunkLen, cudaStream_t s) {
    const int C = p.numChunks, H = p.numHubs;
    const int blocksC = ceilDiv(std::max(C, 1), 8);
    if (p.col16)
        kToSell16<VT><<<blocksC, 256, 0, s>>>(ops.rowPtr, ops.col, (const VT *)ops.val, p.chunkOff.p, p.chunkRow.p,
                                              chunkLen, p.chunkBase.p, C, (VT *)p.sellVal.p, p.sellCol16.p,
                                              p.wideCol.p);
    else
        kToSell<VT><<<blocksC, 256, 0, s>>>(ops.rowPtr, ops.col, (const VT *)ops.val, p.chunkOff.p, p.chunkRow.p,
                                            chunkLen, C, (VT *)p.sellVal.p, p.sellCol.p);
    if (H)
        kGatherHubs<VT><<<ceilDiv(H, 8), 256, 0, s>>>(ops.rowPtr, ops.col, (const VT *)ops.val, p.hubRow.p,
                                                      p.hubPtr.p, H, (VT *)p.hubVal.p, p.hubCol.p);
    RACE_CUDA(cudaGetLastError());
}

}  // namespace

// Builds the SELL-32 copy, the chunk dependency ranges and the wavefront
// item order of one MPK operand set (the user's permuted matrix) for the
// engine's level groups.
std::unique_ptr<MpkPlan> buildMpkPlan(Engine &e, const race_operands &ops, int power) {
    auto plan = std::make_unique<MpkPlan>();
    const int n = ops.n;
    cudaStream_t s = e.stream;
    std::vector<int> rp(n + 1);
    RACE_CUDA(cudaMemcpyAsync(rp.data(), ops.rowPtr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    const std::vector<int> &gp = e.groupPtr;
    const int G = (int)gp.size() - 1;
    // chunks of <= 32 rows inside groups
    std::vector<int> chunkRowH{0}, chunkLen, chunkGroup, rowLen(n);
    std::vector<int> hubRowH, hubPtrH{0}, hubStartH{0};
    std::vector<long long> chunkOff;
    long long off = 0;
    for (int r = 0; r < n; ++r) {
        rowLen[r] = rp[r + 1] - rp[r];
        if (rowLen[r] > kHubRowLen) {
            hubRowH.push_back(r);
            hubPtrH.push_back(hubPtrH.back() + rowLen[r]);
            rowLen[r] = -1;
        }
    }
    size_t hubIdx = 0;
    for (int g = 0; g < G; ++g)
        for (int r = gp[g]; r < gp[g + 1]; r += 32) {
            int r1 = std::min(gp[g + 1], r + 32);
            int L = 0;
            for (int q = r; q < r1; ++q) L = std::max(L, rowLen[q]);
            L = (L + 3) & ~3;  // whole entry groups
            chunkOff.push_back(off);
            chunkLen.push_back(L);
            chunkRowH.push_back(r1);
            chunkGroup.push_back(g);
            off += 32LL * L;
            while (hubIdx < hubRowH.size() && hubRowH[hubIdx] < r1) ++hubIdx;
            hubStartH.push_back((int)hubIdx);
        }
    const int C = (int)chunkLen.size();
    const int H = (int)hubRowH.size();
    plan->numHubs = H;
    plan->hubChunkStart.upload(hubStartH.data(), hubStartH.size(), s);
    plan->hubRow.upload(H ? hubRowH.data() : nullptr, std::max(H, 1), s);
    plan->hubPtr.upload(hubPtrH.data(), hubPtrH.size(), s);
    plan->hubVal.alloc(std::max<long long>(hubPtrH.back(), 1) * valBytes(ops.val_type));
    plan->hubCol.alloc(std::max<long long>(hubPtrH.back(), 1));
    plan->numChunks = C;
    plan->power = power;
    plan->valType = ops.val_type;
    plan->sellSlots = off;
    plan->chunkOff.upload(chunkOff.data(), std::max(C, 1), s);
    plan->chunkRow.upload(chunkRowH.data(), chunkRowH.size(), s);
    plan->rowLen.upload(rowLen.data(), n, s);
    DevBuf<int> dChunkLen;
    dChunkLen.upload(chunkLen.data(), std::max(C, 1), s);
    // 16-bit columns where the chunks' columns fit their windows: worth it
    // while at most half of the slots stay 32-bit
    plan->col16 = e.mpkCol16 && C > 0;
    std::vector<int4> baseH;
    if (plan->col16) {
        plan->chunkBase.alloc(C);
        kChunkWindows<<<C, 128, 0, s>>>(ops.rowPtr, ops.col, plan->chunkRow.p, plan->rowLen.p, C,
                                        std::min(std::max(e.mpkColWindow, 1), kMpkColWindow), plan->chunkBase.p);
        RACE_CUDA(cudaGetLastError());
        baseH.resize(C);
        RACE_CUDA(cudaMemcpyAsync(baseH.data(), plan->chunkBase.p, sizeof(int4) * C, cudaMemcpyDeviceToHost, s));
        RACE_CUDA(cudaStreamSynchronize(s));
        long long wide = 0;
        for (int c = 0; c < C; ++c)
            if (baseH[c].x < 0) {
                baseH[c].y = (int)std::min<long long>(wide, INT_MAX);
                wide += 32LL * chunkLen[c];
                ++plan->wideChunks;
            }
        plan->wideSlots = wide;
        plan->col16 = 2 * wide <= off && wide < INT_MAX;
        if (plan->col16) {
            plan->chunkBase.upload(baseH.data(), C, s);
        } else {
            plan->chunkBase.free();
            plan->wideChunks = 0;
            plan->wideSlots = 0;
        }
    }
    plan->sellVal.alloc(std::max<long long>(off, 1) * valBytes(ops.val_type));
    if (plan->col16) {
        plan->sellCol16.alloc(std::max<long long>(off, 1));
        plan->wideCol.alloc(std::max<long long>(plan->wideSlots, 1));
    } else {
        plan->sellCol.alloc(std::max<long long>(off, 1));
    }
    if (ops.val_type != RACE_VAL_F64) plan->xf.alloc((size_t)(power + 1) * n);
    switch (ops.val_type) {
    case RACE_VAL_F64: copySell<double>(ops, *plan, dChunkLen.p, s); break;
    case RACE_VAL_F32: copySell<float>(ops, *plan, dChunkLen.p, s); break;
    case RACE_VAL_BF16: copySell<__nv_bfloat16>(ops, *plan, dChunkLen.p, s); break;
    default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
    }
    RACE_CUDA(cudaGetLastError());
    plan->stepped = e.powerLevelsType == "L" || e.powerLevelsType == "U";
    plan->schedule = e.mpkSchedule;
    plan->depRange.alloc((size_t)std::max(C, 1) * 6);
    plan->ticket.alloc(2);
    plan->status.alloc(1);
    DevBuf<int> dChunkGroup, dBad(1);
    dChunkGroup.upload(chunkGroup.data(), std::max<size_t>(chunkGroup.size(), 1), s);
    RACE_CUDA(cudaMemsetAsync(dBad.p, 0, sizeof(int), s));
    if (C > 0)
        kChunkRanges<<<C, 128, 0, s>>>(ops.rowPtr, ops.col, plan->chunkRow.p, dChunkGroup.p, C, plan->depRange.p,
                                       dBad.p, plan->stepped ? 1 : 0);
    RACE_CUDA(cudaGetLastError());
    int bad = 0;
    std::vector<int> depRange((size_t)C * 6);
    RACE_CUDA(cudaMemcpyAsync(&bad, dBad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (C > 0)
        RACE_CUDA(cudaMemcpyAsync(depRange.data(), plan->depRange.p, sizeof(int) * depRange.size(),
                                  cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    // Every dependency must come earlier in the wavefront order: the columns
    // of group g lie in groups g-1..g+1 (BFS levels couple neighbours only;
    // for a triangular partition in any group up to g+1). A matrix not
    // permuted with this engine's MPK permutation breaks that and is
    // rejected here instead of stalling the kernel.
    if (bad)
        throw Error(RACE_ERR_INVALID_ARG,
                    "MPK operand is not in the engine's level order (permute it with getPerm/getInvPerm)");
    if (plan->stepped) {
        // A triangular partition (mtxType L/U) lets a row read any earlier
        // group, which the chunk intervals do not describe; it runs step by
        // step in RACE's group order with stride 2 (step s holds power k of
        // group s-2k), so every earlier group's previous power lies in an
        // earlier step.
        std::vector<int> groupFirst(G + 1, C);
        for (int t = C - 1; t >= 0; --t) groupFirst[chunkGroup[t]] = t;
        for (int g = G - 1; g >= 0; --g) groupFirst[g] = std::min(groupFirst[g], groupFirst[g + 1]);
        std::vector<int> itemChunk;
        std::vector<unsigned char> itemPow;
        plan->stepPtr.assign(1, 0);
        for (int st = 0; st < G + 2 * (power - 1); ++st) {
            for (int k = 0; k < power; ++k) {
                const int g = st - 2 * k;
                if (g < 0 || g >= G) continue;
                for (int t = groupFirst[g]; t < groupFirst[g + 1]; ++t) {
                    itemChunk.push_back(t);
                    itemPow.push_back((unsigned char)k);
                }
            }
            plan->stepPtr.push_back((int)itemChunk.size());
        }
        plan->numItems = (int)itemChunk.size();
        plan->itemChunk.upload(itemChunk.data(), std::max<size_t>(itemChunk.size(), 1), s);
        plan->itemPow.upload(itemPow.data(), std::max<size_t>(itemPow.size(), 1), s);
        RACE_CUDA(cudaStreamSynchronize(s));
        return plan;
    }
    // Issue order of the persistent kernel (mpk_order.cpp): by default the
    // chunk-level wavefront, every (chunk, power) item as early as the
    // chunks it reads and the work in flight allow, in runs of consecutive
    // chunks per ticket and one queue per L2 die; RACE's level-group order
    // on request. All orders compute the same rows at the same powers:
    // results are bit-identical.
    const int segLen = e.mpkSplit > 0 && e.mpkSplit < power ? e.mpkSplit : power;
    const DieMap &dies = dieMap();
    const bool twoDies = dies.numDies == 2 && e.mpkOrder == 0 && e.mpkDieQueues;
    const std::vector<int> chunkDie =
        twoDies ? chunkDies(C, dies.smsPerDie[0], dies.smsPerDie[1]) : std::vector<int>();
    // Completion is counted per block of chunks; the order is built from the
    // dependency ranges widened to whole blocks, and the kernel's tables
    // name blocks: each interval as a block range, each run's first block
    // in the flags.
    const std::vector<int> blockStart = mpkFlagBlocks(C, chunkGroup);
    const int NB = (int)blockStart.size() - 1;
    std::vector<int> blockOf(C);
    for (int b = 0; b < NB; ++b)
        for (int c = blockStart[b]; c < blockStart[b + 1]; ++c) blockOf[c] = b;
    const std::vector<int> widened = widenDepsToBlocks(depRange, blockStart);
    const MpkOrder order = e.mpkOrder == 1
                               ? mpkGroupOrder(widened, chunkGroup, G, power, e.mpkStride == 1 ? 1 : 2, segLen)
                               : mpkRunOrder(widened, C, power, segLen, e.mpkRun, e.mpkLag, chunkDie);
    plan->numItems = (int)((size_t)C * power);
    plan->numRuns = order.numRuns();
    plan->numDies = twoDies ? 2 : 1;
    for (int d = 0; d < 3; ++d) plan->dieStart[d] = order.dieStart[d];
    plan->smDie = dies.smDieDev.p;
    plan->numBlocks = NB;
    plan->blockStart.upload(blockStart.data(), blockStart.size(), s);
    plan->done.alloc((size_t)std::max(NB, 1) * power);
    std::vector<int> head(order.head), dep(order.dep);
    for (int r = 0; r < plan->numRuns; ++r) head[4 * (size_t)r + 3] |= blockOf[head[4 * (size_t)r]] << 1;
    for (size_t i = 0; i + 1 < dep.size(); i += 2)
        if (dep[i + 1] >= dep[i]) {
            dep[i] = blockOf[dep[i]];
            dep[i + 1] = blockOf[dep[i + 1]];
        }
    if (plan->numRuns == 0) {
        head.assign(4, 0);
        dep.assign(8, 0);
    }
    plan->runHead.upload((const int4 *)head.data(), head.size() / 4, s);
    plan->runDep.upload((const int4 *)dep.data(), dep.size() / 4, s);
    plan->hints = e.mpkHints;
    plan->ctasPerSm = e.mpkCtasPerSm;
    RACE_CUDA(cudaStreamSynchronize(s));
    return plan;
}

// Host entry to kChunkRanges for other schedules over the same level groups:
// fills range (6 per chunk, local chunk ids) and returns false if some column
// lies outside the previous/own/next group of its row.
bool chunkDependencyRanges(const int *rowPtr, const int *col, const std::vector<int> &chunkRow,
                           const std::vector<int> &chunkGroup, std::vector<int> &range, cudaStream_t s) {
    const int C = (int)chunkGroup.size();
    range.assign((size_t)C * 6, 0);
    if (C == 0) return true;
    DevBuf<int> dRow, dGroup, dRange((size_t)C * 6), dBad(1);
    dRow.upload(chunkRow.data(), chunkRow.size(), s);
    dGroup.upload(chunkGroup.data(), chunkGroup.size(), s);
    RACE_CUDA(cudaMemsetAsync(dBad.p, 0, sizeof(int), s));
    kChunkRanges<<<C, 128, 0, s>>>(rowPtr, col, dRow.p, dGroup.p, C, dRange.p, dBad.p, 0);
    RACE_CUDA(cudaGetLastError());
    int bad = 0;
    RACE_CUDA(cudaMemcpyAsync(range.data(), dRange.p, sizeof(int) * range.size(), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaMemcpyAsync(&bad, dBad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    return bad == 0;
}

namespace {
SellView viewOf(const MpkPlan &p) {
    return SellView{p.sellVal.p,       p.sellCol.p, p.chunkOff.p, p.chunkRow.p, p.rowLen.p,
                    p.hubChunkStart.p, p.hubRow.p,  p.hubPtr.p,   p.hubVal.p,   p.hubCol.p,
                    p.chunkBase.p,     p.sellCol16.p, p.wideCol.p};
}

template <typename VT, bool HUBS, bool C16>
void launchMpkK(const MpkArgs &a, int ctasPerSm, cudaStream_t s) {
    static int resident = residentBlocks(kMpk<VT, HUBS, C16>, kWarpThreads);
    const int blocks = ctasPerSm > 0 ? std::min(resident, devSms() * ctasPerSm) : resident;
    kMpk<VT, HUBS, C16><<<blocks, kWarpThreads, 0, s>>>(a);
}

template <typename VT>
void launchMpk(const MpkArgs &a, const MpkPlan &p, cudaStream_t s) {
    if (p.numHubs > 0) {
        if (p.col16) launchMpkK<VT, true, true>(a, p.ctasPerSm, s);
        else launchMpkK<VT, true, false>(a, p.ctasPerSm, s);
    } else {
        if (p.col16) launchMpkK<VT, false, true>(a, p.ctasPerSm, s);
        else launchMpkK<VT, false, false>(a, p.ctasPerSm, s);
    }
}

template <typename VT, bool HUBS, bool C16>
void launchMpkStepsK(const MpkPlan &p, int n, double *x, cudaStream_t s) {
    const SellView v = viewOf(p);
    for (size_t st = 0; st + 1 < p.stepPtr.size(); ++st) {
        const int first = p.stepPtr[st], count = p.stepPtr[st + 1] - first;
        if (count == 0) continue;
        const int blocks = std::min(ceilDiv(count, kWarpThreads / 32), devSms() * 16);
        kMpkStep<VT, HUBS, C16><<<blocks, kWarpThreads, 0, s>>>(v, p.itemChunk.p + first, p.itemPow.p + first,
                                                                 count, n, x, p.xf.p);
    }
}

template <typename VT>
void launchMpkSteps(const MpkPlan &p, int n, double *x, cudaStream_t s) {
    if (p.numHubs > 0) {
        if (p.col16) launchMpkStepsK<VT, true, true>(p, n, x, s);
        else launchMpkStepsK<VT, true, false>(p, n, x, s);
    } else {
        if (p.col16) launchMpkStepsK<VT, false, true>(p, n, x, s);
        else launchMpkStepsK<VT, false, false>(p, n, x, s);
    }
}

template <typename VT, bool HUBS, bool C16>
void launchSpmvSellK(const SellView &v, int numChunks, int n, int k, double *x, float *xf, cudaStream_t s) {
    static int blocks = residentBlocks(kSpmvSell<VT, HUBS, C16>, kWarpThreads);
    kSpmvSell<VT, HUBS, C16><<<blocks, kWarpThreads, 0, s>>>(v, numChunks, n, k, x, xf);
}

template <typename VT>
void launchSpmvSell(const MpkPlan &p, int n, int k, double *x, cudaStream_t s) {
    const SellView v = viewOf(p);
    if (p.numHubs > 0) {
        if (p.col16) launchSpmvSellK<VT, true, true>(v, p.numChunks, n, k, x, p.xf.p, s);
        else launchSpmvSellK<VT, true, false>(v, p.numChunks, n, k, x, p.xf.p, s);
    } else {
        if (p.col16) launchSpmvSellK<VT, false, true>(v, p.numChunks, n, k, x, p.xf.p, s);
        else launchSpmvSellK<VT, false, false>(v, p.numChunks, n, k, x, p.xf.p, s);
    }
}
}  // namespace

namespace {
// The persistent wavefront kernel over all powers.
void runWavefront(MpkPlan &plan, const race_operands &ops, cudaStream_t s) {
    RACE_CUDA(cudaMemsetAsync(plan.done.p, 0, sizeof(int) * (size_t)plan.numBlocks * plan.power, s));
    RACE_CUDA(cudaMemsetAsync(plan.ticket.p, 0, sizeof(int) * 2, s));
    MpkArgs a{viewOf(plan),
              (double *)ops.x,
              plan.xf.p,
              ops.n,
              plan.runHead.p,
              plan.runDep.p,
              plan.numBlocks,
              plan.blockStart.p,
              plan.done.p,
              plan.ticket.p,
              plan.status.p,
              plan.hints,
              plan.smDie,
              plan.numDies,
              {plan.dieStart[0], plan.dieStart[1], plan.dieStart[2]}};
    switch (plan.valType) {
    case RACE_VAL_F64: launchMpk<double>(a, plan, s); break;
    case RACE_VAL_F32: launchMpk<float>(a, plan, s); break;
    case RACE_VAL_BF16: launchMpk<__nv_bfloat16>(a, plan, s); break;
    default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
    }
    RACE_CUDA(cudaGetLastError());
}

// p plain SpMV launches on the same layout.
void runSweeps(MpkPlan &plan, const race_operands &ops, cudaStream_t s) {
    for (int k = 0; k < plan.power; ++k) {
        switch (plan.valType) {
        case RACE_VAL_F64: launchSpmvSell<double>(plan, ops.n, k, (double *)ops.x, s); break;
        case RACE_VAL_F32: launchSpmvSell<float>(plan, ops.n, k, (double *)ops.x, s); break;
        case RACE_VAL_BF16: launchSpmvSell<__nv_bfloat16>(plan, ops.n, k, (double *)ops.x, s); break;
        default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
        }
        RACE_CUDA(cudaGetLastError());
    }
}

// RACE_MPK_AUTO's choice: each schedule timed on its second run (the first
// warms the code and the caches), the faster kept. Both compute the same
// powers, so the call's result is complete either way; the wavefront's
// status word is cleared afterwards, as the sweeps would leave it.
int chooseSchedule(MpkPlan &plan, const race_operands &ops, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    RACE_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return plan.valType == RACE_VAL_F64 ? RACE_MPK_WAVEFRONT : RACE_MPK_SWEEPS;
    cudaEvent_t ev[2];
    RACE_CUDA(cudaEventCreate(&ev[0]));
    RACE_CUDA(cudaEventCreate(&ev[1]));
    float ms[2] = {0.f, 0.f};
    for (int rep = 0; rep < 2; ++rep)
        for (int sc = 0; sc < 2; ++sc) {
            RACE_CUDA(cudaEventRecord(ev[0], s));
            if (sc == 0) runWavefront(plan, ops, s);
            else runSweeps(plan, ops, s);
            RACE_CUDA(cudaEventRecord(ev[1], s));
            RACE_CUDA(cudaEventSynchronize(ev[1]));
            RACE_CUDA(cudaEventElapsedTime(&ms[sc], ev[0], ev[1]));
        }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    int st = DEV_OK;
    RACE_CUDA(cudaMemcpyAsync(&st, plan.status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    RACE_CUDA(cudaStreamSynchronize(s));
    RACE_CUDA(cudaMemsetAsync(plan.status.p, 0, sizeof(int), s));
    plan.chosen = (st == DEV_OK && ms[0] <= ms[1]) ? RACE_MPK_WAVEFRONT : RACE_MPK_SWEEPS;
    return plan.chosen;
}
}  // namespace

void runMpk(Engine &e, MpkPlan &plan, const race_operands &ops, int power) {
    if (power != plan.power) throw Error(RACE_ERR_INVALID_ARG, "power differs from the planned power");
    cudaStream_t s = e.stream;
    RACE_CUDA(cudaMemsetAsync(plan.status.p, 0, sizeof(int), s));
    if (plan.valType != RACE_VAL_F64) kToFloat<<<ceilDiv(ops.n, 256), 256, 0, s>>>((const double *)ops.x, plan.xf.p, ops.n);
    if (plan.stepped) {
        switch (plan.valType) {
        case RACE_VAL_F64: launchMpkSteps<double>(plan, ops.n, (double *)ops.x, s); break;
        case RACE_VAL_F32: launchMpkSteps<float>(plan, ops.n, (double *)ops.x, s); break;
        case RACE_VAL_BF16: launchMpkSteps<__nv_bfloat16>(plan, ops.n, (double *)ops.x, s); break;
        default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
        }
        RACE_CUDA(cudaGetLastError());
        return;
    }
    const int sched = plan.schedule != RACE_MPK_AUTO ? plan.schedule : plan.chosen;
    if (sched == RACE_MPK_WAVEFRONT) runWavefront(plan, ops, s);
    else if (sched == RACE_MPK_SWEEPS) runSweeps(plan, ops, s);
    else {
        const int c = chooseSchedule(plan, ops, s);
        if (plan.chosen == 0) {  // not timed (stream capture): run the default
            if (c == RACE_MPK_WAVEFRONT) runWavefront(plan, ops, s);
            else runSweeps(plan, ops, s);
        }
    }
}

// One plain SpMV x_{k+1} = A x_k on the registered SELL layout (the p-SpMV
// baseline on the same data as the blocked kernel).
void runSpmvSell(Engine &e, MpkPlan &plan, double *x, int n, int k) {
    cudaStream_t s = e.stream;
    if (plan.valType != RACE_VAL_F64 && k == 0) kToFloat<<<ceilDiv(n, 256), 256, 0, s>>>(x, plan.xf.p, n);
    switch (plan.valType) {
    case RACE_VAL_F64: launchSpmvSell<double>(plan, n, k, x, s); break;
    case RACE_VAL_F32: launchSpmvSell<float>(plan, n, k, x, s); break;
    case RACE_VAL_BF16: launchSpmvSell<__nv_bfloat16>(plan, n, k, x, s); break;
    default: throw Error(RACE_ERR_INVALID_ARG, "unknown value type");
    }
    RACE_CUDA(cudaGetLastError());
}

void Engine::spmvPlain(int nr, const int *rowPtr, const int *col, const double *val, const double *x, double *b) {
    kSpmvCrs<<<ceilDiv(nr, 256), 256, 0, stream>>>(nr, rowPtr, col, val, x, b);
    RACE_CUDA(cudaGetLastError());
}

}  // namespace race
