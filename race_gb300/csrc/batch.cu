// Block matrix-power kernel over many right-hand sides and many matrices in
// one persistent launch.
//
// A block-MPK function is RACE's matrix power (src/matrixPower.cpp level
// groups, executor src/functionManager.cpp:618-823) applied to nrhs vectors
// at once: x_k[r][j] = sum_c A[r][c] x_{k-1}[c][j] for j < nrhs, with x
// stored power-major, then row, then right-hand side (one 8- or 4-byte
// element per right-hand side, consecutive), so a row's nrhs values are one
// contiguous segment. The reference has no multi-vector or multi-matrix
// form: each RACE::Interface runs one matrix with one vector.
//
// Thread mapping: R = nrhs lanes per row (R in {1,2,4,8,16,32}), 32/R rows
// per warp pass. Each lane walks its row's CRS entries in order as a
// sequential fused multiply-add chain, so every right-hand side is computed
// exactly like a single-vector SpMV (MAT_SPMV_KERNEL's order,
// examples/src/helpers/kernels.cpp:749-777): FP64 results are bit-identical
// to p sequential fma SpMVs per right-hand side. The lanes of one row read
// the same value and column (a broadcast) and R consecutive x entries.
//
// Schedule: chunks of <= 32 rows inside level groups; a work item is
// (power, chunk); items of one member follow the stride-2 wavefront of the
// single-vector kernel and members follow each other. Persistent warps take
// items from a global ticket; an item waits (bounded) for the chunks of the
// previous power its columns fall in. Dependencies stay inside a member and
// point to earlier tickets, so the launch cannot deadlock; the next member's
// items fill the warps that the tail of the previous member's wavefront
// leaves idle. A batch is one memset of the completion flags plus one
// kernel, and can be captured once in a CUDA graph and replayed.
#include <algorithm>

#include <cuda_bf16.h>

#include "engine.h"

namespace race {

bool chunkDependencyRanges(const int *rowPtr, const int *col, const std::vector<int> &chunkRow,
                           const std::vector<int> &chunkGroup, std::vector<int> &range, cudaStream_t s);

namespace {

constexpr int kBlockThreads = 256;

__device__ __forceinline__ int ldAcquireB(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ double mulAdd(double v, double x, double acc) { return fma(v, x, acc); }
__device__ __forceinline__ float mulAdd(float v, float x, float acc) { return fmaf(v, x, acc); }
__device__ __forceinline__ float mulAdd(__nv_bfloat16 v, float x, float acc) {
    return fmaf(__bfloat162float(v), x, acc);
}

struct BlockArgs {
    const BlockMember *members;
    const int *chunkMember, *chunkRow, *chunkEnd;
    const int *depRange;
    const int *itemChunk;
    const unsigned char *itemPow;
    int numItems, numChunks;
    int *done, *ticket, *status;
};

// V consecutive right-hand sides of one row as one 16-byte (or smaller)
// vector access.
template <typename XT, int V>
struct alignas(sizeof(XT) * V) XVec {
    XT v[V];
};

// Right-hand sides per lane: one 16-byte access (FP64: 2, FP32: 4), at most R.
template <typename XT, int R>
__host__ __device__ constexpr int kVecOf() {
    return R < (int)(16 / sizeof(XT)) ? R : (int)(16 / sizeof(XT));
}

// Rows [r0, r1) (at most 32) of one member at power k -> k+1, all right-hand
// sides. A lane owns V consecutive right-hand sides of one row (R/V lanes per
// row, 32V/R rows per pass) and runs one sequential fma chain per right-hand
// side over the row's entries in CRS order. The rows' offsets are read once
// per range by one coalesced load and passed around by shuffles.
template <typename VT, typename XT, int R>
__device__ __forceinline__ void blockRows(const BlockMember &m, int r0, int r1, int k) {
    constexpr int V = kVecOf<XT, R>();
    constexpr int L = R / V;        // lanes per row
    constexpr int RPP = 32 / L;     // rows per pass
    using Vec = XVec<XT, V>;
    const int lane = threadIdx.x & 31;
    const int sub = lane / L, q = lane % L;
    const int nr = r1 - r0;
    const VT *__restrict__ val = (const VT *)m.val;
    const int *__restrict__ col = m.col;
    const XT *xin = (const XT *)m.x + (size_t)k * m.n * R + q * V;
    XT *xout = (XT *)m.x + (size_t)(k + 1) * m.n * R + q * V;
    const int rs = lane < nr ? m.rowPtr[r0 + lane] : 0;
    const int rEnd = m.rowPtr[r1];
    for (int base = 0; base < nr; base += RPP) {
        const int i = base + sub;
        const int e0 = __shfl_sync(0xffffffffu, rs, min(i, 31));
        const int eNext = __shfl_sync(0xffffffffu, rs, min(i + 1, 31));
        if (i < nr) {
            const int e1 = i + 1 < nr ? eNext : rEnd;
            Vec acc;
#pragma unroll
            for (int t = 0; t < V; ++t) acc.v[t] = XT(0);
#pragma unroll 4
            for (int e = e0; e < e1; ++e) {
                const VT a = val[e];
                const Vec xv = *reinterpret_cast<const Vec *>(xin + (size_t)col[e] * R);
#pragma unroll
                for (int t = 0; t < V; ++t) acc.v[t] = mulAdd(a, xv.v[t], acc.v[t]);
            }
            *reinterpret_cast<Vec *>(xout + (size_t)(r0 + i) * R) = acc;
        }
    }
}

template <typename VT, typename XT, int R>
__global__ void __launch_bounds__(kBlockThreads) kMpkBlock(BlockArgs a) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.ticket, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= a.numItems) return;
        const int t = a.itemChunk[it];
        const int k = a.itemPow[it];
        if (k > 0) {
            const int *rg = a.depRange + 6 * t;
            const int *done = a.done + (size_t)(k - 1) * a.numChunks;
            long long spins = 0;
            for (;;) {
                bool ok = true;
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    for (int i = rg[2 * d] + lane; i <= rg[2 * d + 1]; i += 32)
                        if (ldAcquireB(done + i) == 0) ok = false;
                if (__all_sync(0xffffffffu, ok)) break;
                if (++spins > kSpinLimit || ldAcquireB(a.status) != DEV_OK) {
                    if (lane == 0) atomicCAS(a.status, DEV_OK, DEV_WAIT_TIMEOUT);
                    return;
                }
                __nanosleep(32);
            }
        }
        const BlockMember m = a.members[a.chunkMember[t]];
        blockRows<VT, XT, R>(m, a.chunkRow[t], a.chunkEnd[t], k);
        __syncwarp();
        if (lane == 0)
            asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(a.done + (size_t)k * a.numChunks + t), "r"(1)
                         : "memory");
    }
}

// Plain x_{k+1} = A x_k for all right-hand sides of one member (the
// p-launch baseline on the same data).
template <typename VT, typename XT, int R>
__global__ void __launch_bounds__(kBlockThreads) kSpmvBlock(BlockMember m, int k) {
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int rowsPerWarp = 32;
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); (long long)w * rowsPerWarp < m.n; w += warps)
        blockRows<VT, XT, R>(m, w * rowsPerWarp, min(m.n, (w + 1) * rowsPerWarp), k);
}

template <typename K>
int residentBlocksOf(K kernel) {
    int dev = 0, sms = 0, occ = 0;
    RACE_CUDA(cudaGetDevice(&dev));
    RACE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    RACE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kBlockThreads, 0));
    return sms * std::max(occ, 1);
}

template <typename VT, typename XT, int R>
void launchBlock(const BlockArgs &a, cudaStream_t s) {
    static const int blocks = residentBlocksOf(kMpkBlock<VT, XT, R>);
    kMpkBlock<VT, XT, R><<<blocks, kBlockThreads, 0, s>>>(a);
}

template <typename VT, typename XT, int R>
void launchSpmv(const BlockMember &m, int k, cudaStream_t s) {
    static const int blocks = residentBlocksOf(kSpmvBlock<VT, XT, R>);
    const int need = ceilDiv(ceilDiv(m.n, 32), kBlockThreads / 32);
    kSpmvBlock<VT, XT, R><<<std::max(1, std::min(blocks, need)), kBlockThreads, 0, s>>>(m, k);
}

// Type and width dispatch: (FP64 values, FP64 x), (FP32, FP32), (BF16, FP32).
template <template <typename, typename, int> class Fn, typename... A>
void dispatch(int valType, int vecType, int nrhs, A &&...args) {
    auto byWidth = [&](auto tag) {
        using VT = typename decltype(tag)::first_type;
        using XT = typename decltype(tag)::second_type;
        switch (nrhs) {
        case 1: Fn<VT, XT, 1>::run(args...); break;
        case 2: Fn<VT, XT, 2>::run(args...); break;
        case 4: Fn<VT, XT, 4>::run(args...); break;
        case 8: Fn<VT, XT, 8>::run(args...); break;
        case 16: Fn<VT, XT, 16>::run(args...); break;
        case 32: Fn<VT, XT, 32>::run(args...); break;
        default: throw Error(RACE_ERR_INVALID_ARG, "nrhs must be 1, 2, 4, 8, 16 or 32");
        }
    };
    if (valType == RACE_VAL_F64 && vecType == RACE_VAL_F64) byWidth(std::pair<double, double>{});
    else if (valType == RACE_VAL_F32 && vecType == RACE_VAL_F32) byWidth(std::pair<float, float>{});
    else if (valType == RACE_VAL_BF16 && vecType == RACE_VAL_F32) byWidth(std::pair<__nv_bfloat16, float>{});
    else throw Error(RACE_ERR_INVALID_ARG, "block MPK types: FP64 values with FP64 x, or FP32/BF16 values with FP32 x");
}

template <typename VT, typename XT, int R>
struct LaunchBlockFn {
    static void run(const BlockArgs &a, cudaStream_t s) { launchBlock<VT, XT, R>(a, s); }
};
template <typename VT, typename XT, int R>
struct LaunchSpmvFn {
    static void run(const BlockMember &m, int k, cudaStream_t s) { launchSpmv<VT, XT, R>(m, k, s); }
};

}  // namespace

void validateBlockTypes(int valType, int vecType, int nrhs) {
    if (!((valType == RACE_VAL_F64 && vecType == RACE_VAL_F64) ||
          ((valType == RACE_VAL_F32 || valType == RACE_VAL_BF16) && vecType == RACE_VAL_F32)))
        throw Error(RACE_ERR_INVALID_ARG, "block MPK types: FP64 values with FP64 x, or FP32/BF16 values with FP32 x");
    if (nrhs != 1 && nrhs != 2 && nrhs != 4 && nrhs != 8 && nrhs != 16 && nrhs != 32)
        throw Error(RACE_ERR_INVALID_ARG, "nrhs must be 1, 2, 4, 8, 16 or 32");
}

void buildBatchTables(BatchTables &t, const std::vector<const BlockPlan *> &plans, cudaStream_t s) {
    if (plans.empty()) throw Error(RACE_ERR_INVALID_ARG, "empty batch");
    const BlockPlan &p0 = *plans[0];
    t.valType = p0.valType;
    t.vecType = p0.vecType;
    t.nrhs = p0.nrhs;
    t.maxPower = 0;
    std::vector<BlockMember> mem;
    std::vector<int> cMember, cRow, cEnd, range, iChunk;
    std::vector<unsigned char> iPow;
    int base = 0;
    for (size_t m = 0; m < plans.size(); ++m) {
        const BlockPlan &p = *plans[m];
        if (p.valType != t.valType || p.vecType != t.vecType || p.nrhs != t.nrhs)
            throw Error(RACE_ERR_INCOMPATIBILITY, "batch members differ in value type, vector type or nrhs");
        t.maxPower = std::max(t.maxPower, p.power);
        mem.push_back(BlockMember{p.ops.rowPtr, p.ops.col, p.ops.val, p.ops.x, p.n, p.power});
        for (int c = 0; c < p.numChunks; ++c) {
            cMember.push_back((int)m);
            cRow.push_back(p.chunkRow[c]);
            cEnd.push_back(p.chunkRow[c + 1]);
            for (int d = 0; d < 3; ++d) {
                const int lo = p.depRange[6 * c + 2 * d], hi = p.depRange[6 * c + 2 * d + 1];
                range.push_back(hi < lo ? 0 : lo + base);  // empty stays empty: [0,-1]
                range.push_back(hi < lo ? -1 : hi + base);
            }
        }
        for (size_t i = 0; i < p.itemChunk.size(); ++i) {
            iChunk.push_back(p.itemChunk[i] + base);
            iPow.push_back(p.itemPow[i]);
        }
        base += p.numChunks;
    }
    t.numMembers = (int)plans.size();
    t.numChunks = base;
    t.numItems = (int)iChunk.size();
    t.members.upload(mem.data(), mem.size(), s);
    t.chunkMember.upload(cMember.data(), std::max<size_t>(cMember.size(), 1), s);
    t.chunkRow.upload(cRow.data(), std::max<size_t>(cRow.size(), 1), s);
    t.chunkEnd.upload(cEnd.data(), std::max<size_t>(cEnd.size(), 1), s);
    t.depRange.upload(range.data(), std::max<size_t>(range.size(), 1), s);
    t.itemChunk.upload(iChunk.data(), std::max<size_t>(iChunk.size(), 1), s);
    t.itemPow.upload(iPow.data(), std::max<size_t>(iPow.size(), 1), s);
    t.done.alloc(std::max<size_t>((size_t)t.maxPower * t.numChunks, 1));
    t.ticket.alloc(1);
    t.status.alloc(1);
    RACE_CUDA(cudaMemsetAsync(t.status.p, 0, sizeof(int), s));
    RACE_CUDA(cudaStreamSynchronize(s));
}

std::unique_ptr<BlockPlan> buildBlockPlan(Engine &e, const race_operands &ops, int power, int nrhs) {
    validateBlockTypes(ops.val_type, ops.vec_type, nrhs);
    // lanes read up to 16 bytes of consecutive right-hand sides at once
    const size_t xs = ops.vec_type == RACE_VAL_F64 ? 8 : 4;
    const size_t vecBytes = std::min<size_t>(16, xs * nrhs);
    if (reinterpret_cast<uintptr_t>(ops.x) % vecBytes != 0)
        throw Error(RACE_ERR_INVALID_ARG, "block MPK x must be aligned to min(16, nrhs * element size) bytes");
    auto plan = std::make_unique<BlockPlan>();
    plan->n = ops.n;
    plan->nrhs = nrhs;
    plan->power = power;
    plan->valType = ops.val_type;
    plan->vecType = ops.vec_type;
    plan->ops = ops;
    const std::vector<int> &gp = e.groupPtr;
    const int G = (int)gp.size() - 1;
    std::vector<int> chunkGroup;
    plan->chunkRow.assign(1, 0);
    for (int g = 0; g < G; ++g)
        for (int r = gp[g]; r < gp[g + 1]; r += 32) {
            plan->chunkRow.push_back(std::min(gp[g + 1], r + 32));
            chunkGroup.push_back(g);
        }
    const int C = (int)chunkGroup.size();
    plan->numChunks = C;
    if (!chunkDependencyRanges(ops.rowPtr, ops.col, plan->chunkRow, chunkGroup, plan->depRange, e.stream))
        throw Error(RACE_ERR_INVALID_ARG,
                    "MPK operand is not in the engine's level order (permute it with getPerm/getInvPerm)");
    // stride-2 wavefront over (group, power), as the single-vector kernel
    std::vector<int> groupFirst(G + 1, C);
    for (int t = C - 1; t >= 0; --t) groupFirst[chunkGroup[t]] = t;
    for (int g = G - 1; g >= 0; --g) groupFirst[g] = std::min(groupFirst[g], groupFirst[g + 1]);
    const int stride = e.mpkStride == 1 ? 1 : 2;
    for (int st = 0; st < G + stride * (power - 1); ++st)
        for (int k = 0; k < power; ++k) {
            const int g = st - stride * k;
            if (g < 0 || g >= G) continue;
            for (int t = groupFirst[g]; t < groupFirst[g + 1]; ++t) {
                plan->itemChunk.push_back(t);
                plan->itemPow.push_back((unsigned char)k);
            }
        }
    buildBatchTables(plan->tables, {plan.get()}, e.stream);
    return plan;
}

// Resets the completion flags, ticket and status word and launches the
// persistent kernel: all stream-ordered, so the sequence can be captured.
void runBatch(BatchTables &t, cudaStream_t s) {
    RACE_CUDA(cudaMemsetAsync(t.done.p, 0, sizeof(int) * (size_t)t.maxPower * t.numChunks, s));
    RACE_CUDA(cudaMemsetAsync(t.ticket.p, 0, sizeof(int), s));
    RACE_CUDA(cudaMemsetAsync(t.status.p, 0, sizeof(int), s));
    if (t.numItems == 0) return;
    BlockArgs a{t.members.p, t.chunkMember.p, t.chunkRow.p, t.chunkEnd.p, t.depRange.p, t.itemChunk.p,
                t.itemPow.p, t.numItems, t.numChunks, t.done.p, t.ticket.p, t.status.p};
    dispatch<LaunchBlockFn>(t.valType, t.vecType, t.nrhs, a, s);
    RACE_CUDA(cudaGetLastError());
}

void runBlockSpmv(const BlockPlan &p, int k, cudaStream_t s) {
    const BlockMember m{p.ops.rowPtr, p.ops.col, p.ops.val, p.ops.x, p.n, p.power};
    if (p.n == 0) return;
    dispatch<LaunchSpmvFn>(p.valType, p.vecType, p.nrhs, m, k, s);
    RACE_CUDA(cudaGetLastError());
}

}  // namespace race
