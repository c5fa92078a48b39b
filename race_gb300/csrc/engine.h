// Engine state behind one race_engine handle.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "coloring.h"
#include "common.cuh"
#include "lb.h"
#include "partition.h"
#include "traverse_host.h"
#include "waves.h"

namespace race {

enum SweepMode {
    SWEEP_AUTO = RACE_SWEEP_AUTO,
    SWEEP_WAVE = RACE_SWEEP_WAVE,
    SWEEP_LEAF = RACE_SWEEP_LEAF,
    SWEEP_GATHER = RACE_SWEEP_GATHER
};

// Device copy of a phase table for the persistent sweep kernel.
struct DevPhases {
    int numPhases = 0, numLeaves = 0, maxLeaves = 0, maxLeafRows = 0;
    DevBuf<int> phasePtr, leafLo, leafHi;
};

// Schedule and layout of one registered matrix-power function: the
// permuted matrix in SELL-32 chunks inside RACE's level groups (4-entry
// groups, 16- or 32-bit columns), the chunks' dependency ranges, and the
// runs of (power, chunk) items in wavefront order, one queue per L2 die.
struct MpkPlan {
    int numChunks = 0;          // SELL-32 chunks (<= 32 rows, inside one level group)
    int power = 0;
    int numItems = 0;           // power * numChunks
    int valType = 0;
    long long sellSlots = 0;    // SELL entries including padding
    DevBuf<long long> chunkOff; // numChunks: first SELL slot of each chunk
    DevBuf<int> chunkRow;       // numChunks+1: first row of each chunk
    DevBuf<int> rowLen;         // n: non-zeros per row (-1: hub row, stored apart)
    // hub rows (more than kHubRowLen entries): contiguous CRS copies, summed
    // by a whole warp; the chunks' SELL width ignores them
    int numHubs = 0;
    DevBuf<int> hubChunkStart;  // numChunks+1: hubs of chunk c are [start[c], start[c+1])
    DevBuf<int> hubRow, hubPtr; // numHubs, numHubs+1
    DevBuf<unsigned char> hubVal;  // hub entries (type valType)
    DevBuf<int> hubCol;
    DevBuf<unsigned char> sellVal;  // sellSlots values (type valType)
    DevBuf<int> sellCol;        // sellSlots column indices (32-bit layout)
    // 16-bit layout (col16): per chunk four column window bases, per slot a
    // 2-bit window and a 14-bit offset; chunks whose columns need more
    // windows (base x < 0) keep 32-bit columns in wideCol from slot y on
    bool col16 = false;
    DevBuf<int4> chunkBase;
    DevBuf<unsigned short> sellCol16;
    DevBuf<int> wideCol;
    int wideChunks = 0;
    long long wideSlots = 0;
    DevBuf<float> xf;           // (power+1)*n FP32 powers (reduced-precision storage)
    DevBuf<int> depRange;       // numChunks*6: chunks read in the previous/own/next group
    int numRuns = 0;            // runs of the persistent kernel (mpk_order.h)
    DevBuf<int4> runHead;       // numRuns: first chunk, end chunk, power, flags | first block << 1
    DevBuf<int4> runDep;        // 2 per run: four block intervals read at the previous power
    int numDies = 1;            // run queues, one per L2 die (dies.h): die d's are dieStart[d] .. dieStart[d+1]-1
    int dieStart[3] = {0, 0, 0};
    const int *smDie = nullptr; // device table: die of every SM
    int hints = 1;              // L2 eviction hints on the matrix loads
    int schedule = 0;           // RACE_MPK_AUTO / WAVEFRONT / SWEEPS
    int chosen = 0;             // the schedule AUTO chose (0: not yet)
    int ctasPerSm = 0;          // kMpk blocks per SM (0: as many as fit)
    int numBlocks = 0;          // completion blocks (mpk_order.h mpkFlagBlocks)
    DevBuf<int> blockStart;     // numBlocks+1
    DevBuf<int> done;           // power * numBlocks: chunks complete per block
    DevBuf<int> ticket;         // next run of each die queue
    DevBuf<int> status;         // 1: device status word
    // Triangular partitions (mtxType L/U): a row may read any earlier group,
    // so the items run as one launch per wavefront step, without waits;
    // items stepPtr[s] .. stepPtr[s+1]) form step s.
    bool stepped = false;
    DevBuf<int> itemChunk;      // numItems: chunk of each work item, step order
    DevBuf<unsigned char> itemPow;  // numItems: power (0-based) of each work item
    std::vector<int> stepPtr;
};

// Device tables of one persistent block-MPK launch over one or more members
// (a member = one registered block-MPK function: matrix, x, power). Chunks
// and items of all members are numbered globally.
struct BlockMember {
    const int *rowPtr;
    const int *col;
    const void *val;
    void *x;  // (power+1) * n * nrhs, power-major, then row, right-hand side fastest
    int n;
    int power;
};

struct BatchTables {
    int valType = 0, vecType = 0, nrhs = 1, maxPower = 0;
    int numChunks = 0, numItems = 0, numMembers = 0;
    DevBuf<BlockMember> members;
    DevBuf<int> chunkMember, chunkRow, chunkEnd;  // numChunks each (local rows)
    DevBuf<int> depRange;                          // numChunks*6, global chunk ids
    DevBuf<int> itemChunk;                         // numItems
    DevBuf<unsigned char> itemPow;                 // numItems
    DevBuf<int> done;                              // maxPower * numChunks
    DevBuf<int> ticket, status;
};

// Schedule of one block-MPK function (local chunk numbering, host copies) and
// its own single-member tables.
struct BlockPlan {
    int n = 0, nrhs = 1, power = 0, valType = 0, vecType = 0, numChunks = 0;
    race_operands ops{};
    std::vector<int> chunkRow;   // numChunks+1
    std::vector<int> depRange;   // numChunks*6 (local chunk ids, empty range [0,-1])
    std::vector<int> itemChunk;  // wavefront order
    std::vector<unsigned char> itemPow;
    BatchTables tables;
};

// Device copy of a wave plan (waves.h) of one sweep direction.
struct DevWaves {
    int numWaves = 0, maxRows = 0;
    DevBuf<int> wavePtr, rows;
    // Rows above the huge-row length run in waves of their own, summed by
    // all warps of the grid: per wave a flag, per plan position the first of
    // its row's segments (positions+1), per segment its position and entry
    // range, and the segments' partial sums (3 per segment).
    int numSegs = 0;
    DevBuf<unsigned char> waveHuge;
    DevBuf<int> segFirst, segPos, segBeg, segEnd;
    DevBuf<double> segScratch;
    // SELL copy of the rows a thread runs (up to midRow entries), in plan
    // order: the rows of a wave sorted by length, cut into chunks of 32
    // positions; each position's entries in groups of four slots (entry k
    // of chunk lane l at off + 32 (k - k % 4) + 4 l + k % 4). Per wave its
    // first chunk (numWaves+1), per chunk its first slot.
    bool sell = false;
    int sellMidRow = 0;
    long long sellSlots = 0;
    DevBuf<int> waveChunk;
    DevBuf<long long> chunkOff;
    DevBuf<unsigned char> sellVal;  // sellSlots values (the operands' value type)
    DevBuf<int> sellCol;
};

// Device copy of a gather plan (waves.h) of one sweep direction, built at
// the first gather-mode call.
struct DevGather {
    bool built = false;
    DevBuf<int> ptr, entry, row;
};

struct FuncEntry {
    int kernel = 0;
    race_operands ops{};
    int power = 1;
    std::unique_ptr<MpkPlan> mpk;
    std::unique_ptr<BlockPlan> block;  // block MPK (race_register_mpk_block)
    DevWaves waves[2];  // forward, reverse
    DevGather gather[2];
};

class Engine {
  public:
    Engine(int nrow, int nthreads, int dist, const int *rowPtr, const int *col, bool symmHint, const int *initPerm,
           const int *initInvPerm, int d2, int lbTarget, const Params &params);
    ~Engine();

    void color();
    void powerPrepare(int highestPower, double cacheSize, double safety, const std::string &mtxType, int subPower);

    // One traversal of [lo,hi) of the current permuted space on the GPU.
    LevelData traverse(int lo, int hi, int mode, const std::string &mtxType = "N");
    long long rangeNnz(int lo, int hi) const;

    int registerFunction(int kernel, const race_operands &ops, int power);
    int registerMpkBlock(const race_operands &ops, int power, int nrhs);
    void execute(int id, bool rev);
    void launch(int id, bool rev);
    void checkStatus();
    int *lastStatus = nullptr;  // device status word of the last launch
    void spmvPlain(int n, const int *rowPtr, const int *col, const double *val, const double *x, double *b);

    int n = 0;
    long long nnz = 0;          // of the traversal graph (symmetrised pattern)
    int dist = 1, requested = 1, d2 = 0, lbTarget = 1;
    Params params;
    cudaStream_t stream = 0;
    std::string lastError;

    std::vector<int> hRowPtr, hCol;  // traversal graph (host)
    std::vector<int> hPerm, hInvPerm;
    DevBuf<int> dRowPtr, dCol, dPerm, dInvPerm;

    // traversal scratch
    DevBuf<int> dDist, dStamp, dQ0, dQ1, dCtr, dLevelRow, dLevelNnz, dKeys, dVals, dKeysOut, dValsOut, dTmp;
    DevBuf<unsigned char> dCubTemp;
    int stamp = 0;

    // sweep execution: SWEEP_AUTO (gather for SpMV/SpMTV/SymmSpMV, else wave
    // or leaf by cost), SWEEP_WAVE (bit-exact wave plans), SWEEP_LEAF (warp
    // per leaf), SWEEP_GATHER
    int sweepMode = SWEEP_AUTO;
    // wave mode: rows of up to this many entries run one thread each, longer
    // ones (up to 512) one warp each; both keep the sequential order (-1:
    // 16 for FP64 vectors, 8 for FP32, the fastest measured on the 4.2M-row
    // power-law GS). With sweepSell the thread rows read a SELL copy in plan
    // order (coalesced vector loads) instead of the caller's CRS.
    int sweepMidRow = -1;
    bool sweepSell = true;

    // coloring results
    std::unique_ptr<ZoneTree> tree;
    int availableThreads = 0;
    bool colored = false;
    PhaseTable phases[2];
    DevPhases dPhases[2];

    // power results
    // MPK issue order and kernel (mpk_order.h, mpk.cu): order 0 the
    // chunk-level wavefront, 1 the level-group order with stride mpkStride
    // (1: RACE's, 2); powers per segment (0: all powers in one sweep);
    // chunks per run; lag in chunks; one queue per L2 die; eviction hints;
    // blocks per SM (0: as many as fit); 16-bit column layout where the
    // columns fit, with windows of mpkColWindow rows (at most
    // kMpkColWindow; smaller windows only make more chunks keep 32-bit
    // columns). The defaults are the fastest measured on the 128^3 27-point
    // stencil.
    int mpkOrder = 0;
    int mpkStride = 2;
    int mpkSplit = 0;
    int mpkRun = 4;
    int mpkLag = 32768;
    bool mpkDieQueues = true;
    int mpkHints = 1;
    int mpkCtasPerSm = 0;
    bool mpkCol16 = true;
    // the default schedule of new MPK functions (RACE_MPK_*)
    int mpkSchedule = 0;
    int mpkColWindow = kMpkColWindow;
    // the MPK partition's leaf tree (the root alone without hopeless regions)
    std::vector<MpkLeaf> powerTree;
    // Coloring ranges shorter than this are traversed on the host (all of
    // them for graphs with rows above 1024 entries, else below 2^20 rows;
    // RACE_GPU_HOST_TRAVERSE_BELOW overrides, 0: never); the device
    // permutation is then refreshed before the next GPU traversal and at the
    // end of the coloring.
    int hostTraverseBelow = 1 << 20;
    bool devPermStale = false;
    HostTraverseScratch hostScratch;
    void syncDevicePerm();
    bool powerReady = false;
    int highestPower = 1, highestSubPower = 1;
    std::vector<int> levelPtr, groupPtr, unlockRow, dangerRow;
    bool powerLevelsCached = false;
    std::string powerLevelsType;
    LevelData powerLevels;

    std::vector<FuncEntry> funcs;
    DevBuf<int> dStatus;
};

}  // namespace race
