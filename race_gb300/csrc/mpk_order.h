// Issue order of the matrix-power wavefront on the GPU (host code).
#pragma once
#include <vector>

namespace race {

// Work of the persistent MPK kernel. A run is up to runLen consecutive
// chunks at one power, taken by one warp with one ticket.
struct MpkOrder {
    // 4 per run: first chunk, end chunk (exclusive), power k (the run computes
    // x_{k+1} from x_k), flags (bit 0: the last power of its segment, so the
    // run's matrix entries are not read again in this call)
    std::vector<int> head;
    // 8 per run: four chunk intervals [lo, hi] whose power k-1 must be
    // complete before the run starts (hi < lo: empty; all empty for k = 0)
    std::vector<int> dep;
    // Runs are grouped by the die whose SMs run their chunks: die d's queue
    // is runs dieStart[d] .. dieStart[d+1]-1, in the global order; rank gives
    // every run's position in the global order (a run only waits on runs of
    // smaller rank).
    std::vector<int> dieStart{0, 0, 0};
    std::vector<int> rank;
    int numRuns() const { return (int)head.size() / 4; }
};

constexpr int kMpkRunDepIntervals = 4;
constexpr int kMpkMaxRunLen = 32;

// The chunk-level wavefront. depRange holds 6 ints per chunk: the chunk
// intervals its columns fall in (previous, own and next level group; hi < lo
// when empty). Chunk c at power k gets the time
//   T_0(c) = c,  T_k(c) = max_{c' <= c} T_{k-1}(maxdep(c')) + 1 + lag,
// where maxdep is the highest chunk c' reads, and, at the first power of
// every segment of segLen powers, at least (k / segLen) * numChunks + c (the
// segment sweeps the rows again from the start). Every T_k is non-decreasing
// in c and larger than T_{k-1} of every chunk the item reads, so sorting the
// items by (T / runLen, k, c) gives an order in which each item follows its
// inputs; equal-power neighbours in that order are merged into runs. The lag
// (in chunks) puts the items issued while an item's inputs are still being
// computed between the two, so that a warp taking the item rarely waits.
// chunkDie (empty: one die) gives the die whose SMs run each chunk; runs
// never mix dies.
MpkOrder mpkRunOrder(const std::vector<int> &depRange, int numChunks, int power, int segLen, int runLen,
                     int lag = 0, const std::vector<int> &chunkDie = {});

// The level-group order: step s holds power k of group s - stride*k, every
// chunk of a group in order, one chunk per run (the order of the first GPU
// executor, kept for comparison); with split > 0 the powers run in segments
// of split powers.
MpkOrder mpkGroupOrder(const std::vector<int> &depRange, const std::vector<int> &chunkGroup, int numGroups,
                       int power, int stride, int split);

// Chunks go to the two dies in blocks of kDieBlockChunks consecutive
// chunks, the blocks dealt in proportion to the dies' SM counts, so both
// dies advance through the wavefront together.
constexpr int kDieBlockChunks = 16;
std::vector<int> chunkDies(int numChunks, int smsDie0, int smsDie1);

// Completion blocks of the persistent kernel: it counts finished chunks per
// block and power instead of flagging every chunk, so a run polls one
// counter per block it reads. A block is a maximal stretch of consecutive
// chunks inside one die block (kDieBlockChunks) and one level group
// (chunkGroup; empty: no groups). Returns the block starts (numBlocks + 1
// entries, the last = numChunks).
std::vector<int> mpkFlagBlocks(int numChunks, const std::vector<int> &chunkGroup);

// depRange with every non-empty interval widened to whole blocks. An order
// built from the widened ranges has every chunk of every block a run polls
// complete before the run in the order; as blocks stay inside level groups,
// the widened ranges still lie in the previous, own and next group.
std::vector<int> widenDepsToBlocks(const std::vector<int> &depRange, const std::vector<int> &blockStart);

}  // namespace race
