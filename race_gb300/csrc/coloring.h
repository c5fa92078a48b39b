// Recursive level coloring: the zone tree RACE builds for distance-1 and
// distance-2 coloring (src/zone_tree.cpp, src/level_recursion.cpp), and its
// flattening into barrier-separated phases for the persistent sweep kernel.
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "lb.h"

namespace race {

// ZoneLeaf (include/zone_tree.h:31-49)
struct ZoneNode {
    std::vector<int> valueZ;    // sub-block row offsets [lo, ..., hi]
    std::vector<int> children;  // pairs [first,last) of child indices per sub-block
    int nthreadsZ = 1;
    int idealNthreadsZ = 1;
    int totalSubBlocks = 1;
    int parentZ = -1;
    int effRowZ = 0;
    int stage = 0;
    bool reachedLimit = false;
    ZoneNode() = default;
    ZoneNode(int lo, int hi, int parent) : valueZ{lo, hi}, parentZ(parent), effRowZ(hi - lo) {}
};

// Knobs the reference reads from the environment (level_recursion.cpp:48-90,
// graph_SoA.cpp:321-330, matrixPowerRecursive.cpp:37-61).
struct Params {
    std::vector<double> effVec{40.0};  // [0] default, [k] stage k (RACE_EFFICIENCY)
    std::vector<int> lvlThreads;       // RACE_THREADS
    int cacheViolationCutoffDefault = 50;
    std::vector<int> cacheViolationCutoff{50};
    int maxRecStages = -1;             // RACE_MAX_RECURSION_STAGES (-1: unset)
    static Params fromEnv();
    double efficiency(unsigned level) const { return level < effVec.size() ? effVec[level] : effVec[0]; }
    int threadsAt(unsigned level) const { return (level - 1) < lvlThreads.size() ? lvlThreads[level - 1] : -1; }
};

// One traversal of rows [lo,hi) of the current permuted index space: BFS,
// level histogram, stable level sort composed into the running permutation.
// Implemented on the GPU by the engine.
using TraverseFn = std::function<LevelData(int lo, int hi)>;
// Non-zeros of rows [lo,hi) of the current permuted space.
using RangeNnzFn = std::function<long long(int lo, int hi)>;

class ZoneTree {
  public:
    ZoneTree(int dist, int d2, int lbTarget) : dist_(dist), d2_(d2), lbTarget_(lbTarget) {}
    std::vector<ZoneNode> nodes;
    int maxStage = 1;
    // ZoneTree::spawnChild (zone_tree.cpp:243-305)
    bool spawnChild(int parentIdx, int parentSubIdx, int requestNthreads, const LevelData &ld, double eff);
    int bpt() const { return blockPerThread(dist_, d2_); }
    int dist() const { return dist_; }

  private:
    void updateTreeEffRow(int parentIdx);
    void updateTreeNThreads(int parentIdx);
    int findKeyChildEffRow(int parentIdx) const;
    int dist_, d2_, lbTarget_;
};

// LevelRecursion (level_recursion.cpp:28-376)
class LevelRecursion {
  public:
    LevelRecursion(int nrow, int requested, int dist, int d2, int lbTarget, const Params &params, TraverseFn trav,
                   RangeNnzFn rangeNnz);
    void levelBalancing();
    ZoneTree tree;
    int availableThreads = 0;

  private:
    void calculateIdealNthreads(int parentIdx, int parentSubIdx, int currLvl);
    void recursivePartition(int parentIdx, int parentSubIdx, int currLevel);
    int nrow_, requested_, dist_, d2_, lbTarget_;
    Params params_;
    TraverseFn trav_;
    RangeNnzFn rangeNnz_;
};

// Execution order of a zone tree flattened into phases. Leaves of one phase
// touch disjoint neighbourhoods and may run concurrently; a phase starts
// after the previous one has finished (FuncManager::Run and recursiveCall,
// functionManager.cpp:201-265, 1453-1501).
struct PhaseTable {
    std::vector<int> phasePtr;  // numPhases+1 offsets into leaves
    std::vector<int> leafLo;    // first row of each leaf (in execution direction)
    std::vector<int> leafHi;    // one past the last row (exclusive bound, direction-aware)
    int numPhases() const { return (int)phasePtr.size() - 1; }
};

// rev=false: forward sweep; rev=true: the reverse sweep (blocks in reverse
// order, rows descending), as executeFunction(id, rev) does. The dense-row
// serial tail [serialLo, serialHi) becomes a final single-leaf phase.
PhaseTable flattenZoneTree(const ZoneTree &t, bool rev, int serialLo, int serialHi);

// Flat serialisation shared with the oracle harness: [numNodes] then per node
// [nthreadsZ, idealNthreadsZ, totalSubBlocks, parentZ, effRowZ, stage,
//  reachedLimit, nValueZ, valueZ..., nChildren, children...].
std::vector<int> serializeZoneTree(const ZoneTree &t);

}  // namespace race
