// Single-stage MPK partition of RACE (mtxPower::findPartition for one
// shared-cache domain, src/matrixPower.cpp:505-605): cache-violating levels,
// hopeless regions (identifyHopelessRegions, :147-503) and the consolidated
// level groups (consolidatePartition, :685-940). Host code; the levels come
// from the engine's BFS.
#pragma once
#include <vector>

#include "lb.h"

namespace race {

struct StagePartition {
    std::vector<int> groupPtr;   // groups+1 row offsets (the reference's consolidated levelPtr, MPLeaf::lp)
    std::vector<int> hopeless;   // groups that are hopeless regions (MPLeaf::hid), ascending
    std::vector<int> unlockRow;  // per group: rows before it are what the previous group's next power needs
    std::vector<int> dangerRow;  // per group: rows from it on need the next group
};

// `power` is highestPower * highestSubPower; `cutoff` the stage's cache
// violation cut-off (INT_MAX disables hopeless regions); graphRows and
// graphNnz give the bytes per non-zero (getBytePerNNZ, :134-140).
StagePartition stagePartition(const LevelData &ld, int startRow, int power, int graphRows, long long graphNnz,
                              double cacheSize, double safety, int cutoff);

// The permutation of one recursion stage into the hopeless groups
// (mtxPowerRecursive::recursivePartition, matrixPowerRecursive.cpp:156-298,
// with Traverse on a range with boundaries, traverse_GAP_graphSoA.cpp:31-90,
// 135-330, 452-575), which is the whole recursion at the default settings:
// for each hopeless group h of groupPtr in turn, a BFS of the group's rows
// from its first row that also walks (without counting) the rows of the
// boundary groups h-w..h+w, w = ceil(power/2)-1; islands of the group
// restart it on the same level; unvisited boundary rows get the level after
// the last. The group and every non-empty boundary group are then sorted
// stably by level and the sort is composed into totalPerm/totalInvPerm
// (new index -> original row and back). rowPtr/col: the traversal pattern,
// indexed by original rows. Returns false if rows of a group went missing.
bool recursePermutation(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                        std::vector<int> &totalInvPerm, const std::vector<int> &groupPtr,
                        const std::vector<int> &hopeless, int power);

// One leaf of the MPK recursion tree (MPLeaf, include/matrixPowerRecursive.h):
// its rows, stage, parent leaf, consolidated level groups and hopeless groups.
struct MpkLeaf {
    int lo = 0, hi = 0, stage = 0, parent = -1;
    std::vector<int> groupPtr;  // MPLeaf::lp
    std::vector<int> hopeless;  // MPLeaf::hid
};

// The whole MPK recursion below a stage-0 partition `root` of rows [0, n)
// (mtxPowerRecursive::recursivePartition, matrixPowerRecursive.cpp:156-338),
// at any depth. Depth first, for each hopeless group h of a leaf in turn, a
// child leaf takes the group's rows and as boundaries (:199-287) the leaf's
// own groups h-w..h+w other than h and, of every boundary region of the
// leaf, its consolidated level groups h-w..h+w (h-1..h+1 as one region),
// w = ceil(power/2)-1, empty ranges left out. The child's BFS (as in
// recursePermutation) permutes its rows and boundary rows; its levels are
// then partitioned like stage 0 (mtxPower::findPartition, matrixPower.cpp:
// 505-605) except that a level's size includes the boundary rows' non-zeros
// of that level (getElemUpperLimit, :88-99), with the cut-off of its stage,
// stageCutoff[stage] (INT_MAX from stageCutoff.size() on); a child with
// hopeless groups recurses before its next sibling is built. Every stage's
// permutation is composed into totalPerm/totalInvPerm; `tree` gets the root
// and every leaf in the reference's order. Returns false if rows of a group
// went missing or a hopeless group lacks its boundary groups.
bool recursivePartition(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                        std::vector<int> &totalInvPerm, const StagePartition &root, int power, long long graphNnz,
                        double cacheSize, double safety, const std::vector<int> &stageCutoff,
                        std::vector<MpkLeaf> &tree);

}  // namespace race
