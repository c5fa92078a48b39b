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

}  // namespace race
