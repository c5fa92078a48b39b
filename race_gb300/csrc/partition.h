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

}  // namespace race
