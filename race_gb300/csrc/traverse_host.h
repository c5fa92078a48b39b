// Host BFS of one row range with RACE's distance-1/distance-2 rules: the
// same levels, level histogram and permutation as the engine's GPU
// traversal (Engine::traverse), for ranges too short to be worth the GPU's
// launches and host round trips. Host code.
#pragma once
#include <vector>

#include "lb.h"

namespace race {

// Per-row scratch of host traversals: a stamp per row (a row belongs to the
// traversal whose stamp it carries), a level per row of the range, and a
// frontier mark per row for the pull steps.
struct HostTraverseScratch {
    std::vector<int> stamp, dist, frontier, next;
    int stampVal = 0;
    std::vector<long long> mark;
    long long markVal = 0;
};

// Traverse::calculateDistance + createLevelData + permuteGraph
// (traverse_GAP_graphSoA.cpp:135-221, 236-383, 385-504, 506-641) for rows
// [lo, hi) of the current permuted space, mode 1 (distance-1) or 2
// (distance-2: rows outside the range reached from rows inside it are
// walked without a level). Roots: lo, then on an exhausted frontier the
// lowest row without a level, one level further. Levels count the rows of
// the range and their non-zeros (row lengths of the traversal graph
// rowPtr/col, indexed by original rows); the range is then sorted stably by
// level and the sort is composed into totalPerm/totalInvPerm (new index ->
// original row and back). Returns false if rows of the range went missing.
// Distance-2 steps are direction-optimised (Beamer, Asanovic, Patterson,
// SC 2012): when the rows outside the range in the frontier have more
// non-zeros than the unvisited rows of the range, those rows are marked and
// every unvisited row of the range looks for a marked neighbour in its own
// row instead (the graph must be structurally symmetric, as the engine's
// traversal graph is). BFS levels, hence the result, do not depend on it.
bool traverseRangeHost(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                       std::vector<int> &totalInvPerm, int lo, int hi, int mode, HostTraverseScratch &s,
                       LevelData &ld);

}  // namespace race
