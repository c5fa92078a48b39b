// Wave plans: RACE's execution order compiled into conflict-free waves
// (see waves.cpp).
#pragma once
#include <vector>

#include "../../include/race_gb300.h"
#include "coloring.h"

namespace race {

struct WavePlan {
    std::vector<int> wavePtr;  // numWaves+1 offsets into rows
    std::vector<int> rows;     // rows grouped by wave, RACE order inside a wave
    int numWaves() const { return (int)wavePtr.size() - 1; }
};

// Wave plan of built-in kernel `kernel` (RACE_K_*) on the operand matrix
// (host CRS) for the execution order given by a phase table.
WavePlan buildWavePlan(int kernel, int n, const int *rowPtr, const int *col, const PhaseTable &pt);

// Gather plan of a scatter kernel (SpMTV or SymmSpMV) for one sweep
// direction: the same updates, grouped by the entry of b they write, so
// that every entry of b is produced by one thread in one launch. For entry
// y the updates are listed in RACE's execution order of the rows that make
// them, each as (entry, row): entry >= 0 is `b[y] = fma(val[entry],
// x[row], b[y])`; for SymmSpMV, entry -1 marks row y's own update (its
// diagonal fma, then b[y] += its off-diagonal dot product). Replaying them
// in that order performs the sequential walk's operations on b[y] in the
// same order, so the results are identical bit for bit.
struct GatherPlan {
    std::vector<int> ptr;    // n+1 offsets into entry/row
    std::vector<int> entry;  // matrix entry of each update (-1: own row, SymmSpMV)
    std::vector<int> row;    // row whose x the update reads (its source row)
};

GatherPlan buildGatherPlan(int kernel, int n, const int *rowPtr, const int *col, const PhaseTable &pt);

}  // namespace race
