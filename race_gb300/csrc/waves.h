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

}  // namespace race
