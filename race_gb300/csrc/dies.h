// L2 die map of the current GPU (dies.cu).
#pragma once
#include <array>
#include <memory>
#include <vector>

#include "common.cuh"

namespace race {

struct DieMap {
    int numDies = 1;                  // 2 on GB300; 1 where no split was measured
    std::vector<int> smDie;           // die of every SM (index: %smid)
    std::array<int, 2> smsPerDie{};   // SMs of each die
    DevBuf<int> smDieDev;             // device copy of smDie
};

// The die map of the current device, measured at its first use in the
// process (well under a millisecond of GPU time; synchronises the device,
// so the first call must not come while a stream is being captured).
// RACE_GPU_DIE_AFFINITY=0 skips the measurement and reports one die.
const DieMap &dieMap();

}  // namespace race
