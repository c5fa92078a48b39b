// Level load balancer: splits the BFS levels of one row range into zones,
// blockPerThread (red/black) zones per thread, balancing rows or non-zeros.
// Restates RACE's LB class (src/lb.cpp, include/lb.h) so that zone
// boundaries and thread counts are identical to the reference's for the
// same level data, thread request and efficiency threshold.
#pragma once
#include <vector>

namespace race {

enum Dist { DIST_ONE = 1, DIST_TWO = 2, DIST_POWER = 3 };
enum D2Method { TWO_BLOCK = 0, THREE_BLOCK = 1 };
enum LBTarget { LB_ROW = 0, LB_NNZ = 1 };

// macros.h:29-38
inline int blockPerThread(int dist, int d2) { return dist == DIST_POWER ? 1 : dist == DIST_ONE ? 2 : d2 == TWO_BLOCK ? 2 : 3; }
inline int minGap(int dist, int d2) { return dist == DIST_POWER ? 1 : dist == DIST_ONE ? 1 : d2 == TWO_BLOCK ? 2 : 1; }

struct LevelData {
    std::vector<int> levelRow, levelNnz;
    int totalLevel = 0;
    long long nrow = 0, nnz = 0;
};

struct LBResult {
    std::vector<int> scale;       // threads each current-level thread may spawn next
    std::vector<int> zonePtr;     // totalBlocks+1 row offsets (base-shifted)
    std::vector<int> subZonePtr;  // totalSubBlocks+1 row offsets (base-shifted)
    std::vector<int> numBlocks;   // sub-blocks per zone
};

// LB::balance (lb.cpp:767-771) followed by getZonePtr/getSubZonePtr/
// getNumBlocks (lb.cpp:709-733). `eff` is the efficiency threshold in percent.
LBResult lbBalance(const LevelData &ld, int nThreads, double eff, int dist, int d2, int lbTarget, int base);

// roundDouble, utility.h:194-198
inline int roundDouble(double v) {
    int vi = static_cast<int>(v);
    return ((v - vi) < 0.5) ? vi : (vi + 1);
}

}  // namespace race
