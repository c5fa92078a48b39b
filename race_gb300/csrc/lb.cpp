// Level load balancer, restating RACE's LB::splitZones (src/lb.cpp:188-667)
// and Stat (src/lb.cpp:742-796). The control flow and every floating-point
// operation follow the reference in the same order, because zone boundaries
// must come out identical; the file is compiled without floating-point
// contraction so x86 and Arm hosts agree with each other and the reference.
#include "lb.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <numeric>

namespace race {
namespace {

// Stat::calculate (lb.cpp:773-796): per partition (block colour) the mean of
// chunk/scale, the variance, and per-chunk deviations.
struct Stat {
    int numPartitions;
    std::vector<double> mean, var, acquireWeight, giveWeight, weight;
    Stat(const std::vector<int> &arr, int numPartitions_, const std::vector<int> &scale) : numPartitions(numPartitions_) {
        int len = (int)arr.size();
        mean.assign(numPartitions, 0.0);
        var.assign(numPartitions, 0.0);
        weight.assign(len, 0.0);
        acquireWeight.assign(len, 0.0);
        giveWeight.assign(len, 0.0);
        for (int p = 0; p < numPartitions; ++p) {
            int ctr = 0;
            for (int i = p; i < len; i += numPartitions) {
                mean[p] = mean[p] + arr[i] / ((double)scale[ctr]);
                ++ctr;
            }
            mean[p] = (numPartitions * mean[p]) / (len);
            ctr = 0;
            for (int i = p; i < len; i += numPartitions) {
                double diff = ((arr[i] / ((double)scale[ctr])) - mean[p]);
                var[p] = var[p] + diff * diff;
                acquireWeight[i] = diff;
                giveWeight[i] = -diff;
                weight[i] = std::fabs(diff);
                ++ctr;
            }
        }
    }
};

// Indices 0..n-1 stably ordered by descending key (sortPerm with rev=true,
// utility.h:50-58).
std::vector<int> rankDescending(const std::vector<double> &key) {
    std::vector<int> perm(key.size());
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] > key[b]; });
    return perm;
}

struct Splitter {
    const LevelData &ld;
    int nThreads;
    double efficiency;
    int dist, d2, lbTarget;
    int minGapV = 1, bpt = 1;
    int totalBlocks = 0, totalSubBlocks = 0, currLvlThreads = 0;
    std::vector<int> scale, levelPtr, subLevelPtr, numBlocks;

    const std::vector<int> &target(bool forceRow) const {
        return (lbTarget == LB_ROW || forceRow) ? ld.levelRow : ld.levelNnz;
    }

    // Per-block sums of the level counts: integer sums, taken from prefix
    // sums (the same values as adding the levels of each block one by one).
    std::vector<long long> prefixRow, prefixTarget;
    void prefixSums() {
        for (int f = 0; f < 2; ++f) {
            const std::vector<int> &t = target(f == 1);
            std::vector<long long> &p = f == 1 ? prefixRow : prefixTarget;
            p.assign(t.size() + 1, 0);
            for (size_t j = 0; j < t.size(); ++j) p[j + 1] = p[j] + t[j];
        }
    }
    void chunkSum(const std::vector<int> &lp, int len, bool forceRow, std::vector<int> &out) const {
        const std::vector<long long> &p = forceRow || lbTarget == LB_ROW ? prefixRow : prefixTarget;
        out.assign(len, 0);
        for (int i = 0; i < len; ++i) out[i] = (int)(p[lp[i + 1]] - p[lp[i]]);
    }

    // findNeighbour (lb.cpp:134-169): the first index of the weights in
    // stable descending order (for acquire: the first whose block is wider
    // than minGapV). That is the largest weight, the smallest index among
    // equal weights, so a linear scan gives it without sorting.
    int findNeighbour(const Stat &s, bool acquire) const {
        const std::vector<double> &w = acquire ? s.acquireWeight : s.giveWeight;
        int best = -1;
        const int m = acquire ? totalBlocks : (int)w.size();
        for (int idx = 0; idx < m; ++idx) {
            if (acquire && (levelPtr[idx + 1] - levelPtr[idx]) <= minGapV) continue;
            if (best < 0 || w[idx] > w[best]) best = idx;
        }
        return best;
    }

    // moveOneStep (lb.cpp:171-185); fromIdx may be -1 (the reference then
    // shifts the leading pointers; the move is discarded by the caller).
    void moveOneStep(int toIdx, int fromIdx) {
        if (toIdx < fromIdx) {
            for (int i = toIdx + 1; i <= fromIdx; ++i) levelPtr[i] += 1;
        } else {
            for (int i = toIdx; i >= fromIdx + 1; --i) levelPtr[i] -= 1;
        }
    }

    void run() {
        const int totalLevel = ld.totalLevel;
        prefixSums();
        // calcEffectiveRatio (lb.cpp:114-132). The product of a level count
        // and the thread count is formed in 32-bit int arithmetic, as in the
        // reference, before the division.
        std::vector<double> effRatio(totalLevel);
        {
            const std::vector<int> &t = target(false);
            int totalElems = (lbTarget == LB_ROW) ? (int)ld.nrow : (int)ld.nnz;
            for (int i = 0; i < totalLevel; ++i) {
                int prod = (int)(int32_t)((uint32_t)t[i] * (uint32_t)nThreads);
                effRatio[i] = prod / ((double)totalElems);
            }
        }
        minGapV = minGap(dist, d2);
        bpt = blockPerThread(dist, d2);
        const int minGapPerThread = minGapV * bpt;

        double accumulator = 0, currRem = 0, localRem = 0, newLocalRem = 0, minLocalRem = 0;
        int minGapCtr = 0, bestIdx = 0;
        std::vector<int> initialLvlPtr{0};

        // initial thread estimate per level range (lb.cpp:221-308)
        for (int i = 0; i < totalLevel; ++i) {
            accumulator += effRatio[i];
            ++minGapCtr;
            if (minGapCtr >= minGapPerThread && roundDouble(accumulator) != 0) {
                if (((1 - std::fabs(accumulator - roundDouble(accumulator))) * 100) > efficiency) {
                    localRem = (accumulator - roundDouble(accumulator));
                    newLocalRem = localRem;
                    minLocalRem = localRem;
                    int roundedVal = roundDouble(accumulator);
                    double tempAccumulator = accumulator;
                    double minTempAccumulator = accumulator;
                    int j = i + 1;
                    bestIdx = i;
                    while ((j < totalLevel) && (std::fabs(newLocalRem) <= std::fabs(localRem))) {
                        tempAccumulator += effRatio[j];
                        newLocalRem = (tempAccumulator - roundedVal);
                        if (std::fabs(minLocalRem) > std::fabs(newLocalRem)) {
                            minLocalRem = newLocalRem;
                            minTempAccumulator = tempAccumulator;
                            bestIdx = j;
                        } else if ((std::fabs(minLocalRem) - std::fabs(newLocalRem)) < 1e-6) {
                            double lhs = minLocalRem + currRem;
                            double rhs = newLocalRem + currRem;
                            if (lhs > rhs) {
                                minLocalRem = newLocalRem;
                                minTempAccumulator = tempAccumulator;
                                bestIdx = j;
                            }
                        }
                        ++j;
                    }
                    minGapCtr += (bestIdx - i);
                    i = bestIdx;
                    accumulator = minTempAccumulator;
                    currRem = currRem + (accumulator - roundDouble(accumulator));
                    scale.push_back(roundDouble(accumulator));
                    initialLvlPtr.push_back(i + 1);
                    accumulator = 0;
                    minGapCtr = 0;
                }
            }
            if (i >= (totalLevel - 5)) {
                double last = accumulator;
                for (int j = i + 1; j < totalLevel; ++j) last += effRatio[j];
                if (roundDouble(last) != 0) {
                    scale.push_back(roundDouble(last));
                    initialLvlPtr.push_back(totalLevel);
                } else {
                    initialLvlPtr.back() = totalLevel;
                }
                break;
            }
        }

        // rounding fix-up of the thread total (lb.cpp:310-365)
        int threadCtr = 0;
        for (auto &s : scale) {
            if (s == 0) s = 1;
            threadCtr += s;
        }
        if (!scale.empty()) {
            if (threadCtr != nThreads) {
                int diff = nThreads - threadCtr;
                if (std::abs(diff) == 1) {
                    if (diff == 1) {
                        scale.back() += 1;
                    } else if (scale.back() == 1) {
                        scale.pop_back();
                        initialLvlPtr.pop_back();
                        initialLvlPtr.back() = totalLevel;
                    } else {
                        scale.back() -= 1;
                    }
                }
            }
            currLvlThreads = (int)scale.size();
        }

        // two (or three) blocks per thread, split evenly in levels
        // (lb.cpp:367-376)
        totalBlocks = bpt * currLvlThreads;
        levelPtr.assign(totalBlocks + 1, 0);
        for (int i = 0; i < currLvlThreads; ++i)
            for (int j = 1; j <= bpt; ++j)
                levelPtr[i * bpt + j] =
                    initialLvlPtr[i] + roundDouble(j * (initialLvlPtr[i + 1] - initialLvlPtr[i]) / ((double)bpt));

        // variance-minimising level moves (lb.cpp:384-564)
        if (!scale.empty()) {
            std::vector<int> cs, ncs, oldLevelPtr;
            bool exitFlag = false;
            while (!exitFlag) {
                chunkSum(levelPtr, totalBlocks, false, cs);
                Stat meanVar(cs, bpt, scale);
                double var = 0;
                for (int p = 0; p < meanVar.numPartitions; ++p) var += meanVar.var[p];
                double newVar = var;
                std::vector<int> rankPerm = rankDescending(meanVar.weight);
                int currRank = 0;
                oldLevelPtr = levelPtr;
                while (newVar >= var) {
                    int rankIdx = rankPerm[currRank];
                    levelPtr = oldLevelPtr;
                    double myMean = meanVar.mean[rankIdx % bpt];
                    bool fail = false, movePossible = true, first = true;
                    while (first || (movePossible && std::fabs(var - newVar) < 1e-5)) {
                        first = false;
                        if ((cs[rankIdx] / (double)scale[rankIdx / bpt]) < myMean) {
                            int acquireIdx = findNeighbour(meanVar, true);
                            if (acquireIdx == -1 || acquireIdx == rankIdx) {
                                fail = true;
                                movePossible = false;
                            }
                            moveOneStep(rankIdx, acquireIdx);
                        } else {
                            if ((levelPtr[rankIdx + 1] - levelPtr[rankIdx]) > minGapV) {
                                int giveIdx = findNeighbour(meanVar, false);
                                if (giveIdx == -1 || rankIdx == giveIdx) {
                                    movePossible = false;
                                    fail = true;
                                }
                                moveOneStep(giveIdx, rankIdx);
                            } else {
                                movePossible = false;
                            }
                        }
                        if (!fail) {
                            chunkSum(levelPtr, totalBlocks, false, ncs);
                            Stat nv(ncs, bpt, scale);
                            newVar = 0;
                            for (int p = 0; p < nv.numPartitions; ++p) newVar += nv.var[p];
                        }
                    }
                    if ((currRank == (totalBlocks - 1)) && (newVar >= var)) {
                        exitFlag = true;
                        levelPtr = oldLevelPtr;
                        break;
                    }
                    currRank += 1;
                }
            }
        }

        // cache sub-blocking (lb.cpp:580-650); the reference fixes the cache
        // size to INT_MAX, so only zones above INT_MAX/340 rows split.
        std::vector<int> zp0;
        zonePtr(0, zp0);
        const int cacheSize = INT_MAX;
        const int nnzr = 27;
        int blockedSize = (int)(ld.nrow * 0) + cacheSize / (8 * 2 + nnzr * 12);
        int maxLvlNrow = 0;
        for (int l = 0; l < totalLevel; ++l) maxLvlNrow = std::max(maxLvlNrow, ld.levelRow[l]);
        blockedSize = std::max(blockedSize, maxLvlNrow);
        numBlocks.assign(totalBlocks, 0);
        subLevelPtr.clear();
        int ctr = 0;
        for (int i = 0; i < totalBlocks; ++i) {
            numBlocks[i] += 1;
            subLevelPtr.push_back(levelPtr[i]);
            ++ctr;
            int currThread = static_cast<int>(i / (double)(bpt));
            if ((zp0[i + 1] - zp0[i]) > blockedSize && scale[currThread] > 1 && (levelPtr[i + 1] - levelPtr[i]) > 1) {
                int currSize = ld.levelRow[levelPtr[i]];
                for (int j = levelPtr[i] + 1; j < levelPtr[i + 1]; ++j) {
                    currSize += ld.levelRow[j];
                    if (currSize > blockedSize) {
                        numBlocks[i] += 1;
                        subLevelPtr.push_back(j);
                        ++ctr;
                        currSize = ld.levelRow[j];
                    }
                }
            }
        }
        subLevelPtr.push_back(levelPtr[totalBlocks]);
        totalSubBlocks = ctr;
    }

    // calcZonePtr / calcSubZonePtr (lb.cpp:669-707): row offsets from level
    // row counts.
    void zonePtr(int base, std::vector<int> &out) const {
        std::vector<int> cs;
        chunkSum(levelPtr, totalBlocks, true, cs);
        out.assign(totalBlocks + 1, base);
        for (int i = 0; i < totalBlocks; ++i) out[i + 1] = out[i] + cs[i];
    }
    void subZonePtr(int base, std::vector<int> &out) const {
        std::vector<int> cs;
        chunkSum(subLevelPtr, totalSubBlocks, true, cs);
        out.assign(totalSubBlocks + 1, base);
        for (int i = 0; i < totalSubBlocks; ++i) out[i + 1] = out[i] + cs[i];
    }
};

}  // namespace

LBResult lbBalance(const LevelData &ld, int nThreads, double eff, int dist, int d2, int lbTarget, int base) {
    // LB ctor (lb.cpp:30-48): an absent nnz histogram falls back to rows.
    Splitter s{ld, nThreads, eff, dist, d2, (lbTarget == LB_NNZ && ld.levelNnz.empty()) ? LB_ROW : lbTarget};
    s.run();
    LBResult r;
    r.scale = s.scale;
    s.zonePtr(base, r.zonePtr);
    s.subZonePtr(base, r.subZonePtr);
    r.numBlocks = s.numBlocks;
    return r;
}

}  // namespace race
