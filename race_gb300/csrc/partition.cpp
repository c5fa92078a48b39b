// Single-stage MPK partition (partition.h). Restates the reference's rules
// in the same order so that the level groups and hopeless groups are the
// reference's for the same levels.
#include "partition.h"

#include <algorithm>
#include <climits>
#include <cmath>

namespace race {
namespace {

// [start, end] (inclusive levels) of hopeless region `i` of a flat list of
// pairs, or (-1, -1) past its end (getHopelessStartEnd, matrixPower.cpp:669-683).
void region(const std::vector<int> &hr, int i, int &start, int &end) {
    start = end = -1;
    if (i >= 0 && 2 * i < (int)hr.size() - 1) {
        start = hr[2 * i];
        end = hr[2 * i + 1];
    }
}

// identifyHopelessRegions (matrixPower.cpp:147-503) for one shared-cache
// domain [0, totalLevel): runs of consecutive violated levels become
// regions; regions closer than power-1 levels merge; a region must keep
// power-1 levels to either end of the domain (it is trimmed, or dropped when
// nothing is left).
std::vector<int> hopelessRegions(std::vector<int> violated, int totalLevel, int power) {
    if (violated.size() > 1) violated.push_back(violated.back() + 2);  // closes the last run
    std::vector<int> flag(violated.size(), 0);
    int prev = -2, block = 1;
    for (size_t i = 0; i < violated.size(); ++i) {
        if (violated[i] == prev + 1) {
            flag[i - 1] = block;
            flag[i] = block;
        } else {
            ++block;
        }
        prev = violated[i];
    }
    std::vector<int> hr;
    int prevFlag = 0;
    for (size_t i = 0; i < flag.size(); ++i) {
        const int cur = flag[i];
        if (cur != prevFlag) {
            if (cur > 0 && prevFlag == 0) {
                hr.push_back(violated[i]);
            } else if (cur > 0 && prevFlag > 0) {
                hr.push_back(violated[i - 1]);
                hr.push_back(violated[i]);
            } else if (cur == 0) {
                hr.push_back(violated[i - 1]);
            }
        }
        prevFlag = cur;
    }

    // merge regions with fewer than power-1 levels between them
    std::vector<int> merged;
    const int nh = (int)(hr.size() / 2);
    int cs, ce, ns, ne;
    region(hr, 0, cs, ce);
    region(hr, 1, ns, ne);
    for (int i = 0; i < nh; ++i) {
        if (cs == -1) continue;
        while (((ns - ce) - 1) < (power - 1) && ns != -1) {
            ce = ne;
            region(hr, i + 2, ns, ne);
            ++i;
        }
        merged.push_back(cs);
        merged.push_back(ce);
        region(hr, i + 1, cs, ce);
        region(hr, i + 2, ns, ne);
    }

    // one domain [0, totalLevel): clip to it, then keep power-1 levels to
    // its start and end
    const int levelStart = 0, levelEnd = totalLevel;
    std::vector<int> clipped, drop;
    for (int i = 0; i < (int)(merged.size() / 2); ++i) {
        region(merged, i, cs, ce);
        if (cs >= levelStart) {
            if (cs < levelEnd) {
                clipped.push_back(cs);
                clipped.push_back(ce > levelEnd ? levelEnd - 1 : ce);
            }
        } else if (ce > levelEnd) {
            clipped.push_back(levelStart);
            clipped.push_back(levelEnd - 1);
        } else if (ce >= levelStart) {
            clipped.push_back(levelStart);
            clipped.push_back(ce);
        }
    }
    region(clipped, 0, cs, ce);
    if (cs != -1 && ((cs - levelStart) - 1) < (power - 1)) {
        const int newStart = levelStart + (power - 1);
        if (ce < newStart)
            drop.push_back(0);
        else
            clipped[0] = newStart;
    }
    const int last = (int)(clipped.size() / 2) - 1;
    region(clipped, last, cs, ce);
    if (ce != -1 && (((levelEnd - 1) - ce) - 1) < (power - 1)) {
        const int newEnd = levelEnd - (power - 1) - 1;
        if (cs > newEnd)
            drop.push_back(last);
        else
            clipped[2 * last + 1] = newEnd;
    }
    std::vector<int> out;
    for (int i = 0; i < (int)(clipped.size() / 2); ++i)
        if (std::find(drop.begin(), drop.end(), i) == drop.end()) {
            out.push_back(clipped[2 * i]);
            out.push_back(clipped[2 * i + 1]);
        }
    return out;
}

}  // namespace

StagePartition stagePartition(const LevelData &ld, int startRow, int power, int graphRows, long long graphNnz,
                              double cacheSize, double safety, int cutoff) {
    StagePartition sp;
    const int L = ld.totalLevel;
    std::vector<int> levelPtr(L + 1, startRow);
    for (int l = 0; l < L; ++l) levelPtr[l + 1] = levelPtr[l] + ld.levelRow[l];
    // getBytePerNNZ / getElemUpperLimit (matrixPower.cpp:88-99, 134-140)
    const double nnzr = graphNnz / (double)graphRows;
    const double bpn = (double)(((1 + power / nnzr) * sizeof(double) + (1 + 1 / nnzr) * sizeof(int)));
    const double cacheElem = cacheSize / bpn;
    auto elem = [&](int l) { return safety * (power + 1) * ld.levelNnz[l]; };

    std::vector<int> violated;
    for (int l = 0; l < L; ++l) {
        const double e = elem(l);
        if (e > cacheElem && static_cast<int>(std::ceil(e / cacheElem)) > cutoff) violated.push_back(l);
    }
    const std::vector<int> hr = hopelessRegions(violated, L, power);

    // consolidatePartition (matrixPower.cpp:685-940) for one domain
    if (L == 0) {
        sp.groupPtr = {startRow, startRow};
        sp.unlockRow = {startRow};
        sp.dangerRow = {startRow};
        return sp;
    }
    std::vector<int> unlock(L + 1, 0), danger(L + 1, 0);
    sp.groupPtr.push_back(levelPtr[0]);
    unlock[0] = levelPtr[std::min(1, L)];
    const int boundary = power - 1;
    int count = 0, hs, he;
    region(hr, count, hs, he);
    int group = 0, levelCtr = 0;
    double sumElem = 0;
    for (int level = 0; level < L; ++level) {
        const double cur = elem(level);
        sumElem += cur;
        bool hopeless = false, force = false;
        if (hs != -1) {
            if (level >= hs - boundary && level <= hs)
                force = true;  // levels before the region
            else if (level > he && level <= he + boundary)
                force = true;  // levels after it
            else if (level > hs && level <= he)
                hopeless = true;  // the region becomes one group
            if (level == he + boundary + 1) {
                region(hr, ++count, hs, he);
                force = true;
            }
            if (level == hs) sp.hopeless.push_back(group + 1);
        }
        if (levelCtr > 0 && !hopeless && (sumElem >= cacheElem || force)) {
            sumElem = cur;
            sp.groupPtr.push_back(levelPtr[level]);
            danger[group] = levelPtr[level - 1];
            if (level + 1 <= L) unlock[group + 1] = levelPtr[level + 1];
            ++group;
        }
        ++levelCtr;
    }
    sp.groupPtr.push_back(levelPtr[L]);
    danger[group] = levelPtr[L - 1];
    ++group;
    sp.unlockRow.assign(unlock.begin(), unlock.begin() + group);
    sp.dangerRow.assign(danger.begin(), danger.begin() + group);
    return sp;
}

bool recursePermutation(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                        std::vector<int> &totalInvPerm, const std::vector<int> &groupPtr,
                        const std::vector<int> &hopeless, int power) {
    const int G = (int)groupPtr.size() - 1;
    const int w = (power + 1) / 2 - 1;  // ceil(power/2) - 1 (workingBoundaryLength_base)
    std::vector<int> level(n, -1);
    std::vector<char> seen(n, 0), boundary(n, 0);
    std::vector<int> frontier, next, sorted;
    for (int h : hopeless) {
        if (h < 0 || h >= G) return false;
        const int lo = groupPtr[h], hi = groupPtr[h + 1];
        std::vector<std::pair<int, int>> regions{{lo, hi}};
        for (int r = -w; r <= w; ++r) {
            const int g = h + r;
            if (r == 0 || g < 0 || g >= G || groupPtr[g + 1] <= groupPtr[g]) continue;
            regions.emplace_back(groupPtr[g], groupPtr[g + 1]);
            for (int i = groupPtr[g]; i < groupPtr[g + 1]; ++i) boundary[i] = 1;
        }
        // BFS from lo (the rows are new indices; their neighbours are looked
        // up through the running permutation)
        int counted = 0, lvl = 0, restart = lo;
        frontier.clear();
        if (lo < hi) {
            frontier.push_back(lo);
            seen[lo] = 1;
            level[lo] = 0;
            counted = 1;
        }
        while (!frontier.empty()) {
            ++lvl;
            next.clear();
            for (int u : frontier) {
                const int pu = totalPerm[u];
                for (int idx = rowPtr[pu]; idx < rowPtr[pu + 1]; ++idx) {
                    if (col[idx] >= n) continue;
                    const int c = totalInvPerm[col[idx]];
                    if (seen[c]) continue;
                    const bool inside = c >= lo && c < hi;
                    if (!inside && !boundary[c]) continue;
                    seen[c] = 1;
                    level[c] = lvl;
                    next.push_back(c);
                    counted += inside;
                }
            }
            frontier.swap(next);
            if (frontier.empty() && counted != hi - lo) {
                while (restart < hi && seen[restart]) ++restart;
                if (restart == hi) return false;
                seen[restart] = 1;
                level[restart] = lvl;
                frontier.push_back(restart);
                ++counted;
            }
        }
        int levels = lvl;
        bool untouched = false;
        for (size_t k = 1; k < regions.size(); ++k)
            for (int i = regions[k].first; i < regions[k].second; ++i)
                if (!seen[i]) {
                    level[i] = lvl;
                    untouched = true;
                }
        levels += untouched ? 1 : 0;
        levels = std::max(levels, 1);
        // stable sort of each region by level, composed into the permutation
        for (const auto &rg : regions) {
            const int a = rg.first, b = rg.second;
            std::vector<int> start(levels + 1, 0);
            for (int i = a; i < b; ++i) ++start[level[i] + 1];
            for (int l = 0; l < levels; ++l) start[l + 1] += start[l];
            sorted.assign(b - a, 0);
            for (int i = a; i < b; ++i) sorted[start[level[i]]++] = totalPerm[i];
            for (int i = a; i < b; ++i) {
                totalPerm[i] = sorted[i - a];
                totalInvPerm[totalPerm[i]] = i;
            }
        }
        for (const auto &rg : regions)
            for (int i = rg.first; i < rg.second; ++i) {
                seen[i] = 0;
                boundary[i] = 0;
                level[i] = -1;
            }
    }
    return true;
}

}  // namespace race
