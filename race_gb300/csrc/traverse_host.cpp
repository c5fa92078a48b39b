// Host BFS of one row range (traverse_host.h). The rules are those of the
// engine's GPU traversal (kExpand, kIsland, kLevelHist and the stable level
// sort in traverse.cu), which restate the reference's Traverse.
#include "traverse_host.h"

#include <climits>

namespace race {

bool traverseRangeHost(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                       std::vector<int> &totalInvPerm, int lo, int hi, int mode, HostTraverseScratch &s,
                       LevelData &ld) {
    ld = LevelData();
    if (hi <= lo) return true;
    const int len = hi - lo;
    if ((int)s.stamp.size() < n) s.stamp.assign(n, 0);
    if (s.stampVal == INT_MAX) {
        s.stamp.assign(n, 0);
        s.stampVal = 0;
    }
    const int st = ++s.stampVal;
    s.dist.assign(len, -1);
    s.frontier.assign(1, lo);
    s.stamp[lo] = st;
    s.dist[0] = 0;
    if (mode == 2 && (int)s.mark.size() < n) s.mark.assign(n, 0);
    // non-zeros of the range's unvisited rows (the work of a pull step)
    long long unvisitedNnz = 0;
    if (mode == 2)
        for (int i = lo; i < hi; ++i) unvisitedNnz += rowPtr[totalPerm[i] + 1] - rowPtr[totalPerm[i]];
    unvisitedNnz -= rowPtr[totalPerm[lo] + 1] - rowPtr[totalPerm[lo]];
    long long counter = 1;
    int currLvl = 0, prevIslandStop = lo;
    while (!s.frontier.empty()) {
        ++currLvl;
        s.next.clear();
        // distance-2: push from the frontier's rows outside the range, or
        // let the unvisited rows of the range pull from them
        bool pull = false;
        if (mode == 2) {
            long long outNnz = 0;
            for (int u : s.frontier)
                if (u < lo || u >= hi) outNnz += rowPtr[totalPerm[u] + 1] - rowPtr[totalPerm[u]];
            pull = outNnz > unvisitedNnz;
        }
        const long long mk = ++s.markVal;
        for (int u : s.frontier) {
            const int pu = totalPerm[u];
            const bool uIn = u >= lo && u < hi;
            if (pull && !uIn) {
                s.mark[u] = mk;
                continue;
            }
            for (int j = rowPtr[pu]; j < rowPtr[pu + 1]; ++j) {
                const int c = col[j];
                if (c < 0 || c >= n) continue;  // columns beyond the matrix are remote
                const int c2 = totalInvPerm[c];
                if (s.stamp[c2] == st) continue;
                const bool inRange = c2 >= lo && c2 < hi;
                if (!inRange && !(mode == 2 && uIn)) continue;
                s.stamp[c2] = st;
                s.next.push_back(c2);
                if (inRange) {
                    s.dist[c2 - lo] = currLvl;
                    ++counter;
                    unvisitedNnz -= rowPtr[c + 1] - rowPtr[c];
                }
            }
        }
        if (pull) {
            for (int w = lo; w < hi; ++w) {
                if (s.stamp[w] == st) continue;
                const int pw = totalPerm[w];
                for (int j = rowPtr[pw]; j < rowPtr[pw + 1]; ++j) {
                    const int c = col[j];
                    if (c < 0 || c >= n) continue;
                    const int c2 = totalInvPerm[c];
                    if ((c2 < lo || c2 >= hi) && s.mark[c2] == mk) {
                        s.stamp[w] = st;
                        s.next.push_back(w);
                        s.dist[w - lo] = currLvl;
                        ++counter;
                        unvisitedNnz -= rowPtr[pw + 1] - rowPtr[pw];
                        break;
                    }
                }
            }
        }
        s.frontier.swap(s.next);
        if (s.frontier.empty() && counter != len) {
            // island restart: the lowest row without a level, one level on
            int isl = -1;
            for (int i = prevIslandStop; i < hi; ++i)
                if (s.dist[i - lo] == -1) {
                    isl = i;
                    break;
                }
            if (isl < 0) return false;
            ++currLvl;
            s.stamp[isl] = st;
            s.dist[isl - lo] = currLvl;
            if (mode == 2) unvisitedNnz -= rowPtr[totalPerm[isl] + 1] - rowPtr[totalPerm[isl]];
            s.frontier.assign(1, isl);
            ++counter;
            prevIslandStop = isl;
        }
    }
    const int L = currLvl;
    ld.totalLevel = L;
    ld.levelRow.assign(L, 0);
    ld.levelNnz.assign(L, 0);
    for (int i = lo; i < hi; ++i) {
        const int d = s.dist[i - lo];
        const int p = totalPerm[i];
        ++ld.levelRow[d];
        ld.levelNnz[d] += rowPtr[p + 1] - rowPtr[p];
    }
    // stable counting sort of the range by level, composed into the permutation
    std::vector<int> start(L + 1, 0), sorted(len);
    for (int l = 0; l < L; ++l) start[l + 1] = start[l] + ld.levelRow[l];
    for (int i = lo; i < hi; ++i) sorted[start[s.dist[i - lo]]++] = totalPerm[i];
    for (int i = 0; i < len; ++i) {
        totalPerm[lo + i] = sorted[i];
        totalInvPerm[sorted[i]] = lo + i;
    }
    for (int l = 0; l < L; ++l) {
        ld.nrow += ld.levelRow[l];
        ld.nnz += ld.levelNnz[l];
    }
    return true;
}

}  // namespace race
