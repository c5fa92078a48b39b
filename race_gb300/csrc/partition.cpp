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

// consolidatePartition (matrixPower.cpp:685-940) for one domain of L >= 1
// levels: levelPtr (L+1 row offsets) of the stage's rows, nnzInLevel the
// non-zeros of each level including those of the boundary regions
// (getElemUpperLimit, :88-99), bndPtr the level offsets (L+1) of each
// boundary region. bndGroupPtr gets each region's offsets at the
// consolidated group starts (newBoundaryLevelPtr). With checkBoundaries,
// false where a hopeless region lacks its boundary levels (the reference
// stops there); the trimming of the regions rules that out, so stage 0
// groups without the check, as before.
bool consolidate(const std::vector<int> &levelPtr, const std::vector<int> &nnzInLevel, int power, int graphRows,
                 long long graphNnz, double cacheSize, double safety, int cutoff,
                 const std::vector<std::vector<int>> &bndPtr, StagePartition &sp,
                 std::vector<std::vector<int>> &bndGroupPtr, bool checkBoundaries) {
    const int L = (int)nnzInLevel.size();
    // getBytePerNNZ / getElemUpperLimit (matrixPower.cpp:88-99, 134-140)
    const double nnzr = graphNnz / (double)graphRows;
    const double bpn = (double)(((1 + power / nnzr) * sizeof(double) + (1 + 1 / nnzr) * sizeof(int)));
    const double cacheElem = cacheSize / bpn;
    auto elem = [&](int l) { return safety * (power + 1) * nnzInLevel[l]; };

    std::vector<int> violated;
    for (int l = 0; l < L; ++l) {
        const double e = elem(l);
        if (e > cacheElem && static_cast<int>(std::ceil(e / cacheElem)) > cutoff) violated.push_back(l);
    }
    const std::vector<int> hr = hopelessRegions(violated, L, power);

    std::vector<int> unlock(L + 1, 0), danger(L + 1, 0);
    sp.groupPtr.assign(1, levelPtr[0]);
    sp.hopeless.clear();
    bndGroupPtr.assign(bndPtr.size(), {});
    for (size_t b = 0; b < bndPtr.size(); ++b) bndGroupPtr[b].push_back(bndPtr[b][0]);
    unlock[0] = levelPtr[std::min(1, L)];
    const int boundary = power - 1;
    int count = 0, hs, he;
    region(hr, count, hs, he);
    int group = 0, levelCtr = 0;
    double sumElem = 0;
    for (int level = 0; level < L; ++level) {
        if (checkBoundaries && hs >= 0 && (hs - boundary < 0 || he + boundary > L - 1)) return false;
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
            for (size_t b = 0; b < bndPtr.size(); ++b) bndGroupPtr[b].push_back(bndPtr[b][level]);
            danger[group] = levelPtr[level - 1];
            if (level + 1 <= L) unlock[group + 1] = levelPtr[level + 1];
            ++group;
        }
        ++levelCtr;
    }
    sp.groupPtr.push_back(levelPtr[L]);
    for (size_t b = 0; b < bndPtr.size(); ++b) bndGroupPtr[b].push_back(bndPtr[b][L]);
    danger[group] = levelPtr[L - 1];
    ++group;
    sp.unlockRow.assign(unlock.begin(), unlock.begin() + group);
    sp.dangerRow.assign(danger.begin(), danger.begin() + group);
    return true;
}

struct Range {
    int lo, hi;
};

// Per-row scratch of the leaf traversals, all -1 / 0 between leaves.
struct Scratch {
    std::vector<int> level;
    std::vector<char> seen, boundary;
    std::vector<int> frontier, next, sorted;
    explicit Scratch(int n) : level(n, -1), seen(n, 0), boundary(n, 0) {}
};

// One recursion stage's traversal (Traverse on a range with boundaries,
// traverse_GAP_graphSoA.cpp:31-90, 135-330, 452-575): a BFS of rows
// [lo, hi) from lo that also walks, without counting them, the rows of the
// boundary regions; islands of the range restart it on the same level;
// unvisited boundary rows get the level after the last (at least one level
// in all). The range and then every boundary region are sorted stably by
// level and the sort is composed into totalPerm/totalInvPerm (new index ->
// original row and back). Row lengths of the traversal graph give each
// level's non-zeros. Returns the number of levels, or -1 if rows of the
// range went missing. levelPtr/nnzInLevel: the range's level offsets and
// the non-zeros of range and boundary rows per level; bndPtr: each boundary
// region's level offsets.
int traverseLeaf(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                 std::vector<int> &totalInvPerm, int lo, int hi, const std::vector<Range> &bnd, Scratch &s,
                 std::vector<int> *levelPtr, std::vector<int> *nnzInLevel, std::vector<std::vector<int>> *bndPtr) {
    for (const Range &r : bnd)
        for (int i = r.lo; i < r.hi; ++i) s.boundary[i] = 1;
    int counted = 0, lvl = 0, restart = lo;
    s.frontier.clear();
    if (lo < hi) {
        s.frontier.push_back(lo);
        s.seen[lo] = 1;
        s.level[lo] = 0;
        counted = 1;
    }
    bool missing = false;
    while (!s.frontier.empty()) {
        ++lvl;
        s.next.clear();
        for (int u : s.frontier) {
            const int pu = totalPerm[u];
            for (int idx = rowPtr[pu]; idx < rowPtr[pu + 1]; ++idx) {
                if (col[idx] >= n) continue;
                const int c = totalInvPerm[col[idx]];
                if (s.seen[c]) continue;
                const bool inside = c >= lo && c < hi;
                if (!inside && !s.boundary[c]) continue;
                s.seen[c] = 1;
                s.level[c] = lvl;
                s.next.push_back(c);
                counted += inside;
            }
        }
        s.frontier.swap(s.next);
        if (s.frontier.empty() && counted != hi - lo) {
            while (restart < hi && s.seen[restart]) ++restart;
            if (restart == hi) {
                missing = true;
                break;
            }
            s.seen[restart] = 1;
            s.level[restart] = lvl;
            s.frontier.push_back(restart);
            ++counted;
        }
    }
    int levels = lvl;
    bool untouched = false;
    for (const Range &r : bnd)
        for (int i = r.lo; i < r.hi; ++i)
            if (!s.seen[i]) {
                s.level[i] = lvl;
                untouched = true;
            }
    levels += untouched ? 1 : 0;
    levels = std::max(levels, 1);

    std::vector<Range> regions{{lo, hi}};
    regions.insert(regions.end(), bnd.begin(), bnd.end());
    if (!missing) {
        if (levelPtr) {
            levelPtr->assign(levels + 1, lo);
            nnzInLevel->assign(levels, 0);
            bndPtr->assign(bnd.size(), {});
            for (size_t k = 0; k < regions.size(); ++k) {
                std::vector<int> rows(levels + 1, 0);
                for (int i = regions[k].lo; i < regions[k].hi; ++i) {
                    ++rows[s.level[i] + 1];
                    const int pi = totalPerm[i];
                    (*nnzInLevel)[s.level[i]] += rowPtr[pi + 1] - rowPtr[pi];
                }
                rows[0] = regions[k].lo;
                for (int l = 0; l < levels; ++l) rows[l + 1] += rows[l];
                if (k == 0)
                    *levelPtr = rows;
                else
                    (*bndPtr)[k - 1] = rows;
            }
        }
        // stable sort of each region by level, composed into the permutation
        for (const Range &rg : regions) {
            const int a = rg.lo, b = rg.hi;
            std::vector<int> start(levels + 1, 0);
            for (int i = a; i < b; ++i) ++start[s.level[i] + 1];
            for (int l = 0; l < levels; ++l) start[l + 1] += start[l];
            s.sorted.assign(b - a, 0);
            for (int i = a; i < b; ++i) s.sorted[start[s.level[i]]++] = totalPerm[i];
            for (int i = a; i < b; ++i) {
                totalPerm[i] = s.sorted[i - a];
                totalInvPerm[totalPerm[i]] = i;
            }
        }
    }
    for (const Range &rg : regions)
        for (int i = rg.lo; i < rg.hi; ++i) {
            s.seen[i] = 0;
            s.boundary[i] = 0;
            s.level[i] = -1;
        }
    return missing ? -1 : levels;
}

// The direct boundaries of hopeless group h of a leaf with groups groupPtr
// (its own groups h-w..h+w but h) and, with w >= 1, the sub-ranges
// h-w..h+w of every boundary region of the leaf by its consolidated group
// offsets, h-1..h+1 as one range (matrixPowerRecursive.cpp:199-287). Empty
// ranges are left out; false if a group index falls outside the leaf.
bool childBoundaries(const std::vector<int> &groupPtr, const std::vector<std::vector<int>> &bndGroupPtr, int h,
                     int w, std::vector<Range> &out) {
    const int G = (int)groupPtr.size() - 1;
    out.clear();
    if (h - w < 0 || h + w + 1 > G) return false;
    if (w > 0)
        for (const std::vector<int> &bp : bndGroupPtr)
            for (int r = -w; r <= w; ++r) {
                Range rg;
                if (r == -1) {
                    rg = {bp[h - 1], bp[h + 2]};
                    r = 1;
                } else {
                    rg = {bp[h + r], bp[h + r + 1]};
                }
                if (rg.hi > rg.lo) out.push_back(rg);
            }
    for (int r = -w; r <= w; ++r)
        if (r != 0 && groupPtr[h + r + 1] > groupPtr[h + r]) out.push_back({groupPtr[h + r], groupPtr[h + r + 1]});
    return true;
}

struct RecursionContext {
    int n;
    const int *rowPtr, *col;
    std::vector<int> &totalPerm, &totalInvPerm;
    int power;
    long long graphNnz;
    double cacheSize, safety;
    const std::vector<int> &stageCutoff;
    std::vector<MpkLeaf> &tree;
    Scratch scratch;
};

// recursivePartition (matrixPowerRecursive.cpp:156-298) below leaf `parent`
// whose boundary regions have consolidated offsets bndGroupPtr.
bool recurse(RecursionContext &ctx, int parent, const std::vector<std::vector<int>> &bndGroupPtr) {
    const int w = (ctx.power + 1) / 2 - 1;  // ceil(power/2) - 1 (workingBoundaryLength_base)
    const std::vector<int> hid = ctx.tree[parent].hopeless;
    const std::vector<int> gp = ctx.tree[parent].groupPtr;
    const int stage = ctx.tree[parent].stage + 1;
    const int cutoff = stage < (int)ctx.stageCutoff.size() ? ctx.stageCutoff[stage] : INT_MAX;
    std::vector<Range> bnd;
    for (int h : hid) {
        if (h < 0 || h >= (int)gp.size() - 1 || !childBoundaries(gp, bndGroupPtr, h, w, bnd)) return false;
        MpkLeaf leaf;
        leaf.lo = gp[h];
        leaf.hi = gp[h + 1];
        leaf.stage = stage;
        leaf.parent = parent;
        std::vector<int> levelPtr, nnzInLevel;
        std::vector<std::vector<int>> bndPtr, childBnd;
        if (traverseLeaf(ctx.n, ctx.rowPtr, ctx.col, ctx.totalPerm, ctx.totalInvPerm, leaf.lo, leaf.hi, bnd,
                         ctx.scratch, &levelPtr, &nnzInLevel, &bndPtr) < 0)
            return false;
        StagePartition sp;
        if (!consolidate(levelPtr, nnzInLevel, ctx.power, ctx.n, ctx.graphNnz, ctx.cacheSize, ctx.safety, cutoff,
                         bndPtr, sp, childBnd, true))
            return false;
        leaf.groupPtr = sp.groupPtr;
        leaf.hopeless = sp.hopeless;
        ctx.tree.push_back(leaf);
        const int idx = (int)ctx.tree.size() - 1;
        if (!sp.hopeless.empty() && !recurse(ctx, idx, childBnd)) return false;
    }
    return true;
}

}  // namespace

StagePartition stagePartition(const LevelData &ld, int startRow, int power, int graphRows, long long graphNnz,
                              double cacheSize, double safety, int cutoff) {
    StagePartition sp;
    const int L = ld.totalLevel;
    if (L == 0) {
        sp.groupPtr = {startRow, startRow};
        sp.unlockRow = {startRow};
        sp.dangerRow = {startRow};
        return sp;
    }
    std::vector<int> levelPtr(L + 1, startRow);
    for (int l = 0; l < L; ++l) levelPtr[l + 1] = levelPtr[l] + ld.levelRow[l];
    std::vector<int> nnzInLevel(ld.levelNnz.begin(), ld.levelNnz.begin() + L);
    std::vector<std::vector<int>> none;
    consolidate(levelPtr, nnzInLevel, power, graphRows, graphNnz, cacheSize, safety, cutoff, {}, sp, none, false);
    return sp;
}

bool recursePermutation(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                        std::vector<int> &totalInvPerm, const std::vector<int> &groupPtr,
                        const std::vector<int> &hopeless, int power) {
    const int G = (int)groupPtr.size() - 1;
    const int w = (power + 1) / 2 - 1;  // ceil(power/2) - 1 (workingBoundaryLength_base)
    Scratch s(n);
    std::vector<Range> bnd;
    for (int h : hopeless) {
        if (h < 0 || h >= G) return false;
        bnd.clear();
        for (int r = -w; r <= w; ++r) {
            const int g = h + r;
            if (r == 0 || g < 0 || g >= G || groupPtr[g + 1] <= groupPtr[g]) continue;
            bnd.push_back({groupPtr[g], groupPtr[g + 1]});
        }
        if (traverseLeaf(n, rowPtr, col, totalPerm, totalInvPerm, groupPtr[h], groupPtr[h + 1], bnd, s, nullptr,
                         nullptr, nullptr) < 0)
            return false;
    }
    return true;
}

bool recursivePartition(int n, const int *rowPtr, const int *col, std::vector<int> &totalPerm,
                        std::vector<int> &totalInvPerm, const StagePartition &root, int power, long long graphNnz,
                        double cacheSize, double safety, const std::vector<int> &stageCutoff,
                        std::vector<MpkLeaf> &tree) {
    tree.clear();
    MpkLeaf r;
    r.lo = 0;
    r.hi = n;
    r.groupPtr = root.groupPtr;
    r.hopeless = root.hopeless;
    tree.push_back(r);
    RecursionContext ctx{n, rowPtr, col, totalPerm, totalInvPerm, power, graphNnz, cacheSize, safety, stageCutoff,
                         tree, Scratch(n)};
    return recurse(ctx, 0, {});
}

}  // namespace race
