// Zone tree and level recursion. Restates RACE's ZoneTree::spawnChild /
// findKeyChild / updateTreeEffRow / updateTreeNThreads (src/zone_tree.cpp)
// and LevelRecursion (src/level_recursion.cpp) so that the tree matches the
// reference node for node; traversals of row ranges are delegated to the
// GPU through TraverseFn.
#include "coloring.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>

namespace race {

namespace {
// getEnv (utility.h:94-111): comma-separated tokens parsed with atoi, for
// integer and floating-point knobs alike.
template <typename T>
void readEnvList(const char *name, std::vector<T> &out) {
    const char *v = getenv(name);
    if (!v) return;
    std::string s(v);
    size_t pos = 0;
    while (pos <= s.size()) {
        size_t c = s.find(',', pos);
        std::string tok = s.substr(pos, c == std::string::npos ? std::string::npos : c - pos);
        if (!tok.empty()) out.push_back((T)atoi(tok.c_str()));
        if (c == std::string::npos) break;
        pos = c + 1;
    }
}
}  // namespace

Params Params::fromEnv() {
    Params p;
    readEnvList("RACE_THREADS", p.lvlThreads);
    readEnvList("RACE_EFFICIENCY", p.effVec);
    // level_recursion.cpp:86-90: a thread request for a stage drops its
    // efficiency threshold to 0 (entries beyond the list are not stored).
    for (unsigned lvl = 1; lvl < p.lvlThreads.size() + 1 && lvl < p.effVec.size(); ++lvl) p.effVec[lvl] = 0;
    std::vector<int> cd;
    readEnvList("RACE_CACHE_VIOLATION_CUTOFF_DEFAULT", cd);
    p.cacheViolationCutoffDefault = cd.empty() ? 50 : cd[0];
    p.cacheViolationCutoff.assign(1, p.cacheViolationCutoffDefault);
    readEnvList("RACE_CACHE_VIOLATION_CUTOFF", p.cacheViolationCutoff);
    std::vector<int> ms;
    readEnvList("RACE_MAX_RECURSION_STAGES", ms);
    p.maxRecStages = ms.empty() ? -1 : ms[0];
    return p;
}

// findKeyChild (zone_tree.cpp:91-155): the effective rows of the parent are
// the sum over blocks of the largest child per block, summed over sub-blocks.
int ZoneTree::findKeyChildEffRow(int parentIdx) const {
    const std::vector<int> &ch = nodes[parentIdx].children;
    int totalSubBlock = (int)ch.size() / 2;
    int b = bpt();
    std::vector<int> maxRow(b, 0);
    for (int sb = 0; sb < totalSubBlock; ++sb) {
        std::vector<int> tmp(b, 0);
        for (int blk = 0; blk < b; ++blk)
            for (int i = ch[2 * sb] + blk; i < ch[2 * sb + 1]; i += b)
                if (nodes[i].effRowZ > tmp[blk]) tmp[blk] = nodes[i].effRowZ;
        for (int blk = 0; blk < b; ++blk) maxRow[blk] += tmp[blk];
    }
    int s = 0;
    for (int blk = 0; blk < b; ++blk) s += maxRow[blk];
    return s;
}

void ZoneTree::updateTreeEffRow(int parentIdx) {
    nodes[parentIdx].effRowZ = findKeyChildEffRow(parentIdx);
    int nxt = nodes[parentIdx].parentZ;
    if (nxt != -1) updateTreeEffRow(nxt);
}

// updateTreeNThreads (zone_tree.cpp:176-206)
void ZoneTree::updateTreeNThreads(int parentIdx) {
    const std::vector<int> &ch = nodes[parentIdx].children;
    int totalSubBlocks = (int)ch.size() / 2;
    int b = bpt();
    int nThreads = 0;
    for (int sb = 0; sb < totalSubBlocks; ++sb) {
        int sub = 0;
        int numThreads = (ch[2 * sb + 1] - ch[2 * sb]) / b;
        for (int i = 0; i < numThreads; ++i) {
            int m = 0;
            for (int blk = 0; blk < b; ++blk) m = std::max(nodes[ch[2 * sb] + b * i + blk].nthreadsZ, m);
            sub += m;
        }
        nThreads = std::max(nThreads, sub);
    }
    nodes[parentIdx].nthreadsZ = nThreads;
    int nxt = nodes[parentIdx].parentZ;
    if (nxt != -1) updateTreeNThreads(nxt);
}

bool ZoneTree::spawnChild(int parentIdx, int parentSubIdx, int requestNthreads, const LevelData &ld, double eff) {
    int base = nodes[parentIdx].valueZ[parentSubIdx];
    LBResult lb = lbBalance(ld, requestNthreads, eff, dist_, d2_, lbTarget_, base);
    int baseLen = (int)nodes.size();
    int parentStage = nodes[parentIdx].stage;
    int totalBlocks = (int)lb.numBlocks.size();
    nodes[parentIdx].children.push_back(baseLen);
    int ctr = 0;
    for (int blk = 0; blk < totalBlocks; ++blk) {
        ZoneNode leaf(lb.zonePtr[blk], lb.zonePtr[blk + 1], parentIdx);
        leaf.valueZ.resize(lb.numBlocks[blk] + 1);
        for (int sb = 0; sb < lb.numBlocks[blk]; ++sb) leaf.valueZ[sb] = lb.subZonePtr[ctr++];
        leaf.valueZ[lb.numBlocks[blk]] = lb.subZonePtr[ctr];
        leaf.totalSubBlocks = lb.numBlocks[blk];
        leaf.stage = parentStage + 1;
        nodes.push_back(leaf);
    }
    nodes[parentIdx].children.push_back(baseLen + totalBlocks);
    if (parentSubIdx == nodes[parentIdx].totalSubBlocks - 1) {
        updateTreeEffRow(parentIdx);
        updateTreeNThreads(parentIdx);
    }
    return (int)lb.scale.size() == requestNthreads;
}

LevelRecursion::LevelRecursion(int nrow, int requested, int dist, int d2, int lbTarget, const Params &params,
                               TraverseFn trav, RangeNnzFn rangeNnz)
    : tree(dist, d2, lbTarget), nrow_(nrow), requested_(requested), dist_(dist), d2_(d2), lbTarget_(lbTarget),
      params_(params), trav_(std::move(trav)), rangeNnz_(std::move(rangeNnz)) {}

// calculateIdealNthreads (level_recursion.cpp:149-263): share the parent's
// thread budget among the children threads in proportion to their rows or
// non-zeros, flooring, then hand the leftover threads to the largest
// remainders.
void LevelRecursion::calculateIdealNthreads(int parentIdx, int parentSubIdx, int currLvl) {
    std::vector<ZoneNode> &N = tree.nodes;
    std::vector<int> ch = N[parentIdx].children;
    int b = tree.bpt();
    int nThreads = (ch[2 * parentSubIdx + 1] - ch[2 * parentSubIdx]) / b;
    if (params_.threadsAt(currLvl) == -1) {
        int parentThreads = N[parentIdx].idealNthreadsZ;
        int startRow = N[parentIdx].valueZ[parentSubIdx];
        int endRow = N[parentIdx].valueZ[parentSubIdx + 1];
        int parentRow = endRow - startRow;
        int parentNnz = 0;
        if (lbTarget_ == LB_NNZ) parentNnz = (int)rangeNnz_(startRow, endRow);
        std::vector<double> remainder(nThreads);
        int remaining = parentThreads;
        for (int i = 0; i < nThreads; ++i) {
            const std::vector<int> &first = N[ch[2 * parentSubIdx] + i * b].valueZ;
            const std::vector<int> &last = N[ch[2 * parentSubIdx] + b * (i + 1) - 1].valueZ;
            int s = first.front(), e = last.back();
            double myWeight = (e - s) / (static_cast<double>(parentRow));
            if (lbTarget_ == LB_NNZ) {
                int totalNnz = (int)rangeNnz_(s, e);
                myWeight = totalNnz / (static_cast<double>(parentNnz));
            }
            double myThreadsD = myWeight * parentThreads;
            int myThreads = static_cast<int>(myThreadsD);
            for (int blk = 0; blk < b; ++blk) N[ch[2 * parentSubIdx] + b * i + blk].idealNthreadsZ = myThreads;
            remainder[i] = (myThreads != 0) ? (myThreadsD - myThreads) : 1;
            remaining -= myThreads;
        }
        if (remaining > 0) {
            std::vector<int> rank(nThreads);
            std::iota(rank.begin(), rank.end(), 0);
            std::stable_sort(rank.begin(), rank.end(), [&](int a, int c) { return remainder[a] > remainder[c]; });
            int r = 0;
            while (remaining != 0 && r < nThreads) {
                int t = rank[r];
                for (int blk = 0; blk < b; ++blk) N[ch[2 * parentSubIdx] + b * t + blk].idealNthreadsZ += 1;
                remaining -= 1;
                r++;
            }
        }
    } else {
        int my = params_.threadsAt(currLvl);
        for (int i = 0; i < nThreads; ++i)
            for (int blk = 0; blk < b; ++blk) N[ch[2 * parentSubIdx] + b * i + blk].idealNthreadsZ = my;
    }
}

// recursivePartition (level_recursion.cpp:265-319)
void LevelRecursion::recursivePartition(int parentIdx, int parentSubIdx, int currLevel) {
    calculateIdealNthreads(parentIdx, parentSubIdx, currLevel);
    std::vector<int> ch = tree.nodes[parentIdx].children;
    for (int cur = ch[2 * parentSubIdx]; cur < ch[2 * parentSubIdx + 1]; ++cur) {
        int n = tree.nodes[cur].idealNthreadsZ;
        std::vector<int> range = tree.nodes[cur].valueZ;
        if (n > 1) {
            for (unsigned j = 0; j + 1 < range.size(); ++j) {
                if (range[j + 1] > range[j]) {
                    LevelData ld = trav_(range[j], range[j + 1]);
                    bool ok = tree.spawnChild(cur, (int)j, n, ld, params_.efficiency(currLevel));
                    if (!ok) {
                        int b = tree.bpt();
                        const std::vector<int> &cc = tree.nodes[cur].children;
                        int sub = (cc[2 * j + 1] - cc[2 * j]) / b;
                        if (sub == 1) tree.nodes[cur].reachedLimit = true;
                        if (sub > 1) recursivePartition(cur, (int)j, currLevel + 1);
                    }
                } else {
                    tree.nodes[cur].reachedLimit = true;
                }
            }
        }
    }
}

// levelBalancing (level_recursion.cpp:321-376)
void LevelRecursion::levelBalancing() {
    ZoneNode root(0, nrow_, -1);
    root.idealNthreadsZ = requested_;
    root.totalSubBlocks = 1;
    tree.nodes.push_back(root);
    LevelData ld = trav_(0, nrow_);
    int lvlOne = requested_;
    if (params_.threadsAt(1) != -1) lvlOne = params_.threadsAt(1);
    tree.spawnChild(0, 0, lvlOne, ld, params_.efficiency(1));
    if (tree.nodes[0].nthreadsZ != requested_) recursivePartition(0, 0, 2);
    availableThreads = tree.nodes[0].nthreadsZ;
    int m = 0;
    for (auto &z : tree.nodes) m = std::max(m, z.stage);
    tree.maxStage = m;
}

namespace {
struct Leaf {
    int lo, hi;
};
using Steps = std::vector<std::vector<Leaf>>;

Steps flattenNode(const ZoneTree &t, int node, bool rev) {
    const ZoneNode &z = t.nodes[node];
    const int b = t.bpt();
    Steps out;
    for (int sb = 0; sb < z.totalSubBlocks; ++sb) {
        int nthr = z.children.empty() ? 0 : (z.children[2 * sb + 1] - z.children[2 * sb]) / b;
        if (nthr <= 1) {
            // recursiveCall runs the node's first range as a leaf
            // (functionManager.cpp:218-230)
            Leaf l = rev ? Leaf{z.valueZ[1] - 1, z.valueZ[0] - 1} : Leaf{z.valueZ[0], z.valueZ[1]};
            out.push_back({l});
            continue;
        }
        int b0 = rev ? b - 1 : 0, b1 = rev ? -1 : b, inc = rev ? -1 : 1;
        for (int blk = b0; blk != b1; blk += inc) {
            Steps merged;
            for (int tid = 0; tid < nthr; ++tid) {
                Steps s = flattenNode(t, z.children[2 * sb] + b * tid + blk, rev);
                if (s.size() > merged.size()) merged.resize(s.size());
                for (size_t i = 0; i < s.size(); ++i) merged[i].insert(merged[i].end(), s[i].begin(), s[i].end());
            }
            out.insert(out.end(), merged.begin(), merged.end());
        }
    }
    return out;
}
}  // namespace

PhaseTable flattenZoneTree(const ZoneTree &t, bool rev, int serialLo, int serialHi) {
    Steps s = flattenNode(t, 0, rev);
    if (serialHi > serialLo) s.push_back({rev ? Leaf{serialHi, serialLo} : Leaf{serialLo, serialHi}});
    PhaseTable pt;
    pt.phasePtr.push_back(0);
    for (auto &step : s) {
        for (auto &l : step) {
            if (l.lo == l.hi) continue;  // empty range: the callback does nothing
            pt.leafLo.push_back(l.lo);
            pt.leafHi.push_back(l.hi);
        }
        if ((int)pt.leafLo.size() > pt.phasePtr.back()) pt.phasePtr.push_back((int)pt.leafLo.size());
    }
    return pt;
}

std::vector<int> serializeZoneTree(const ZoneTree &t) {
    std::vector<int> buf;
    buf.push_back((int)t.nodes.size());
    for (const ZoneNode &z : t.nodes) {
        buf.push_back(z.nthreadsZ);
        buf.push_back(z.idealNthreadsZ);
        buf.push_back(z.totalSubBlocks);
        buf.push_back(z.parentZ);
        buf.push_back(z.effRowZ);
        buf.push_back(z.stage);
        buf.push_back(z.reachedLimit ? 1 : 0);
        buf.push_back((int)z.valueZ.size());
        buf.insert(buf.end(), z.valueZ.begin(), z.valueZ.end());
        buf.push_back((int)z.children.size());
        buf.insert(buf.end(), z.children.begin(), z.children.end());
    }
    return buf;
}

}  // namespace race
