// Issue order of the matrix-power wavefront on the GPU (host code).
//
// RACE runs its level groups as a diagonal wavefront over (group, power)
// (src/functionManager.cpp:618-823): power k of group g after power k-1 of
// groups g-1..g+1. On a GPU the unit of work is a 32-row chunk, and the
// engine records per chunk the exact chunk intervals it reads, so the
// wavefront can run at chunk granularity: an item can start as soon as the
// chunks it reads are complete at the previous power. The order below keeps
// a chunk's consecutive powers as close in time as its dependencies and the
// work in flight allow, which bounds the matrix data between two uses of a
// chunk to about (powers in flight) x (rows a chunk reaches ahead + lag).
#include "mpk_order.h"

#include <algorithm>
#include <stdexcept>

namespace race {

namespace {

struct Item {
    long long t;  // time / runLen
    int k, c;
};

// Merges intervals that overlap or touch, then closes the smallest gaps
// until at most kMpkRunDepIntervals remain. Closing a gap only adds chunks
// below the highest one read; their previous power precedes the run in the
// order (the times are monotone in the chunk index).
void mergeIntervals(std::vector<std::pair<int, int>> &iv) {
    std::sort(iv.begin(), iv.end());
    std::vector<std::pair<int, int>> m;
    for (const auto &p : iv) {
        if (!m.empty() && p.first <= m.back().second + 1)
            m.back().second = std::max(m.back().second, p.second);
        else
            m.push_back(p);
    }
    while ((int)m.size() > kMpkRunDepIntervals) {
        size_t best = 0;
        long long gap = -1;
        for (size_t i = 0; i + 1 < m.size(); ++i) {
            const long long g = (long long)m[i + 1].first - m[i].second;
            if (gap < 0 || g < gap) {
                gap = g;
                best = i;
            }
        }
        m[best].second = std::max(m[best].second, m[best + 1].second);
        m.erase(m.begin() + (long)best + 1);
    }
    iv.swap(m);
}

void appendRun(MpkOrder &o, const std::vector<int> &depRange, int c0, int c1, int k, bool last, int rank) {
    o.head.insert(o.head.end(), {c0, c1, k, last ? 1 : 0});
    o.rank.push_back(rank);
    std::vector<std::pair<int, int>> iv;
    if (k > 0)
        for (int c = c0; c < c1; ++c)
            for (int d = 0; d < 3; ++d) {
                const int lo = depRange[6 * (size_t)c + 2 * d], hi = depRange[6 * (size_t)c + 2 * d + 1];
                if (hi >= lo) iv.emplace_back(lo, hi);
            }
    mergeIntervals(iv);
    for (int i = 0; i < kMpkRunDepIntervals; ++i) {
        if (i < (int)iv.size())
            o.dep.insert(o.dep.end(), {iv[i].first, iv[i].second});
        else
            o.dep.insert(o.dep.end(), {0, -1});
    }
}

bool lastOfSegment(int k, int power, int segLen) { return k == power - 1 || (k + 1) % segLen == 0; }

}  // namespace

MpkOrder mpkRunOrder(const std::vector<int> &depRange, int numChunks, int power, int segLen, int runLen, int lag,
                     const std::vector<int> &chunkDie) {
    const int C = numChunks;
    if (C < 0 || power < 1 || lag < 0 || (size_t)C * 6 > depRange.size() ||
        (!chunkDie.empty() && (int)chunkDie.size() != C))
        throw std::invalid_argument("mpkRunOrder: sizes");
    auto dieOf = [&](int c) { return chunkDie.empty() ? 0 : (chunkDie[c] ? 1 : 0); };
    segLen = segLen < 1 || segLen > power ? power : segLen;
    runLen = std::clamp(runLen, 1, kMpkMaxRunLen);
    std::vector<int> maxdep(C, -1);
    for (int c = 0; c < C; ++c)
        for (int d = 0; d < 3; ++d) {
            const int lo = depRange[6 * (size_t)c + 2 * d], hi = depRange[6 * (size_t)c + 2 * d + 1];
            if (hi >= lo) maxdep[c] = std::max(maxdep[c], hi);
        }
    std::vector<Item> items;
    items.reserve((size_t)C * power);
    std::vector<long long> prev(C), cur(C);
    for (int c = 0; c < C; ++c) prev[c] = c;
    for (int k = 0; k < power; ++k) {
        if (k > 0) {
            long long run = 0;
            for (int c = 0; c < C; ++c) {
                long long t = maxdep[c] >= 0 ? prev[maxdep[c]] + 1 + lag : 0;
                if (k % segLen == 0) t = std::max(t, (long long)(k / segLen) * C + c);
                run = std::max(run, t);
                cur[c] = run;
            }
            prev.swap(cur);
        }
        for (int c = 0; c < C; ++c) items.push_back({prev[c] / runLen, k, c});
    }
    std::sort(items.begin(), items.end(), [](const Item &a, const Item &b) {
        if (a.t != b.t) return a.t < b.t;
        if (a.k != b.k) return a.k < b.k;
        return a.c < b.c;
    });
    // runs in the global order, one list per die
    MpkOrder per[2];
    int rank = 0;
    for (size_t i = 0; i < items.size();) {
        size_t j = i + 1;
        while (j < items.size() && (int)(j - i) < runLen && items[j].k == items[i].k && items[j].t == items[i].t &&
               items[j].c == items[j - 1].c + 1 && dieOf(items[j].c) == dieOf(items[i].c))
            ++j;
        appendRun(per[dieOf(items[i].c)], depRange, items[i].c, items[j - 1].c + 1, items[i].k,
                  lastOfSegment(items[i].k, power, segLen), rank++);
        i = j;
    }
    MpkOrder o;
    for (int d = 0; d < 2; ++d) {
        o.head.insert(o.head.end(), per[d].head.begin(), per[d].head.end());
        o.dep.insert(o.dep.end(), per[d].dep.begin(), per[d].dep.end());
        o.rank.insert(o.rank.end(), per[d].rank.begin(), per[d].rank.end());
    }
    o.dieStart = {0, per[0].numRuns(), per[0].numRuns() + per[1].numRuns()};
    return o;
}

MpkOrder mpkGroupOrder(const std::vector<int> &depRange, const std::vector<int> &chunkGroup, int numGroups,
                       int power, int stride, int split) {
    const int C = (int)chunkGroup.size(), G = numGroups;
    std::vector<int> groupFirst(G + 1, C);
    for (int t = C - 1; t >= 0; --t) groupFirst[chunkGroup[t]] = t;
    for (int g = G - 1; g >= 0; --g) groupFirst[g] = std::min(groupFirst[g], groupFirst[g + 1]);
    const int seg = split > 0 && split < power ? split : power;
    MpkOrder o;
    for (int k0 = 0; k0 < power; k0 += seg) {
        const int kn = std::min(power, k0 + seg) - k0;
        for (int st = 0; st < G + stride * (kn - 1); ++st)
            for (int k = 0; k < kn; ++k) {
                const int g = st - stride * k;
                if (g < 0 || g >= G) continue;
                for (int t = groupFirst[g]; t < groupFirst[g + 1]; ++t)
                    appendRun(o, depRange, t, t + 1, k0 + k, lastOfSegment(k0 + k, power, seg), o.numRuns());
            }
    }
    o.dieStart = {0, o.numRuns(), o.numRuns()};
    return o;
}

std::vector<int> chunkDies(int numChunks, int smsDie0, int smsDie1) {
    std::vector<int> die(std::max(numChunks, 0), 0);
    const long long total = (long long)smsDie0 + smsDie1;
    if (smsDie0 <= 0 || smsDie1 <= 0) return die;
    for (int c = 0; c < numChunks; ++c) {
        const long long b = c / kDieBlockChunks;
        // block b goes to die 0 when die 0's share of blocks 0..b grows by one
        die[c] = ((b + 1) * smsDie0 / total > b * smsDie0 / total) ? 0 : 1;
    }
    return die;
}

std::vector<int> mpkFlagBlocks(int numChunks, const std::vector<int> &chunkGroup) {
    if (!chunkGroup.empty() && (int)chunkGroup.size() != numChunks)
        throw std::invalid_argument("mpkFlagBlocks: sizes");
    std::vector<int> start;
    for (int c = 0; c < numChunks; ++c)
        if (c % kDieBlockChunks == 0 || (!chunkGroup.empty() && chunkGroup[c] != chunkGroup[c - 1]))
            start.push_back(c);
    start.push_back(std::max(numChunks, 0));
    return start;
}

std::vector<int> widenDepsToBlocks(const std::vector<int> &depRange, const std::vector<int> &blockStart) {
    std::vector<int> out(depRange);
    const int C = blockStart.empty() ? 0 : blockStart.back();
    for (size_t i = 0; i + 1 < out.size(); i += 2) {
        const int lo = out[i], hi = out[i + 1];
        if (hi < lo) continue;
        if (lo < 0 || hi >= C) throw std::invalid_argument("widenDepsToBlocks: interval outside the chunks");
        // block of a chunk: the last start <= it
        const size_t bl = std::upper_bound(blockStart.begin(), blockStart.end() - 1, lo) - blockStart.begin() - 1;
        const size_t bh = std::upper_bound(blockStart.begin(), blockStart.end() - 1, hi) - blockStart.begin() - 1;
        out[i] = blockStart[bl];
        out[i + 1] = blockStart[bh + 1] - 1;
    }
    return out;
}

}  // namespace race
