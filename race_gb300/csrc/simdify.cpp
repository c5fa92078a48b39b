// SELL-C-sigma preparation for SIMD kernels (simdify.h). Restates the
// reference's padding rule (src/sell_c_sigmize.cpp:25-45) and its two
// in-row reordering passes (include/simdify.h:70-301 distance-2,
// include/simdify.h:389-447 distance-1) so that the rearranged columns and
// values are identical to the reference's for the same input.
#include "simdify.h"

#include <algorithm>
#include <cstring>

namespace race {
namespace {

// Slot addressing of one SELL matrix and the swap of two entries.
struct Slots {
    const SellArrays &m;
    long long at(int chunk, int group, int lane, int slot) const {
        return (long long)m.chunkStart[chunk] + (long long)slot * m.C + (long long)group * m.simdWidth + lane;
    }
    void swap(long long a, long long b) const {
        std::swap(m.col[a], m.col[b]);
        if (!m.val) return;
        const size_t es = (size_t)m.valBytes;
        unsigned char t[8];
        memcpy(t, m.val + a * es, es);
        memcpy(m.val + a * es, m.val + b * es, es);
        memcpy(m.val + b * es, t, es);
    }
};

int checkArgs(const SellArrays &m, std::string &msg) {
    if (m.simdWidth < 1 || m.C < 1 || m.nrows < 0 || !m.col || !m.chunkStart || !m.clp) {
        msg = "simdify: simdWidth and C must be positive, col, chunkStart and clp given";
        return SIMDIFY_BAD_ARG;
    }
    if (m.C % m.simdWidth) {
        msg = "simdify: the chunk length C must be a multiple of simdWidth";
        return SIMDIFY_BAD_ARG;
    }
    if (m.valBytes != 2 && m.valBytes != 4 && m.valBytes != 8) {
        msg = "simdify: values must be 2, 4 or 8 bytes wide";
        return SIMDIFY_BAD_ARG;
    }
    return SIMDIFY_OK;
}

int numChunks(const SellArrays &m) { return (m.nrows + m.C - 1) / m.C; }

}  // namespace

int simdifyD2(const SellArrays &m, const std::vector<int> &leafLo, const std::vector<int> &leafHi, bool diagFirst,
              int *collisions, std::string &msg) {
    if (int st = checkArgs(m, msg)) return st;
    if (!m.rl || leafLo.size() != leafHi.size()) {
        msg = "simdify: row lengths and a forward schedule are needed";
        return SIMDIFY_BAD_ARG;
    }
    // Padding: inside each leaf, the rows' unused slots point at the leaf's
    // first simdWidth rows, one per lane, so padding never collides across
    // the lanes of a group that starts at the leaf's start.
    for (size_t l = 0; l < leafLo.size(); ++l) {
        const int lo = leafLo[l], hi = leafHi[l];
        if (lo < 0 || hi > m.nrows || lo > hi) {
            msg = "simdify: the schedule has a leaf outside the rows";
            return SIMDIFY_BAD_ARG;
        }
        for (int r = lo; r < hi; ++r) {
            const int c = r / m.C;
            const long long home = (long long)m.chunkStart[c] + r % m.C;
            for (int j = m.rl[r]; j < m.clp[c]; ++j) m.col[home + (long long)j * m.C] = lo + (r - lo) % m.simdWidth;
        }
    }

    // Reordering, slot by slot and lane by lane inside each SIMD group: a
    // lane whose entry repeats a column already chosen by an earlier lane in
    // this slot takes the next entry of its own row that does not, searching
    // forward and then wrapping to the first movable slot. Once wrapped, the
    // candidate slot is settled for the other lanes, so the entry moved out
    // of this slot must not repeat any of their columns there either.
    const int W = m.simdWidth, groups = m.C / W, first = diagFirst ? 1 : 0;
    Slots s{m};
    std::vector<int> chosen(W);
    std::vector<char> moved(m.nrows, 0);
    for (int c = 0; c < numChunks(m); ++c) {
        const int len = m.clp[c];
        for (int g = 0; g < groups; ++g) {
            const int base = c * m.C + g * W;
            const int lanes = std::min(W, m.nrows - base);
            if (lanes <= 0) break;
            for (int j = first; j < len; ++j) {
                for (int i = 0; i < lanes; ++i) {
                    const long long home = s.at(c, g, i, j);
                    int cand = j, tries = 0;
                    bool wrapped = false;
                    for (;;) {
                        const int v = m.col[s.at(c, g, i, cand)];
                        bool clash = std::find(chosen.begin(), chosen.begin() + i, v) != chosen.begin() + i;
                        if (clash) moved[base + i] = 1;
                        for (int k = 0; wrapped && !clash && k < W; ++k)
                            clash = k != i && m.col[home] == m.col[s.at(c, g, k, cand)];
                        if (!clash) break;
                        if (tries >= len) {
                            msg = "simdify: row " + std::to_string(base + i) + " (length " +
                                  std::to_string(m.rl[base + i]) + ", chunk length " + std::to_string(len) +
                                  ") has no entry that keeps the " + std::to_string(W) +
                                  " lanes of its group on different columns";
                            if (collisions) *collisions = (int)std::count(moved.begin(), moved.end(), 1);
                            return SIMDIFY_UNPLACEABLE;
                        }
                        if (cand != len - 1) {
                            ++cand;
                        } else {
                            cand = first;
                            wrapped = true;
                        }
                        ++tries;
                    }
                    chosen[i] = m.col[s.at(c, g, i, cand)];
                    if (cand != j) s.swap(home, s.at(c, g, i, cand));
                }
            }
        }
    }
    if (collisions) *collisions = (int)std::count(moved.begin(), moved.end(), 1);
    return SIMDIFY_OK;
}

int simdifyD1(const SellArrays &m, bool dist2Compatible, std::string &msg) {
    if (int st = checkArgs(m, msg)) return st;
    const int W = m.simdWidth, groups = m.C / W;
    Slots s{m};
    std::vector<int> dep(W);
    // `next` is the first row the lane loop has not reached. It is tested
    // before lane 1 of each group, so a group whose first row is the last
    // row also treats its lane 1, a padding row inside the last chunk's
    // storage, as the reference's loop does (include/simdify.h:406).
    int next = 0;
    for (int c = 0; c < numChunks(m); ++c) {
        const int len = m.clp[c];
        for (int g = 0; g < groups; ++g) {
            const int base = c * m.C + g * W;
            for (int i = 1; i < W && next < m.nrows; ++i) {
                const int row = base + i;
                // the group's earlier rows, nearest first (or last)
                for (int k = 0; k < i; ++k) dep[dist2Compatible ? k : i - k - 1] = row - (k + 1);
                for (int j = 0; j < len; ++j) {
                    const long long p = s.at(c, g, i, j);
                    for (int k = 0; k < i; ++k) {
                        if (m.col[p] != dep[k]) continue;
                        // The reference takes slot len-(k+1) unchecked
                        // (include/simdify.h:426); below 0 it lies in the
                        // previous chunk and the swap would trade entries
                        // between two rows. Refused here instead.
                        const int ex = len - (k + 1);
                        if (ex < 0) {
                            msg = "simdifyD1: row " + std::to_string(row) + " has an entry on row " +
                                  std::to_string(dep[k]) + ", more slots back than chunk " + std::to_string(c) +
                                  " is long (" + std::to_string(len) + ")";
                            return SIMDIFY_BAD_ARG;
                        }
                        if (ex != j) s.swap(p, s.at(c, g, i, ex));
                    }
                }
                next = row + 1;
            }
        }
    }
    return SIMDIFY_OK;
}

}  // namespace race
