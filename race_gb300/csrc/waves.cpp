// Wave plans: RACE's execution order compiled into conflict-free waves.
//
// RACE runs a kernel leaf by leaf, each leaf a row range processed in order
// (src/functionManager.cpp:201-265); only the order of rows that touch the
// same vector entries matters. A wave plan assigns every row the smallest
// wave such that each row comes after every earlier row (in RACE's order)
// whose writes it reads, whose reads it overwrites, or whose writes it
// overwrites. Rows of one wave touch disjoint entries and can run in any
// order or all at once; running the waves in sequence performs, on every
// vector entry, the same operations in the same order as RACE's sequential
// walk, so the results are identical bit for bit. The depth is the length of
// the longest dependency chain, usually far below the longest leaf (a 200k-row
// power-law graph with distance-2 coloring: 376 waves for leaves of up to
// 57,753 rows).
#include "waves.h"

#include <algorithm>

namespace race {

namespace {
// Entries read and written by one row of each kernel (vector entries are
// indexed by row; x and b are separate vectors). Kernel bodies:
// examples/src/helpers/kernels.cpp (SpMV :5-15, SpMTV :107-115, GS :174-186,
// KACZ :285-302, SymmSpMV :403-417).
struct Access {
    // entries of b written (accumulated) and of x written / read
    template <typename F>
    static void forEach(int kernel, int r, const int *rowPtr, const int *col, F &&f) {
        // f(vec, entry, isWrite) with vec 0 = x, 1 = b
        const int s = rowPtr[r], e = rowPtr[r + 1];
        switch (kernel) {
        case RACE_K_SPMV:
            f(1, r, true);
            break;
        case RACE_K_SPMTV:
            for (int j = s; j < e; ++j) f(1, col[j], true);
            break;
        case RACE_K_SYMMSPMV:
            f(1, r, true);
            for (int j = s + 1; j < e; ++j) f(1, col[j], true);
            break;
        case RACE_K_GS:
            for (int j = s + 1; j < e; ++j) f(0, col[j], false);
            f(0, r, true);
            break;
        case RACE_K_KACZ:
            for (int j = s; j < e; ++j) f(0, col[j], true);
            break;
        default: break;
        }
    }
};
}  // namespace

WavePlan buildWavePlan(int kernel, int n, const int *rowPtr, const int *col, const PhaseTable &pt) {
    WavePlan wp;
    // rows in RACE's execution order
    std::vector<int> order;
    order.reserve(n);
    for (size_t l = 0; l < pt.leafLo.size(); ++l) {
        const int lo = pt.leafLo[l], hi = pt.leafHi[l];
        if (lo <= hi)
            for (int r = lo; r < hi; ++r) order.push_back(r);
        else
            for (int r = lo; r > hi; --r) order.push_back(r);
    }
    // per entry: wave of the last write and of the latest read, x and b
    std::vector<int> lastW[2], lastR[2];
    for (int v = 0; v < 2; ++v) {
        lastW[v].assign(n, 0);
        lastR[v].assign(n, 0);
    }
    std::vector<int> wave(order.size());
    int depth = 0;
    for (size_t i = 0; i < order.size(); ++i) {
        const int r = order[i];
        int w = 0;
        Access::forEach(kernel, r, rowPtr, col, [&](int v, int c, bool isWrite) {
            if (c < 0 || c >= n) return;
            w = std::max(w, lastW[v][c]);            // read-after-write, write-after-write
            if (isWrite) w = std::max(w, lastR[v][c]);  // write-after-read
        });
        w += 1;
        Access::forEach(kernel, r, rowPtr, col, [&](int v, int c, bool isWrite) {
            if (c < 0 || c >= n) return;
            if (isWrite)
                lastW[v][c] = w;
            else
                lastR[v][c] = std::max(lastR[v][c], w);
        });
        wave[i] = w;
        depth = std::max(depth, w);
    }
    // counting sort of the order by wave (stable: RACE order inside a wave)
    wp.wavePtr.assign(depth + 1, 0);
    for (int w : wave) wp.wavePtr[w]++;
    for (int w = 0; w < depth; ++w) wp.wavePtr[w + 1] += wp.wavePtr[w];
    wp.rows.resize(order.size());
    std::vector<int> pos(wp.wavePtr.begin(), wp.wavePtr.end() - 1);
    for (size_t i = 0; i < order.size(); ++i) wp.rows[pos[wave[i] - 1]++] = order[i];
    return wp;
}

GatherPlan buildGatherPlan(int kernel, int n, const int *rowPtr, const int *col, const PhaseTable &pt) {
    GatherPlan gp;
    if (kernel != RACE_K_SPMTV && kernel != RACE_K_SYMMSPMV) return gp;
    // rows in RACE's execution order
    std::vector<int> order;
    order.reserve(n);
    for (size_t l = 0; l < pt.leafLo.size(); ++l) {
        const int lo = pt.leafLo[l], hi = pt.leafHi[l];
        if (lo <= hi)
            for (int r = lo; r < hi; ++r) order.push_back(r);
        else
            for (int r = lo; r > hi; --r) order.push_back(r);
    }
    // count, then fill the updates of every b entry in execution order
    const bool symm = kernel == RACE_K_SYMMSPMV;
    std::vector<int> count(n + 1, 0);
    for (int r : order) {
        const int first = symm ? rowPtr[r] + 1 : rowPtr[r];
        if (symm) ++count[r + 1];
        for (int j = first; j < rowPtr[r + 1]; ++j)
            if (col[j] >= 0 && col[j] < n) ++count[col[j] + 1];
    }
    for (int y = 0; y < n; ++y) count[y + 1] += count[y];
    gp.ptr = count;
    gp.entry.assign(count[n], 0);
    gp.row.assign(count[n], 0);
    std::vector<int> fill(count.begin(), count.end() - 1);
    for (int r : order) {
        const int first = symm ? rowPtr[r] + 1 : rowPtr[r];
        if (symm) {
            gp.entry[fill[r]] = -1;
            gp.row[fill[r]++] = r;
        }
        for (int j = first; j < rowPtr[r + 1]; ++j) {
            const int c = col[j];
            if (c < 0 || c >= n) continue;
            gp.entry[fill[c]] = j;
            gp.row[fill[c]++] = r;
        }
    }
    return gp;
}

}  // namespace race
