// SELL-C-sigma preparation for SIMD kernels under RACE's coloring
// (RACE::Interface::simdify / simdifyD1, include/simdify.h, and the padding
// step sell_c_sigmize, src/sell_c_sigmize.cpp). Host code: it runs once per
// matrix on the caller's host arrays.
//
// Layout (the reference's): entry j of row r sits at
//   chunkStart[r / C] + r % C + j * C,
// clp[c] is chunk c's padded length, rl[r] row r's own length. A SIMD group
// is simdWidth consecutive rows of one chunk.
#pragma once
#include <string>
#include <vector>

namespace race {

struct SellArrays {
    int simdWidth = 0, C = 0, nrows = 0;
    int *col = nullptr;
    const int *chunkStart = nullptr, *rl = nullptr, *clp = nullptr;
    unsigned char *val = nullptr;  // may be null: columns only
    int valBytes = 8;
};

// Status of the two passes: 0 success, 1 an argument is unusable, 2 a row
// cannot be placed (the reference's `false`); `msg` says which.
enum SimdifyStatus { SIMDIFY_OK = 0, SIMDIFY_BAD_ARG = 1, SIMDIFY_UNPLACEABLE = 2 };

// Distance-2 variant: pads every row of every leaf [lo, hi) of the forward
// schedule (leafLo/leafHi) with columns lo + (row - lo) % simdWidth, then
// reorders each row so that the rows of a SIMD group hold pairwise different
// columns in every slot (from slot 1 on when diagFirst). `collisions` counts
// the rows that needed a move.
int simdifyD2(const SellArrays &m, const std::vector<int> &leafLo, const std::vector<int> &leafHi, bool diagFirst,
              int *collisions, std::string &msg);

// Distance-1 variant: moves each row's entries on the group's earlier rows to
// the row's last slots (nearest row last, or first when dist2Compatible).
int simdifyD1(const SellArrays &m, bool dist2Compatible, std::string &msg);

}  // namespace race
