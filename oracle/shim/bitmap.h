/* Bit set with the members RACE's BFS calls on its boundary bitmap
 * (traverse_GAP_graphSoA.cpp:79-84, 184-186, 583-586): Bitmap(n), reset(),
 * set_bit(i), set_bit_atomic(i), get_bit(i). Written for the oracle build
 * from RACE's call sites. Test infrastructure only. */
#ifndef ORACLE_BITMAP_H
#define ORACLE_BITMAP_H
#include <cstdint>
#include <cstddef>
#include <vector>
class Bitmap {
  public:
    explicit Bitmap(size_t size) : words_((size + 63) / 64 + 1, 0) {}
    void reset() { for (auto &w : words_) w = 0; }
    void set_bit(size_t pos) { words_[pos >> 6] |= (uint64_t(1) << (pos & 63)); }
    void set_bit_atomic(size_t pos) { __sync_fetch_and_or(&words_[pos >> 6], uint64_t(1) << (pos & 63)); }
    bool get_bit(size_t pos) const { return (words_[pos >> 6] >> (pos & 63)) & 1; }
  private:
    std::vector<uint64_t> words_;
};
#endif
