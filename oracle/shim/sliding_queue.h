/* Frontier queue with the members RACE's level-synchronous BFS uses
 * (traverse_GAP_graphSoA.cpp:137-219, 262-305): SlidingQueue<T>(n) with
 * push_back, slide_window, empty, begin, end, size; and a per-thread
 * QueueBuffer<T>(queue) with push_back and flush. The window [begin,end) is the
 * current frontier; pushes land after it and become the next frontier on
 * slide_window(). Written for the oracle build from RACE's call sites.
 * Test infrastructure only. */
#ifndef ORACLE_SLIDING_QUEUE_H
#define ORACLE_SLIDING_QUEUE_H
#include <cstddef>
#include <vector>
#include "platform_atomics.h"

template <typename T> class QueueBuffer;

template <typename T>
class SlidingQueue {
  public:
    explicit SlidingQueue(size_t shared_size) : data_(shared_size + 1), in_(0), lo_(0), hi_(0) {}
    void push_back(T v) { data_[in_++] = v; }
    bool empty() const { return lo_ == hi_; }
    void reset() { in_ = 0; lo_ = 0; hi_ = 0; }
    void slide_window() { lo_ = hi_; hi_ = in_; }
    typedef T *iterator;
    iterator begin() { return data_.data() + lo_; }
    iterator end() { return data_.data() + hi_; }
    size_t size() const { return hi_ - lo_; }
  private:
    friend class QueueBuffer<T>;
    std::vector<T> data_;
    size_t in_, lo_, hi_;
};

template <typename T>
class QueueBuffer {
  public:
    explicit QueueBuffer(SlidingQueue<T> &master, size_t cap = 16384) : master_(master), cap_(cap) { buf_.reserve(cap); }
    void push_back(T v) {
        if (buf_.size() == cap_) flush();
        buf_.push_back(v);
    }
    void flush() {
        if (buf_.empty()) return;
        size_t at = __sync_fetch_and_add(&master_.in_, buf_.size());
        for (size_t i = 0; i < buf_.size(); ++i) master_.data_[at + i] = buf_[i];
        buf_.clear();
    }
  private:
    SlidingQueue<T> &master_;
    size_t cap_;
    std::vector<T> buf_;
};
#endif
