// Minimal stand-in for tbb::blocked_range (TBB is absent from this image).
// Test infrastructure only: used to build the reference's own sources with
// -DUSE_TBB so its multithreaded code path can be timed as the CPU baseline.
#pragma once
#include <cstddef>

namespace tbb {

template <typename Value>
class blocked_range {
  Value begin_, end_;
  std::size_t grain_;

 public:
  blocked_range(Value b, Value e, std::size_t grain = 1)
      : begin_(b), end_(e), grain_(grain ? grain : 1) {}
  Value begin() const { return begin_; }
  Value end() const { return end_; }
  std::size_t grainsize() const { return grain_; }
  bool empty() const { return !(begin_ < end_); }
};

}  // namespace tbb
