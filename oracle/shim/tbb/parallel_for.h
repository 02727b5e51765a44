// Minimal stand-in for tbb::parallel_for over a blocked_range, on std::thread.
// Chunks of `grainsize` indices are handed out from an atomic counter to
// `task_scheduler_init`'s thread count (default: hardware concurrency).
// Test infrastructure only (CPU baseline build of the reference sources).
#pragma once
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "tbb/blocked_range.h"
#include "tbb/task_scheduler_init.h"

namespace tbb {

template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &range, const Body &body) {
  const Value b = range.begin(), e = range.end();
  if (!(b < e)) return;
  const std::size_t grain = range.grainsize();
  const std::size_t total = static_cast<std::size_t>(e - b);
  int nthreads = task_scheduler_init::current_threads();
  const std::size_t nchunks = (total + grain - 1) / grain;
  if (nthreads > static_cast<int>(nchunks)) nthreads = static_cast<int>(nchunks);
  if (nthreads <= 1) {
    for (std::size_t c = 0; c < nchunks; ++c) {
      Value lo = b + static_cast<Value>(c * grain);
      Value hi = b + static_cast<Value>(std::min(total, (c + 1) * grain));
      body(blocked_range<Value>(lo, hi, grain));
    }
    return;
  }
  std::atomic<std::size_t> next(0);
  auto worker = [&]() {
    for (;;) {
      std::size_t c = next.fetch_add(1);
      if (c >= nchunks) break;
      Value lo = b + static_cast<Value>(c * grain);
      Value hi = b + static_cast<Value>(std::min(total, (c + 1) * grain));
      body(blocked_range<Value>(lo, hi, grain));
    }
  };
  std::vector<std::thread> pool;
  pool.reserve(nthreads - 1);
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
  worker();
  for (auto &t : pool) t.join();
}

}  // namespace tbb
