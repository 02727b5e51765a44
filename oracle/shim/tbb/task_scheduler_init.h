// Minimal stand-in for tbb::task_scheduler_init: records the thread count the
// shim's parallel_for uses. Test infrastructure only.
#pragma once
#include <thread>

namespace tbb {

class task_scheduler_init {
 public:
  static int &threads_ref() {
    static int n = 0;
    return n;
  }
  static int current_threads() {
    int n = threads_ref();
    if (n <= 0) {
      n = static_cast<int>(std::thread::hardware_concurrency());
      if (n <= 0) n = 1;
    }
    return n;
  }
  explicit task_scheduler_init(int n = -1) {
    prev_ = threads_ref();
    threads_ref() = n;
  }
  ~task_scheduler_init() { threads_ref() = prev_; }

 private:
  int prev_;
};

}  // namespace tbb
