/* Stand-in for tbb/task_scheduler_init.h.  default_num_threads() is the worker count the
 * reference splits its y ranges over: MBIR_REF_THREADS when set (1 gives the sequential ICD of
 * one y range), else the host's hardware threads.  Test infrastructure only. */
#ifndef REF_SHIM_TBB_TASK_SCHEDULER_INIT_H
#define REF_SHIM_TBB_TASK_SCHEDULER_INIT_H
#include <cstdlib>
#include <thread>
namespace tbb {
class task_scheduler_init {
 public:
  task_scheduler_init() {}
  explicit task_scheduler_init(int) {}
  static int default_num_threads() {
    const char* s = std::getenv("MBIR_REF_THREADS");
    if (s && std::atoi(s) > 0) return std::atoi(s);
    const unsigned n = std::thread::hardware_concurrency();
    return n ? static_cast<int>(n) : 1;
  }
};
}
#endif
