/* Stand-in for tbb/task.h: root tasks collected in a task_list and run by
 * spawn_root_and_wait.  With one worker (MBIR_REF_THREADS=1) the tasks run on the calling
 * thread in list order; otherwise each runs on its own std::thread (the reference gives each
 * worker one task).  Tasks are destroyed after they ran, as TBB does.  Test infrastructure. */
#ifndef REF_SHIM_TBB_TASK_H
#define REF_SHIM_TBB_TASK_H
#include <cstddef>
#include <new>
#include <thread>
#include <vector>
#include "tbb/task_scheduler_init.h"
namespace tbb {
class task;
class task_list {
 public:
  void push_back(task& t) { items_.push_back(&t); }
  std::vector<task*> items_;
};
struct root_allocation {};
class task {
 public:
  virtual ~task() {}
  virtual task* execute() = 0;
  static root_allocation allocate_root() { return root_allocation(); }
  static void spawn_root_and_wait(task_list& list) {
    std::vector<task*> items;
    items.swap(list.items_);
    if (task_scheduler_init::default_num_threads() <= 1 || items.size() <= 1) {
      for (task* t : items) t->execute();
    } else {
      std::vector<std::thread> workers;
      workers.reserve(items.size());
      for (task* t : items) workers.emplace_back([t] { t->execute(); });
      for (std::thread& w : workers) w.join();
    }
    for (task* t : items) delete t;
  }
};
}
inline void* operator new(std::size_t n, tbb::root_allocation) { return ::operator new(n); }
inline void operator delete(void* p, tbb::root_allocation) { ::operator delete(p); }
#endif
