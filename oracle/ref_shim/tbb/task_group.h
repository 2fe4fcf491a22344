/* Stand-in for tbb/task_group.h.  run() executes the functor at once on the calling thread:
 * the reference's forward projection adds the z slices' contributions into shared sinogram
 * entries without synchronisation, and running them in turn gives the deterministic sums of
 * the serial build.  Test infrastructure only. */
#ifndef REF_SHIM_TBB_TASK_GROUP_H
#define REF_SHIM_TBB_TASK_GROUP_H
namespace tbb {
class task_group {
 public:
  template <class F>
  void run(F f) { f(); }
  void wait() {}
};
}
#endif
