// mbir_batch.h -- batched execution of many resident reconstructions (see mbir_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "mbir_engine.h"

namespace mbir {

// Runs fn(i) for i in [0, n) on up to 16 host threads (the caller's included), each with
// `device` current; fn(i) touches only item i's state.  Returns the results per item.  The
// engines' host steps (list and schedule set-up, gain/offset and variance solves, cost) wait on
// their own streams, so running them side by side overlaps those waits and the engines' small
// kernels.
template <typename F>
std::vector<int> parallel_for(int n, int device, F fn) {
  std::vector<int> rc(static_cast<size_t>(std::max(n, 0)), 0);
  if (n <= 0) return rc;
  const int hw = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
  const int nt = std::min(n, std::min(hw, 16));
  std::atomic<int> next{0};
  auto work = [&](bool set_device) {
    if (set_device) cudaSetDevice(device);
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n) break;
      rc[i] = fn(i);
    }
  };
  std::vector<std::thread> pool;
  pool.reserve(nt > 0 ? nt - 1 : 0);
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, true);
  work(false);
  for (auto& t : pool) t.join();
  return rc;
}

class Batch {
 public:
  explicit Batch(int device);
  ~Batch();
  int add(Engine* e);
  int remove(Engine* e);
  size_t size() const { return eng_.size(); }
  // one sweep of every engine; iters[i] = (outer, inner) of engine i (empty: all (0,0));
  // stats (optional) receives 4 values per engine
  int sweep(const std::vector<std::pair<int, int>>& iters, double* stats);
  int run(int max_outer, double tol, int* outer_done, double* final_cost);
  double last_ms() const { return last_ms_; }
  double total_ms() const { return total_ms_; }
  int sweeps() const { return sweeps_; }
  void set_grid(int g) { grid_ = g; }
  // limit of the device-side wait of a colour-1 slice for its series' colour-0 slices; a wait
  // that runs out skips the slice and the sweep returns MBIR_ETIMEOUT
  int set_wait_limit(double seconds) {
    if (!(seconds > 0) || seconds > 600) return MBIR_EINVAL;
    wait_ns_ = static_cast<unsigned long long>(seconds * 1e9);
    return MBIR_OK;
  }
  // slice-group shape of the persistent sweep: 512 threads per CTA (one CTA per SM), 256 (two
  // per SM; a slice is staged in shared memory only when two CTAs' worth fits), or 0 (default):
  // tuned online over the second to fifth sweeps (512, 256, 256, 512), the one with the lower
  // device time per updated voxel kept.  Results do not depend on it.
  int set_threads(int t) {
    if (t != 0 && t != 256 && t != 512) return MBIR_EINVAL;
    threads_ = t;
    tuned_ = 0;
    tune_sweeps_ = 0;
    tune_ms_[0] = tune_ms_[1] = tune_vox_[0] = tune_vox_[1] = 0.0;
    return MBIR_OK;
  }
  // threads per CTA in use: the fixed or tuned value, 0 while the tuning sweeps run
  int threads() const { return threads_ ? threads_ : tuned_; }
  const char* last_error() const { return err_.c_str(); }
  int fail(int code, const std::string& m);

 private:
  int ensure_resources();
  int build_items(const std::vector<SweepArgs>& args);

  int device_;
  std::vector<Engine*> eng_;
  std::vector<int2> items_;
  std::vector<int> need_;
  bool dirty_ = true;
  std::string err_;
  SweepArgs* d_series_ = nullptr;
  int2* d_items_ = nullptr;
  int* d_ctr_ = nullptr;
  double* d_st4_ = nullptr;
  size_t cap_series_ = 0, cap_items_ = 0;
  void* stream_ = nullptr;
  void* ev0_ = nullptr;
  void* ev1_ = nullptr;
  int grid_ = 0;
  int threads_ = 0;                            // 0: tuned online
  int tuned_ = 0;                              // the tuning's choice once made
  int tune_sweeps_ = 0;
  double tune_ms_[2] = {0.0, 0.0}, tune_vox_[2] = {0.0, 0.0};  // [512, 256]
  unsigned long long wait_ns_ = 10000000000ull;  // colour-1 wait limit (10 s)
  // launch groups: voxel-group shape (4) x modality (HAADF, bright field), one launch each
  static constexpr int kShapes = 8;
  int group_off_[kShapes] = {0};
  int group_cnt_[kShapes] = {0};
  double last_ms_ = 0, total_ms_ = 0;
  int sweeps_ = 0;
};

}  // namespace mbir
