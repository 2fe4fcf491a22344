// mbir_batch.h -- batched execution of many resident reconstructions (see mbir_batch.cu).
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "mbir_engine.h"

namespace mbir {

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
  double last_ms_ = 0, total_ms_ = 0;
  int sweeps_ = 0;
};

}  // namespace mbir
