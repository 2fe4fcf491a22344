// mbir_server.h -- continuous-batching request server over Engine + Batch (mbir_server.cpp).
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mbir_batch.h"

namespace mbir {

struct Request {
  int64_t id = 0;
  mbir_params params{};
  std::vector<float> counts, tilts;
  int n_theta = 0, n_r = 0, n_t = 0;
  double delta_r = 1, delta_t = 1;
  int max_outer = 20;
  double tol = 1e-4;
  // lifecycle
  int state = 0;            // 0 queued or being prepared, 1 active, 2 done, <0 error code
  double t_submit = 0, t_admit = 0, t_done = 0;  // seconds (steady clock)
  int outer_done = 0;
  double cost = 0, prev_cost = 0;
  size_t bytes = 0;
  std::unique_ptr<Engine> engine;
  std::vector<float> result;  // [z][x][y]
  int dims[3] = {0, 0, 0};
  std::string error;
};

struct ServerStats {
  int64_t submitted = 0, completed = 0, failed = 0;
  int32_t active = 0, queued = 0;
  double p50_ms = 0, p99_ms = 0, mean_ms = 0;
  double voxel_updates = 0;   // voxel visits over all completed and active requests
  double busy_s = 0;          // time the worker spent with at least one active request
  double batched_sweep_ms = 0;
  int64_t batched_sweeps = 0;
  int64_t budget_bytes = 0, peak_bytes = 0;
  int32_t peak_active = 0;
  int64_t admitted = 0, admitted_out_of_order = 0;
};

class Server {
 public:
  Server(int device, int64_t mem_budget, int max_active);
  ~Server();
  int64_t submit(const mbir_params& p, const float* counts, const float* tilts, int n_theta,
                 int n_r, int n_t, double delta_r, double delta_t, int max_outer, double tol);
  // state, latency_ms, outer iterations, cost
  int poll(int64_t id, int* state, double* latency_ms, int* outer_done, double* cost);
  int wait(int64_t id, double timeout_s);
  int result(int64_t id, float* out, int64_t n, int32_t* dims);
  int release(int64_t id);
  int stats(ServerStats* st);
  // a copy taken under the lock, owned by the calling thread (valid until its next call)
  const char* last_error() const;

 private:
  void loop();
  void prepare_loop();
  size_t estimate_bytes(const Request& r) const;
  int admit_locked(std::vector<Request*>& admitted);
  void retire(Request* r, int code, const std::string& msg);

  int device_;
  int64_t budget_;
  int max_active_;
  int64_t used_ = 0;
  int64_t last_admitted_id_ = 0;
  int64_t next_id_ = 1;
  mutable std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<Request*> queue_;
  std::vector<Request*> active_;
  std::vector<Request*> prepared_;  // prepared, joining the batch at the worker's next step
  int preparing_ = 0;               // admitted, being prepared
  std::map<int64_t, std::unique_ptr<Request>> all_;
  std::vector<double> latencies_ms_;
  bool stop_ = false;
  std::thread worker_, preparer_;
  std::unique_ptr<Batch> batch_;
  std::string err_;
  ServerStats stats_;
};

}  // namespace mbir
