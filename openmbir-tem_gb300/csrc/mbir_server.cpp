// mbir_server.cpp -- continuous-batching reconstruction server.
//
// Requests (a tilt series + parameters) are queued by submit().  A preparer thread admits
// queued requests in arrival order while their estimated device footprint fits the memory
// budget and a slot is free, and prepares each (upload, tables, forward projection, on the
// request's own engine stream, so this overlaps the batched sweeps).  The worker thread adds
// prepared requests to the batch between steps, runs one outer iteration for every active
// request (one persistent batched ICD sweep, then per-request gain/offset, variance and FP64
// cost), and retires requests whose relative cost change fell below their tolerance (or that
// reached max_outer), copying their volume to host memory and freeing the device memory for
// the next arrivals.  Latency = completion - submission.
#include "mbir_server.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <cmath>

namespace mbir {

namespace {
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

Server::Server(int device, int64_t mem_budget, int max_active)
    : device_(device), budget_(mem_budget), max_active_(max_active > 0 ? max_active : 64) {
  if (budget_ <= 0) {
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(device_);
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
      budget_ = static_cast<int64_t>(free_b * 0.8);
    else
      budget_ = int64_t(8) << 30;
  }
  worker_ = std::thread([this] { loop(); });
  preparer_ = std::thread([this] { prepare_loop(); });
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_.notify_all();
  if (preparer_.joinable()) preparer_.join();
  if (worker_.joinable()) worker_.join();
  batch_.reset();
  for (auto& kv : all_) kv.second->engine.reset();
}

const char* Server::last_error() const {
  thread_local std::string copy;
  std::lock_guard<std::mutex> lk(mu_);
  copy = err_;
  return copy.c_str();
}

size_t Server::estimate_bytes(const Request& r) const {
  const size_t rb = r.params.precision == MBIR_PRECISION_FP64 ? 8 : 4;
  const size_t n_rp = (static_cast<size_t>(r.n_r) + 3) / 4 * 4;
  const size_t sino = static_cast<size_t>(r.n_t) * r.n_theta * n_rp;
  const size_t vox = static_cast<size_t>(r.dims[0]) * r.dims[1] * r.dims[2];
  const size_t host_layout = std::max(static_cast<size_t>(r.n_theta) * r.n_r * r.n_t, vox) * 4;
  size_t bf = 0;
  if (r.params.modality == MBIR_MODALITY_BF) {
    const size_t n_sp = (static_cast<size_t>(r.n_r) + 15) / 16 * 16;
    const size_t lines = static_cast<size_t>(r.dims[0]) * r.dims[1];
    bf = rb * sino + static_cast<size_t>(r.n_t) * r.n_theta * n_sp +
         8 * static_cast<size_t>(r.n_theta) * r.n_r * r.n_t + lines * (8 * 3 + 1);
    if (r.params.nhicd && r.params.call_schedule != 1) {
      // scheduled NHICD calls (Engine::bf_prepare_schedule): the A-column table of every line,
      // [lines][n_theta][acol_width(nb)] float4 with nb = 2 * (voxel / detector size) + 1, the
      // schedule, and the device colouring's packed bins, conflict words and colour planes
      const int levels = std::max(1, r.params.num_resolutions);
      const int lvl = (r.params.level < 0 || r.params.level >= levels) ? levels - 1
                                                                       : r.params.level;
      const int factor = (1 << (levels - 1 - lvl)) * std::max(1, r.params.final_resolution);
      const size_t acol_w = static_cast<size_t>(2 * factor + 1 + 4) / 4;
      const size_t entries = lines * r.n_theta;
      const size_t words = 16;  // 64-bit colour words per bin / line (1024 colours)
      const size_t blocks = (lines + 30) / 31;  // 31-line blocks of the multi-CTA colouring
      bf += entries * acol_w * 16 + (2 * lines + 1) * 4 + entries * 4 + lines * (4 + 20 + 2 + 4) +
            static_cast<size_t>(r.n_theta) * r.n_r * words * 8 + lines * words * 8 +
            blocks * 31 * words * 8 + (3 * blocks + 1) * 4 +
            20 * (std::min<size_t>(64 * words, lines) + 1) * 4 + 64;
    }
  }
  return rb * (3 * sino + vox) + host_layout + bf + (1u << 20);
}

int64_t Server::submit(const mbir_params& p, const float* counts, const float* tilts, int n_theta,
                       int n_r, int n_t, double delta_r, double delta_t, int max_outer,
                       double tol) {
  auto r = std::make_unique<Request>();
  r->params = p;
  r->params.device = device_;
  r->params.order_mode = MBIR_ORDER_PARALLEL;
  r->params.precision = MBIR_PRECISION_FP32;
  r->n_theta = n_theta;
  r->n_r = n_r;
  r->n_t = n_t;
  r->delta_r = delta_r;
  r->delta_t = delta_t;
  r->max_outer = max_outer > 0 ? max_outer : 1;
  r->tol = tol;
  r->engine = std::make_unique<Engine>(r->params);
  int rc = r->engine->set_sinogram(counts, tilts, n_theta, n_r, n_t, delta_r, delta_t);
  int32_t d[6];
  if (rc == 0) rc = r->engine->dims(d);
  if (rc) {
    std::lock_guard<std::mutex> lk(mu_);
    err_ = r->engine->last_error();
    return rc;
  }
  r->dims[0] = d[0];
  r->dims[1] = d[1];
  r->dims[2] = d[2];
  r->bytes = estimate_bytes(*r);
  r->t_submit = now_s();
  std::lock_guard<std::mutex> lk(mu_);
  if (static_cast<int64_t>(r->bytes) > budget_) {
    err_ = "request larger than the server's device-memory budget";
    return MBIR_ENOMEM;
  }
  r->id = next_id_++;
  const int64_t id = r->id;
  queue_.push_back(r.get());
  all_[id] = std::move(r);
  stats_.submitted++;
  cv_.notify_all();
  return id;
}

int Server::admit_locked(std::vector<Request*>& admitted) {
  while (!queue_.empty() && static_cast<int>(active_.size() + prepared_.size() + preparing_ +
                                             admitted.size()) < max_active_) {
    Request* r = queue_.front();
    if (used_ + static_cast<int64_t>(r->bytes) > budget_) break;  // arrival order: no overtaking
    queue_.pop_front();
    used_ += static_cast<int64_t>(r->bytes);
    admitted.push_back(r);
    stats_.admitted++;
    if (r->id < last_admitted_id_) stats_.admitted_out_of_order++;
    last_admitted_id_ = r->id;
    stats_.peak_bytes = std::max(stats_.peak_bytes, used_);
    stats_.peak_active = std::max(
        stats_.peak_active, static_cast<int32_t>(active_.size() + prepared_.size() + preparing_ +
                                                 admitted.size()));
  }
  return 0;
}

void Server::retire(Request* r, int code, const std::string& msg) {
  // called with mu_ held
  r->t_done = now_s();
  r->state = code == 0 ? 2 : code;
  r->error = msg;
  used_ -= static_cast<int64_t>(r->bytes);
  if (code == 0) {
    stats_.completed++;
    latencies_ms_.push_back((r->t_done - r->t_submit) * 1e3);
  } else {
    stats_.failed++;
  }
  done_cv_.notify_all();
  cv_.notify_all();  // memory and a slot are free for the preparer
}

void Server::prepare_loop() {
  cudaSetDevice(device_);
  std::unique_lock<std::mutex> lk(mu_);
  for (;;) {
    std::vector<Request*> admitted;
    cv_.wait(lk, [&] {
      if (stop_) return true;
      admit_locked(admitted);
      return !admitted.empty();
    });
    if (stop_) {
      for (Request* r : admitted) retire(r, MBIR_ESTATE, "server stopped");
      break;
    }
    preparing_ += static_cast<int>(admitted.size());
    lk.unlock();
    std::vector<int> rcs(admitted.size());
    std::vector<std::string> msgs(admitted.size());
    for (size_t k = 0; k < admitted.size(); k++) {
      Request* r = admitted[k];
      r->t_admit = now_s();
      rcs[k] = r->engine->prepare();
      if (rcs[k]) {
        // the request's device memory goes back now: the budget already counts it as free
        msgs[k] = r->engine->last_error();
        r->engine.reset();
      }
    }
    lk.lock();
    preparing_ -= static_cast<int>(admitted.size());
    for (size_t k = 0; k < admitted.size(); k++) {
      if (rcs[k])
        retire(admitted[k], MBIR_EDEVICE, msgs[k]);
      else
        prepared_.push_back(admitted[k]);
    }
    cv_.notify_all();
  }
}

void Server::loop() {
  cudaSetDevice(device_);
  batch_ = std::make_unique<Batch>(device_);
  std::unique_lock<std::mutex> lk(mu_);
  for (;;) {
    cv_.wait(lk, [&] { return stop_ || !prepared_.empty() || !active_.empty(); });
    if (stop_) break;
    std::vector<Request*> joining;
    joining.swap(prepared_);
    lk.unlock();
    const double t_busy0 = now_s();
    std::vector<std::pair<Request*, std::string>> failed;
    std::vector<Request*> ok;
    for (Request* r : joining) {
      if (batch_->add(r->engine.get())) {
        failed.emplace_back(r, batch_->last_error());
        r->engine.reset();  // not in the batch: free its device memory outside the lock
      } else {
        ok.push_back(r);
      }
    }
    lk.lock();
    for (auto& f : failed) retire(f.first, MBIR_EDEVICE, f.second);
    for (Request* r : ok) {
      r->state = 1;
      active_.push_back(r);
    }
    std::vector<Request*> cur = active_;
    lk.unlock();

    std::vector<Request*> finished;
    std::vector<std::pair<Request*, std::string>> broken;
    if (!cur.empty()) {
      // the batch keeps engines in insertion order; map each to its own outer index
      std::vector<std::pair<int, int>> iters;
      iters.reserve(cur.size());
      for (Request* r : cur) iters.emplace_back(r->outer_done, 0);
      int rc = batch_->sweep(iters, nullptr);
      if (rc) {
        for (Request* r : cur) broken.emplace_back(r, batch_->last_error());
      } else {
        // per request, side by side: gain/offset, variance, cost and the stop test
        // (outcome 0: continue, 1: finished, 2: failed)
        std::vector<int> outcome(cur.size(), 0);
        parallel_for(static_cast<int>(cur.size()), device_, [&](int k) {
          Request* r = cur[k];
          Engine* e = r->engine.get();
          const bool bf = r->params.modality == MBIR_MODALITY_BF;
          int erc = 0;
          if (r->params.joint_estimation) erc = e->joint_estimation();
          if (!erc && (bf ? r->params.noise_estimation : r->params.noise_model))
            erc = e->update_weights();
          if (erc) return outcome[k] = 2;
          r->outer_done++;
          // a bright-field call updates 1/20 of the voxel lines (NHICD): the cost is compared
          // once per equivalent iteration of 20 calls
          const int period = bf ? 20 : 1;
          bool conv = false;
          if (r->outer_done % period == 0 || r->outer_done >= r->max_outer) {
            double c = 0;
            if (e->compute_cost(nullptr, &c)) return outcome[k] = 2;
            conv = r->outer_done > period && std::fabs(c - r->cost) <= r->tol * std::fabs(c);
            r->prev_cost = r->cost;
            r->cost = c;
          }
          if (conv || r->outer_done >= r->max_outer) outcome[k] = 1;
          return 0;
        });
        for (size_t k = 0; k < cur.size(); k++) {
          if (outcome[k] == 2)
            broken.emplace_back(cur[k], cur[k]->engine->last_error());
          else if (outcome[k] == 1)
            finished.push_back(cur[k]);
        }
      }
      for (auto it = finished.begin(); it != finished.end();) {
        Request* r = *it;
        r->result.resize(static_cast<size_t>(r->dims[0]) * r->dims[1] * r->dims[2]);
        if (r->engine->get_volume(r->result.data(), static_cast<int64_t>(r->result.size()))) {
          broken.emplace_back(r, r->engine->last_error());
          it = finished.erase(it);
        } else {
          ++it;
        }
      }
    }
    lk.lock();
    stats_.busy_s += now_s() - t_busy0;
    stats_.batched_sweeps = batch_->sweeps();
    stats_.batched_sweep_ms = batch_->total_ms();
    auto drop = [&](Request* r) {
      batch_->remove(r->engine.get());
      mbir_status st{};
      r->engine->status(&st);
      stats_.voxel_updates += static_cast<double>(st.voxels_visited);
      r->engine.reset();
      active_.erase(std::remove(active_.begin(), active_.end(), r), active_.end());
    };
    for (Request* r : finished) {
      drop(r);
      retire(r, 0, "");
    }
    for (auto& b : broken) {
      drop(b.first);
      retire(b.first, MBIR_EDEVICE, b.second);
    }
  }
}

int Server::poll(int64_t id, int* state, double* latency_ms, int* outer_done, double* cost) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end()) return MBIR_EINVAL;
  Request* r = it->second.get();
  if (state) *state = r->state;
  if (latency_ms) *latency_ms = r->state == 2 ? (r->t_done - r->t_submit) * 1e3 : -1.0;
  if (outer_done) *outer_done = r->outer_done;
  if (cost) *cost = r->cost;
  return MBIR_OK;
}

int Server::wait(int64_t id, double timeout_s) {
  std::unique_lock<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end()) return MBIR_EINVAL;
  Request* r = it->second.get();
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                            std::chrono::duration<double>(timeout_s));
  if (!done_cv_.wait_until(lk, deadline, [&] { return r->state == 2 || r->state < 0; }))
    return MBIR_ETIMEOUT;
  if (r->state < 0) err_ = "request " + std::to_string(id) + ": " + r->error;
  return r->state == 2 ? MBIR_OK : r->state;
}

int Server::result(int64_t id, float* out, int64_t n, int32_t* dims) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end()) return MBIR_EINVAL;
  Request* r = it->second.get();
  if (r->state != 2) return r->state < 0 ? r->state : MBIR_ESTATE;
  if (dims)
    for (int i = 0; i < 3; i++) dims[i] = r->dims[i];
  if (out) {
    if (n < static_cast<int64_t>(r->result.size())) return MBIR_EINVAL;
    std::copy(r->result.begin(), r->result.end(), out);
  }
  return MBIR_OK;
}

int Server::release(int64_t id) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = all_.find(id);
  if (it == all_.end()) return MBIR_EINVAL;
  if (it->second->state == 0 || it->second->state == 1) return MBIR_ESTATE;
  all_.erase(it);
  return MBIR_OK;
}

int Server::stats(ServerStats* st) {
  std::lock_guard<std::mutex> lk(mu_);
  ServerStats s = stats_;
  s.budget_bytes = budget_;
  s.active = static_cast<int32_t>(active_.size());
  s.queued = static_cast<int32_t>(queue_.size());
  if (!latencies_ms_.empty()) {
    std::vector<double> v = latencies_ms_;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) {
      const double pos = q * (v.size() - 1);
      const size_t i = static_cast<size_t>(pos);
      const double f = pos - i;
      return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
    };
    s.p50_ms = pct(0.5);
    s.p99_ms = pct(0.99);
    double m = 0;
    for (double x : v) m += x;
    s.mean_ms = m / v.size();
  }
  *st = s;
  return MBIR_OK;
}

}  // namespace mbir
