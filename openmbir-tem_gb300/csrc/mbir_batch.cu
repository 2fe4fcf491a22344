// mbir_batch.cu -- many reconstructions of uneven size advanced together: one persistent,
// cooperative launch per ICD sweep covers every voxel slice of every engine in the batch
// (batch_sweep_kernel in mbir_sweep.cuh); gain/offset, variance and cost updates stay per
// engine.  Each engine keeps its volume, error sinogram and nuisance state resident in HBM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "mbir_batch.h"

namespace mbir {

Batch::Batch(int device) : device_(device) {}

Batch::~Batch() {
  if (d_series_) cudaFree(d_series_);
  if (d_items_) cudaFree(d_items_);
  if (d_ctr_) cudaFree(d_ctr_);
  if (d_st4_) cudaFree(d_st4_);
  if (ev0_) cudaEventDestroy(static_cast<cudaEvent_t>(ev0_));
  if (ev1_) cudaEventDestroy(static_cast<cudaEvent_t>(ev1_));
  if (stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
}

int Batch::fail(int code, const std::string& m) {
  err_ = m;
  return code;
}

int Batch::add(Engine* e) {
  if (!e) return fail(MBIR_EINVAL, "batch_add: null engine");
  if (e->state() < 2) return fail(MBIR_ESTATE, "batch_add: prepare the engine first");
  if (e->fp64() || e->params().order_mode != MBIR_ORDER_PARALLEL)
    return fail(MBIR_ENOTSUP, "batch_add: FP32 parallel-order engines only");
  if (e->params().device != device_) return fail(MBIR_EINVAL, "batch_add: engine on another device");
  if (std::find(eng_.begin(), eng_.end(), e) != eng_.end()) return MBIR_OK;
  eng_.push_back(e);
  dirty_ = true;
  return MBIR_OK;
}

int Batch::remove(Engine* e) {
  auto it = std::find(eng_.begin(), eng_.end(), e);
  if (it == eng_.end()) return fail(MBIR_EINVAL, "batch_remove: engine not in batch");
  eng_.erase(it);
  dirty_ = true;
  return MBIR_OK;
}

int Batch::ensure_resources() {
  if (!stream_) {
    if (cudaSetDevice(device_) != cudaSuccess) return fail(MBIR_EDEVICE, "batch: cudaSetDevice");
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      return fail(MBIR_EDEVICE, "batch: stream");
    stream_ = s;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    ev0_ = a;
    ev1_ = b;
  }
  const size_t n = eng_.size();
  if (n > cap_series_) {
    if (d_series_) cudaFree(d_series_);
    if (d_ctr_) cudaFree(d_ctr_);
    if (d_st4_) cudaFree(d_st4_);
    cap_series_ = std::max<size_t>(n, 64);
    if (cudaMalloc(&d_series_, sizeof(SweepArgs) * cap_series_) != cudaSuccess ||
        cudaMalloc(&d_ctr_, sizeof(int) * (kShapes + 2 * cap_series_)) != cudaSuccess ||
        cudaMalloc(&d_st4_, sizeof(double) * kStatSlots * cap_series_) != cudaSuccess)
      return fail(MBIR_ENOMEM, "batch: device allocation");
  }
  return MBIR_OK;
}

// Items grouped by voxel-group shape and modality (one launch each); within a group, colour-0 slices of
// every engine, then colour-1 slices, engines with the most voxels per slice first so the long
// items start early.
int Batch::build_items(const std::vector<SweepArgs>& args) {
  const int n = static_cast<int>(args.size());
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return static_cast<long long>(args[a].g.n_z) * args[a].g.n_x >
           static_cast<long long>(args[b].g.n_z) * args[b].g.n_x;
  });
  items_.clear();
  need_.assign(n, 0);
  for (int g = 0; g < kShapes; g++) {
    group_off_[g] = static_cast<int>(items_.size());
    for (int colour = 0; colour < 2; colour++)
      for (int s : order) {
        const int sh = (args[s].shape >= 1 && args[s].shape <= 4) ? args[s].shape : 4;
        if (2 * (sh - 1) + (args[s].bf ? 1 : 0) != g) continue;
        for (int y = colour; y < args[s].g.n_y; y += 2) {
          items_.push_back(make_int2(s, y));
          if (colour == 0) need_[s]++;
        }
      }
    group_cnt_[g] = static_cast<int>(items_.size()) - group_off_[g];
  }
  if (items_.size() > cap_items_) {
    if (d_items_) cudaFree(d_items_);
    cap_items_ = items_.size() * 2;
    if (cudaMalloc(&d_items_, sizeof(int2) * cap_items_) != cudaSuccess)
      return fail(MBIR_ENOMEM, "batch: item allocation");
  }
  cudaMemcpy(d_items_, items_.data(), sizeof(int2) * items_.size(), cudaMemcpyHostToDevice);
  return MBIR_OK;
}

int Batch::sweep(const std::vector<std::pair<int, int>>& iters, double* stats) {
  if (eng_.empty()) return MBIR_OK;
  int rc = ensure_resources();
  if (rc) return rc;
  const int n = static_cast<int>(eng_.size());
  std::vector<SweepArgs> args(n);
  size_t smem = 0;
  int nb = -1, max_theta = 0;
  int max_optin = 0, per_sm = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_);
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device_);
  // staged slices must leave room for the kernel's static shared memory (and, with 256-thread
  // CTAs, for a second CTA on the SM)
  // online tuning: the batch's first sweep (every voxel updated) runs at 512 threads and is not
  // measured; the next four run 512, 256, 256, 512 (a drift in the cost per voxel as the
  // reconstructions converge cancels)
  const bool tuning = threads_ == 0 && tuned_ == 0;
  const int trial = tune_sweeps_ - 1;
  const int threads = threads_ ? threads_
                               : (tuned_ ? tuned_ : (trial == 1 || trial == 2 ? 256 : 512));
  const bool two = threads == 256;
  const size_t stage_cap = two ? static_cast<size_t>(std::min(max_optin, per_sm / 2 - 1024)) - 2048
                               : static_cast<size_t>(max_optin) - 2048;
  // per-engine set-up (row order, bright-field list, active mask, level schedule) side by side
  std::vector<size_t> needs(n, 0);
  const std::vector<int> rcs = parallel_for(n, device_, [&](int i) {
    const int outer = iters.empty() ? 0 : iters[i].first;
    const int inner = iters.empty() ? 0 : iters[i].second;
    return eng_[i]->batch_args(outer, inner, &args[i], &needs[i]);
  });
  for (int i = 0; i < n; i++)
    if (rcs[i]) return fail(rcs[i], eng_[i]->last_error());
  for (int i = 0; i < n; i++) {
    const size_t need = needs[i];
    if (nb < 0) nb = eng_[i]->nb();
    if (eng_[i]->nb() != nb) return fail(MBIR_ENOTSUP, "batch: engines at different voxel sizes");
    max_theta = std::max(max_theta, args[i].g.n_theta);
    if (args[i].smem_rows) {
      if (need > stage_cap) {
        args[i].smem_rows = 0;
        args[i].n_rs = 0;
      } else {
        smem = std::max(smem, need);
      }
    }
  }
  for (int i = 0; i < n; i++)
    if (!args[i].smem_rows)
      smem = std::max(smem, sweep_smem_bytes(args[i].g.n_theta, args[i].g.n_x, 0, 1,
                                             args[i].g.bins, 0, 0));
  (void)max_theta;
  if (dirty_ || items_.empty()) {
    if ((rc = build_items(args))) return rc;
    dirty_ = false;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  cudaMemcpyAsync(d_series_, args.data(), sizeof(SweepArgs) * n, cudaMemcpyHostToDevice, s);
  // counters: one queue per shape group, then done[n], need[n]
  std::vector<int> ctr(kShapes + 2 * n, 0);
  // MBIR_TEST_UNMET_BATCH_WAIT=1 (failure-detection tests only): every series needs one more
  // colour-0 slice than it has, so each colour-1 slice's bounded wait runs out
  const char* unmet_env = std::getenv("MBIR_TEST_UNMET_BATCH_WAIT");
  const bool unmet = unmet_env != nullptr && unmet_env[0] == '1';
  for (int i = 0; i < n; i++) ctr[kShapes + n + i] = need_[i] + (unmet ? 1 : 0);
  cudaMemcpyAsync(d_ctr_, ctr.data(), sizeof(int) * ctr.size(), cudaMemcpyHostToDevice, s);
  cudaEventRecord(static_cast<cudaEvent_t>(ev0_), s);
  for (int g = 0; g < kShapes; g++) {
    if (group_cnt_[g] == 0) continue;
    BatchArgs b{};
    b.series = d_series_;
    b.items = d_items_ + group_off_[g];
    b.n_items = group_cnt_[g];
    b.queue = d_ctr_ + g;
    b.done = d_ctr_ + kShapes;
    b.need = d_ctr_ + kShapes + n;
    b.wait_ns = wait_ns_;
    rc = launch_batch_sweep(b, nb, g, threads, smem, grid_, s);
    if (rc) return fail(MBIR_EDEVICE, std::string("batch sweep launch: ") +
                                          cudaGetErrorString(cudaGetLastError()));
  }
  for (int i = 0; i < n; i++) {
    const int ny = args[i].g.n_y;
    if ((rc = launch_reduce_stats(eng_[i]->slice_stats(), ny, kStatSlots, d_st4_ + kStatSlots * i, s)))
      return fail(MBIR_EDEVICE, "batch stats reduce");
  }
  cudaEventRecord(static_cast<cudaEvent_t>(ev1_), s);
  std::vector<double> st(static_cast<size_t>(kStatSlots) * n);
  cudaMemcpyAsync(st.data(), d_st4_, sizeof(double) * st.size(), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return fail(MBIR_EDEVICE, std::string("batch sweep: ") + cudaGetErrorString(cudaGetLastError()));
  float ms = 0;
  cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev0_), static_cast<cudaEvent_t>(ev1_));
  last_ms_ = ms;
  total_ms_ += ms;
  sweeps_++;
  // every engine's error word is read (and cleared) before the first failure is reported, so
  // that no stale word fails the next sweep
  int first_bad = -1, first_rc = MBIR_OK;
  for (int i = 0; i < n; i++)
    if ((rc = eng_[i]->check_errors()) && first_bad < 0) {
      first_bad = i;
      first_rc = rc;
    }
  if (first_bad >= 0) return fail(first_rc, eng_[first_bad]->last_error());
  const std::vector<int> fin = parallel_for(n, device_, [&](int i) {
    const int outer = iters.empty() ? 0 : iters[i].first;
    const int inner = iters.empty() ? 0 : iters[i].second;
    return eng_[i]->batch_finish(outer, inner, st.data() + kStatSlots * i, ms / n);
  });
  for (int i = 0; i < n; i++) {
    if (fin[i]) return fail(fin[i], eng_[i]->last_error());
    if (stats)
      for (int k = 0; k < kStatSlots; k++) stats[kStatSlots * i + k] = st[kStatSlots * i + k];
  }
  if (tuning) {
    // device time per updated voxel of each slice-group shape
    if (trial >= 0) {
      double vox = 0.0;
      for (int i = 0; i < n; i++) vox += st[kStatSlots * i + 3];
      const int k = two ? 1 : 0;
      tune_ms_[k] += ms;
      tune_vox_[k] += vox;
    }
    if (++tune_sweeps_ >= 5) {
      tuned_ = (tune_vox_[0] > 0 && tune_vox_[1] > 0 &&
                tune_ms_[1] / tune_vox_[1] < tune_ms_[0] / tune_vox_[0])
                   ? 256
                   : 512;
    }
  }
  return MBIR_OK;
}

// Outer iterations for every engine: batched sweep, then per engine gain/offset and variance
// estimation and the FP64 MAP cost; an engine leaves the batch once its relative cost change
// falls below tol (after its first outer iteration) or after max_outer iterations.
int Batch::run(int max_outer, double tol, int* outer_done, double* final_cost) {
  std::vector<Engine*> all = eng_;
  const int n = static_cast<int>(all.size());
  std::vector<double> prev(n, 0.0), cost(n, 0.0);
  std::vector<int> done_at(n, 0);
  std::vector<char> active(n, 1);
  for (int it = 0; it < max_outer; ++it) {
    std::vector<Engine*> cur;
    std::vector<int> idx;
    for (int i = 0; i < n; i++)
      if (active[i]) {
        cur.push_back(all[i]);
        idx.push_back(i);
      }
    if (cur.empty()) break;
    if (cur.size() != eng_.size() || !std::equal(cur.begin(), cur.end(), eng_.begin())) {
      eng_ = cur;
      dirty_ = true;
    }
    std::vector<std::pair<int, int>> iters(cur.size(), std::make_pair(it, 0));
    int rc = sweep(iters, nullptr);
    if (rc) return rc;
    // per engine (side by side): gain/offset, variance, cost and the stop test
    const std::vector<int> rcs = parallel_for(static_cast<int>(cur.size()), device_, [&](int k) {
      Engine* e = cur[k];
      const int i = idx[k];
      const mbir_params& p = e->params();
      const bool bf = p.modality == MBIR_MODALITY_BF;
      int erc;
      if (p.joint_estimation && (erc = e->joint_estimation())) return erc;
      if ((bf ? p.noise_estimation : p.noise_model) && (erc = e->update_weights())) return erc;
      done_at[i] = it + 1;
      // bright field: one NHICD call per outer iteration, the cost compared once per
      // equivalent iteration (20 calls)
      const int period = bf ? 20 : 1;
      if ((it + 1) % period != 0 && it + 1 < max_outer) return 0;
      if ((erc = e->compute_cost(nullptr, &cost[i]))) return erc;
      if (it + 1 > period && std::fabs(cost[i] - prev[i]) <= tol * std::fabs(cost[i])) active[i] = 0;
      prev[i] = cost[i];
      return 0;
    });
    for (size_t k = 0; k < cur.size(); k++)
      if (rcs[k]) return fail(rcs[k], cur[k]->last_error());
  }
  eng_ = all;
  dirty_ = true;
  for (int i = 0; i < n; i++) {
    if (outer_done) outer_done[i] = done_at[i];
    if (final_cost) final_cost[i] = cost[i];
  }
  return MBIR_OK;
}

}  // namespace mbir
