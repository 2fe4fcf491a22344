// mbir_engine_bf.cu -- bright-field (BF) side of the engine: -log counts, per-entry weights and
// the Bragg selector, the non-homogeneous ICD (NHICD) line lists, offset-only joint estimation,
// the single global noise variance, the BF cost and the BFReconstructionEngine::execute loops.
//
// Reference: Code/MBIRLib/BrightField/BFReconstructionEngine.cpp:555-858 (execute loops),
// BFReconstructionEngine_Extra.cpp:476-1273 (updateVoxels, NHICD, stop rule),
// BFForwardModel.cpp:328-531, 812-972 (weights, estimates, selector, cost, raw counts).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "mbir_engine.h"

namespace mbir {

namespace {
constexpr int kNumHomogeneous = 20;     // MBIR::Constants::k_NumHomogeniousIter
constexpr int kNumNonHomogeneous = 20;  // k_NumNonHomogeniousIter
constexpr double kDefBragg = 5e10;      // DefBraggThreshold (BFConstants.h)

template <typename T>
void dfree_any(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// boost::uniform_int<uint32_t>(0, range) on mt19937: the raw draw divided by the bucket size,
// redrawn when the quotient exceeds range
uint32_t uniform_draw(MT19937& gen, uint32_t range) {
  const uint32_t brange = 0xffffffffu;
  if (range == 0) return 0;
  if (range == brange) return gen.next();
  uint32_t bucket = brange / (range + 1u);
  if (brange % (range + 1u) == range) ++bucket;
  for (;;) {
    const uint32_t r = gen.next() / bucket;
    if (r <= range) return r;
  }
}
}  // namespace

void rand_list_perm(uint32_t seed, int n, std::vector<int32_t>& out) {
  out.resize(std::max(n, 0));
  for (int i = 0; i < n; i++) out[i] = i;
  if (n < 2) return;
  MT19937 gen(seed);
  for (int i = 1; i < n; i++) {
    const uint32_t r = uniform_draw(gen, static_cast<uint32_t>(n - 1));
    if (r >= static_cast<uint32_t>(n)) continue;
    std::swap(out[i], out[r]);
  }
}

// the BF command line passes the offset d = -log(default_dosage + bf_offset)
// (BFReconstructionArgsParser.cpp:272-274)
double Engine::bf_default_offset() const {
  const double d = -std::log(p_.default_dosage + p_.bf_offset);
  // the reference's pipeline stores it in a float member (BFMultiResolutionReconstruction.h:83)
  return p_.float_params ? static_cast<double>(static_cast<float>(d)) : d;
}

// processRawCounts (BFForwardModel.cpp:939-972): counts + bf_offset, then -log(c / BF_MAX) with
// BF_MAX = 1; the nuisance parameters were created from the raw counts before this (execute
// :374-385).  A negative count ends its (theta, r) row early, as the reference's break does.
int Engine::bf_prepare_host() {
  const Geometry& g = g_;
  const size_t nh = static_cast<size_t>(g.n_theta) * g.n_r * g.n_t;
  ylog_.resize(nh);
  host_parallel(g.n_theta, [&](int th_begin, int th_end) {
    for (int th = th_begin; th < th_end; th++)
      for (int r = 0; r < g.n_r; r++) {
        const size_t b = (static_cast<size_t>(th) * g.n_r + r) * g.n_t;
        bool stopped = false;
        for (int t = 0; t < g.n_t; t++) {
          double v = static_cast<double>(counts_[b + t]);
          if (!stopped) {
            v += p_.bf_offset;
            if (v < 0) {
              stopped = true;
            } else {
              v = -std::log(v / 1.0);
            }
          }
          ylog_[b + t] = v;
        }
      }
  });
  // GenRegularList + GenRandList (execute :555-559): position perm[i] holds line i
  const int nl = g.n_z * g.n_x;
  std::vector<int32_t> perm;
  rand_list_perm(p_.seed, nl, perm);
  bf_master_.assign(nl, 0);
  for (int i = 0; i < nl; i++) bf_master_[perm[i]] = i;
  bf_listsel_ = 0;
  bf_eff_ = 0;
  bf_calls_ = 0;
  bragg_t_ = p_.bragg_threshold;
  return MBIR_OK;
}

BfSino Engine::bf_sino() const {
  BfSino b{};
  b.e = d_e_;
  b.w = d_w_;
  b.sel = d_sel_;
  b.n_theta = g_.n_theta;
  b.n_r = g_.n_r;
  b.n_rp = n_rp_;
  b.n_sp = n_sp_;
  b.n_t = g_.n_t;
  b.fp64 = fp64_;
  return b;
}

// calculateMeasurementWeight (BFForwardModel.cpp:328-385) without IDENTITY_NOISE_MODEL:
// w = BF_MAX / exp(y), divided by the view's variance when NOISE_ESTIMATION is on; every entry
// selected.
int Engine::bf_upload() {
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nh = static_cast<size_t>(g.n_theta) * g.n_r * g.n_t;
  // every entry is written below, by the threads (so they also take the first-touch faults)
  std::unique_ptr<double[]> w(new double[nh]);
  host_parallel(g.n_theta, [&](int th_begin, int th_end) {
    for (int th = th_begin; th < th_end; th++)
      for (int r = 0; r < g.n_r; r++)
        for (int t = 0; t < g.n_t; t++) {
          const size_t i = (static_cast<size_t>(th) * g.n_r + r) * g.n_t + t;
          double v = 1.0 / std::exp(ylog_[i]);
          if (p_.noise_estimation) v /= alpha_[th];
          w[i] = v;
        }
  });
  cudaMemcpyAsync(d_stage64_, w.get(), sizeof(double) * nh, cudaMemcpyHostToDevice, s);
  int rc = launch_layout_from_double(d_stage64_, d_w_, g.n_theta, g.n_r, n_rp_, g.n_t, fp64_, s);
  if (rc) return cuda_check(rc, "weights upload");
  cudaMemsetAsync(d_sel_, 1, static_cast<size_t>(g.n_t) * g.n_theta * n_sp_, s);
  const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
  cudaMemsetAsync(d_magfx_, 0, sizeof(unsigned long long) * nl, s);
  cudaMemsetAsync(d_mag_, 0, sizeof(double) * nl, s);
  cudaMemsetAsync(d_filt_, 0, sizeof(double) * nl, s);
  cudaMemsetAsync(d_active_, 1, nl, s);
  cudaMemcpyAsync(d_alpha_, alpha_.data(), sizeof(double) * g.n_theta, cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "BF upload");
  return MBIR_OK;
}

// Level-scheduled calls (FP32, parallel order, NHICD): the A-column table of every voxel line
// (built once on the device by the sweep's own arithmetic) and each entry's first bin and
// nonzero mask: packed on the device for the device colouring, unpacked on the host
// (host_footprint_bins) for the host schedules.  Without room for the table the calls walk the
// rows.
int Engine::bf_prepare_schedule() {
  if (fp64_ || !p_.nhicd || p_.order_mode != MBIR_ORDER_PARALLEL || p_.call_schedule == 1)
    return MBIR_OK;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t n4 = nl * g.n_theta * acol_width(nb_);
  if (cudaMalloc(&d_acol_, n4 * sizeof(float4)) != cudaSuccess ||
      cudaMalloc(&d_sched_, nl * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&d_lofs_, (nl + 1) * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    dfree_any(d_acol_);
    dfree_any(d_sched_);
    dfree_any(d_lofs_);
    return MBIR_OK;
  }
  const DevTables tab{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_,
                      d_lineok_};
  int rc = launch_acol_f32(dg_, tab, nb_, d_acol_, s);
  if (rc) return cuda_check(rc, "A-column table");
  acol_lo_.clear();
  acol_mask_.clear();
  // host schedules: the footprint bins on the host now
  const size_t per_call = nl / kNumHomogeneous + nl % kNumHomogeneous;
  cwords_ = per_call <= 4096 ? 8 : 16;
  if (p_.call_schedule != 0 || !colour_schedule_fits(g.n_theta, cwords_))
    return host_footprint_bins();
  // device colour schedule: packed bins and scratch
  const size_t n_entries = nl * g.n_theta;
  if (cudaMalloc(&d_packed_, n_entries * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&d_vis_, nl * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&d_conf_, 5 * nl * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&d_colour_, nl * sizeof(int16_t)) != cudaSuccess ||
      cudaMalloc(&d_bin_used_, static_cast<size_t>(g.n_theta) * g.n_r * cwords_ * 8) !=
          cudaSuccess ||
      cudaMalloc(&d_line_used_, nl * cwords_ * 8) != cudaSuccess ||
      cudaMalloc(&d_sched_count_, 2 * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&d_hc_lines_, nl * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&d_hc_lofs_, kNumHomogeneous * lofs_cap() * sizeof(int32_t)) != cudaSuccess ||
      cudaMalloc(&d_hc_count_, kNumHomogeneous * 2 * sizeof(int32_t)) != cudaSuccess) {
    cudaGetLastError();
    dfree_any(d_packed_);
    dfree_any(d_vis_);
    dfree_any(d_conf_);
    dfree_any(d_colour_);
    dfree_any(d_bin_used_);
    dfree_any(d_line_used_);
    dfree_any(d_sched_count_);
    dfree_any(d_hc_lines_);
    dfree_any(d_hc_lofs_);
    dfree_any(d_hc_count_);
    return host_footprint_bins();  // host colouring instead
  }
  // scratch of the multi-CTA colouring (without it the one-CTA form runs)
  const size_t nblk = (nl + 30) / 31;
  if (cudaMalloc(&d_cfsets_, nblk * 31 * cwords_ * 8) != cudaSuccess ||
      cudaMalloc(&d_cflags_, (3 * nblk + 1) * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    dfree_any(d_cfsets_);
    dfree_any(d_cflags_);
  }
  hc_valid_.assign(kNumHomogeneous, 0);
  hc_start_.assign(kNumHomogeneous, 0);
  if ((rc = launch_pack_footprints(d_acol_, n_entries, nb_, d_packed_, s)))
    return cuda_check(rc, "packed bins");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "packed bins");
  return MBIR_OK;
}

// The A-column table's first bins and nonzero masks on the host (acol_lo_, acol_mask_), read
// back from the device table once; used by the host schedules and mbir_get_footprint_bins.
int Engine::host_footprint_bins() {
  if (!acol_lo_.empty() || d_acol_ == nullptr) return MBIR_OK;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t n4 = nl * g.n_theta * acol_width(nb_);
  std::vector<float> host(n4 * 4);
  cudaMemcpyAsync(host.data(), d_acol_, n4 * sizeof(float4), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "A-column table");
  acol_lo_.assign(nl * g.n_theta, 0);
  acol_mask_.assign(nl * g.n_theta, 0);
  acol_bins(host.data(), static_cast<int>(nl), g.n_theta, nb_, acol_lo_.data(), acol_mask_.data());
  return MBIR_OK;
}

// The call's schedule, uploaded for the sweep: colour classes of its conflict graph
// (call_schedule 0; the levels of the row walk when more colours than kMaxColours would be
// needed) or the dependency levels of the row walk (call_schedule 2).  The call's visit order
// (call_lines_) becomes the schedule's line order.  Leaves `a` walking the rows when the engine
// has no A-column table.
int Engine::bf_schedule(const std::vector<int32_t>& rows, SweepArgs& a) {
  const int kMaxColours = 64 * cwords_;
  if (d_acol_ == nullptr) return MBIR_OK;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  // a colour class holds at most as many lines as the kernel has voxel groups
  const int groups = kWarps * (shape_ == 1 ? 2 : 1);
  sched_on_device_ = false;
  if (p_.call_schedule == 0 && d_packed_ != nullptr) {
    int32_t* out_lines = d_sched_;
    int32_t* out_lofs = d_lofs_;
    int32_t* out_count = d_sched_count_;
    bool build = true;
    if (cur_hslot_ >= 0) {  // a homogeneous sub-list: its cached schedule, built the first time
      out_lines = d_hc_lines_ + hc_start_[cur_hslot_];
      out_lofs = d_hc_lofs_ + static_cast<size_t>(cur_hslot_) * lofs_cap();
      out_count = d_hc_count_ + 2 * cur_hslot_;
      build = !hc_valid_[cur_hslot_];
    }
    rb_lines_ = out_lines;
    rb_lofs_ = out_lofs;
    rb_count_ = out_count;
    sched_on_device_ = true;
    a.sched_lines = out_lines;
    a.sched_lofs = out_lofs;
    a.sched_count = out_count;
    a.n_levels = 0;
    a.acol = d_acol_;
    if (!build) return MBIR_OK;
    ColourArgs ca{};
    ca.n_z = g.n_z;
    ca.n_x = g.n_x;
    ca.n_theta = g.n_theta;
    ca.n_r = g.n_r;
    ca.nb = nb_;
    ca.words = cwords_;
    ca.max_colours = 64 * cwords_;
    ca.class_cap = groups;
    ca.packed = d_packed_;
    ca.lineok = d_lineok_;
    ca.active = d_active_;
    // the call's lines (lineok and active), ascending
    vis_host_.clear();
    for (size_t l = 0; l < active_host_.size(); ++l)
      if (active_host_[l] && tab_.line_nonempty[l]) vis_host_.push_back(static_cast<int32_t>(l));
    if (!vis_host_.empty())
      cudaMemcpyAsync(d_vis_, vis_host_.data(), vis_host_.size() * sizeof(int32_t),
                      cudaMemcpyHostToDevice, s);
    ca.vis = d_vis_;
    ca.n = static_cast<int>(vis_host_.size());
    ca.conf = d_conf_;
    ca.conf_p1 = d_conf_ + static_cast<size_t>(g.n_z) * g.n_x;
    ca.conf_p2 = d_conf_ + 2 * static_cast<size_t>(g.n_z) * g.n_x;
    ca.conf_p3 = d_conf_ + 3 * static_cast<size_t>(g.n_z) * g.n_x;
    ca.conf_p4 = d_conf_ + 4 * static_cast<size_t>(g.n_z) * g.n_x;
    ca.colour = d_colour_;
    ca.bin_used = d_bin_used_;
    ca.line_used = d_line_used_;
    ca.lines = out_lines;
    ca.lofs = out_lofs;
    ca.count = out_count;
    ca.err = d_err_;
    // MBIR_COLOUR_SEQUENTIAL=1: every block of the colouring line by line (same schedule; for
    // checking the parallel form)
    const char* seq = std::getenv("MBIR_COLOUR_SEQUENTIAL");
    ca.sequential = (seq != nullptr && seq[0] == '1') ? 1 : 0;
    if (d_cfsets_ != nullptr && d_cflags_ != nullptr) {
      // MBIR_COLOUR_HELPERS: helper CTAs of the multi-CTA colouring (default 8, 0: one CTA)
      const char* hv = std::getenv("MBIR_COLOUR_HELPERS");
      const int helpers = hv ? std::max(0, std::min(64, std::atoi(hv))) : 8;
      const size_t nblk = (static_cast<size_t>(g.n_z) * g.n_x + 30) / 31;
      ca.fsets = d_cfsets_;
      ca.flags = d_cflags_;
      ca.abort_flag = d_cflags_ + 3 * nblk;
      ca.wait_ns = 2000000000ull;
      ca.helpers = helpers;
    }
    cudaEventRecord(static_cast<cudaEvent_t>(ev4_), s);
    const int crc = launch_colour_schedule(ca, s);
    cudaEventRecord(static_cast<cudaEvent_t>(ev5_), s);
    colour_timed_ = crc == 0;
    if (crc) {
      // -1000 - e: CUDA error e pending from an earlier call; -k000 - e: error e at step k
      const int e = crc <= -1000 ? (-crc) % 1000 : 0;
      return fail(MBIR_EDEVICE, "colour schedule: step " + std::to_string(-crc / 1000) + ": " +
                                    (e ? cudaGetErrorString(static_cast<cudaError_t>(e))
                                       : "invalid arguments"));
    }
    if (cur_hslot_ >= 0) hc_valid_[cur_hslot_] = 1;
    return MBIR_OK;
  }
  if (int rc = host_footprint_bins()) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  LevelScheduleIn in{g.n_z, g.n_x, g.n_theta, g.n_r, nb_, stride_, rows.data(),
                     tab_.line_nonempty.data(), active_host_.data(), acol_lo_.data(),
                     acol_mask_.data()};
  int levels = -2;
  if (p_.call_schedule == 0)
    levels = colour_schedule(in, kMaxColours, groups, sched_work_, sched_lines_, sched_lofs_);
  if (levels == -2) levels = level_schedule(in, sched_work_, sched_lines_, sched_lofs_);
  if (levels < 0) return fail(MBIR_EINVAL, "call schedule: invalid row order");
  call_lines_ = sched_lines_;
  sched_ms_ += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                   .count();
  n_levels_ = levels;
  if (!sched_lines_.empty())
    cudaMemcpyAsync(d_sched_, sched_lines_.data(), sizeof(int) * sched_lines_.size(),
                    cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_lofs_, sched_lofs_.data(), sizeof(int) * sched_lofs_.size(),
                  cudaMemcpyHostToDevice, s);
  a.sched_lines = d_sched_;
  a.sched_lofs = d_lofs_;
  a.n_levels = levels;
  a.acol = d_acol_;
  return MBIR_OK;
}

// The lines of one updateVoxels call (BFReconstructionEngine.cpp:610-646 and
// BFReconstructionEngine_Extra.cpp:576-628): without NHICD every line; with NHICD the even
// calls take the next 1/20 of the master permutation (the last sublist takes the remainder),
// the odd calls the lines whose VSC-filtered update magnitude exceeds the order statistic at
// N - N/20.  Uploads the active mask and clears the calls' line magnitudes.
int Engine::bf_call_begin(int outer, int inner, DevBF* out) {
  (void)outer;
  (void)inner;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const int nl = g.n_z * g.n_x;
  std::vector<int32_t> list;
  cur_hslot_ = -1;
  if (!p_.nhicd) {
    list = bf_master_;
  } else if (bf_eff_ % 2 == 0) {
    bf_listsel_ %= kNumHomogeneous;
    int n_el = static_cast<int>(std::floor(static_cast<double>(nl) / kNumHomogeneous));
    if (bf_listsel_ == kNumHomogeneous - 1) n_el += nl - n_el * kNumHomogeneous;
    const int start = static_cast<int>(std::floor(static_cast<double>(nl) / kNumHomogeneous) *
                                       bf_listsel_);
    list.assign(bf_master_.begin() + start, bf_master_.begin() + start + n_el);
    if (!hc_valid_.empty()) {
      cur_hslot_ = static_cast<int>(bf_listsel_);
      hc_start_[cur_hslot_] = start;
    }
    bf_listsel_++;
  } else {
    // ComputeVSC + SetNonHomThreshold + GenNonHomList (_Extra.cpp:888-1047)
    int rc = launch_bf_vsc(d_mag_, d_filt_, g.n_z, g.n_x, s);
    if (rc) return cuda_check(rc, "VSC filter");
    std::vector<double> filt(nl);
    cudaMemcpyAsync(filt.data(), d_filt_, sizeof(double) * nl, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "VSC read");
    std::vector<double> tmp = filt;
    size_t k = static_cast<size_t>(nl) - static_cast<size_t>(nl) / kNumNonHomogeneous;
    if (k >= static_cast<size_t>(nl)) k = nl - 1;
    std::nth_element(tmp.begin(), tmp.begin() + k, tmp.end());
    const double thr = tmp[k];
    for (int l = 0; l < nl; l++)
      if (filt[l] > thr) list.push_back(l);
  }
  if (p_.order_mode == MBIR_ORDER_REFERENCE) {
    // the call's visit order: the worker's GenRandList of its list (one worker,
    // BFReconstructionEngine_Extra.cpp:691).  A non-homogeneous list was already shuffled once
    // by GenNonHomList (:1044); the reference seeds both from its millisecond clock, which
    // gives both the same seed, so the same permutation is applied twice.
    const uint32_t call_seed =
        p_.seed_mode == MBIR_SEED_FIXED ? p_.seed : p_.seed + 1u + static_cast<uint32_t>(bf_calls_);
    std::vector<int32_t> perm;
    rand_list_perm(call_seed, static_cast<int>(list.size()), perm);
    call_lines_.assign(list.size(), 0);
    if (p_.nhicd && bf_eff_ % 2 == 1) {
      for (size_t i = 0; i < list.size(); i++) call_lines_[perm[i]] = list[i];
      list = call_lines_;
    }
    for (size_t i = 0; i < list.size(); i++) call_lines_[perm[i]] = list[i];
  } else {
    call_lines_ = list;
    std::sort(call_lines_.begin(), call_lines_.end());
  }
  active_host_.assign(nl, 0);
  for (int32_t l : list) active_host_[l] = 1;
  cudaMemcpyAsync(d_active_, active_host_.data(), nl, cudaMemcpyHostToDevice, s);
  int rc = launch_bf_mag_reset(d_magfx_, d_active_, nl, s);
  if (rc) return cuda_check(rc, "magnitude reset");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "call setup");
  if (out) {
    out->w = d_w_;
    out->sel = d_sel_;
    out->n_sp = n_sp_;
    out->active = d_active_;
    out->mag_fx = d_magfx_;
    out->bragg_t = bragg_t_;
    out->bragg_dt = p_.bragg_delta * bragg_t_;
  }
  return MBIR_OK;
}

// The device schedule's lines, offsets and counts, copied to the host behind the call (the
// caller synchronises the stream before bf_schedule_settle).
void Engine::bf_schedule_readback() {
  readback_pending_ = false;
  if (!sched_on_device_) return;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  size_t n_call = 0;
  for (size_t l = 0; l < active_host_.size(); ++l)
    n_call += (active_host_[l] && tab_.line_nonempty[l]) ? 1 : 0;
  call_lines_.assign(n_call, 0);
  sched_lofs_.assign(lofs_cap(), 0);
  if (n_call)
    cudaMemcpyAsync(call_lines_.data(), rb_lines_, n_call * sizeof(int32_t),
                    cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(sched_lofs_.data(), rb_lofs_, sched_lofs_.size() * sizeof(int32_t),
                  cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(sched_count_host_, rb_count_, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  readback_pending_ = true;
}

// colours <= lines, so a call's colour offsets fit in min(max colours, lines) + 1 values
size_t Engine::lofs_cap() const {
  return std::min<size_t>(64 * cwords_, static_cast<size_t>(g_.n_z) * g_.n_x) + 1;
}

void Engine::bf_schedule_settle() {
  if (colour_timed_) {
    colour_timed_ = false;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev4_),
                             static_cast<cudaEvent_t>(ev5_)) == cudaSuccess)
      colour_ms_ += ms;
  }
  if (!readback_pending_) return;
  readback_pending_ = false;
  n_levels_ = sched_count_host_[1];
  if (sched_count_host_[0] >= 0 && static_cast<size_t>(sched_count_host_[0]) <= call_lines_.size())
    call_lines_.resize(static_cast<size_t>(sched_count_host_[0]));
  sched_lofs_.resize(static_cast<size_t>(std::max(n_levels_, 0)) + 1);
  sched_lines_ = call_lines_;
}

int Engine::bf_call_end() {
  bf_schedule_readback();
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const int nl = g_.n_z * g_.n_x;
  if (!exact_) {
    int rc = launch_bf_mag_update(d_magfx_, d_active_, d_mag_, nl, s);
    if (rc) return cuda_check(rc, "magnitude map");
  }
  bf_calls_++;
  bf_eff_++;
  return MBIR_OK;
}

// One updateVoxels call: lines of the call in the GPU slice order (parallel) or in the call's
// visit order with y ascending (reference order).
int Engine::bf_call(int outer, int inner, double* st4) {
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const int iter_nonzero = (inner > 0 || outer > 0) ? 1 : 0;
  DevBF bfa{};
  int rc = bf_call_begin(outer, inner, &bfa);
  if (rc) return rc;
  cudaEventRecord(static_cast<cudaEvent_t>(ev0_), s);
  if (p_.order_mode == MBIR_ORDER_REFERENCE) {
    cudaMemcpyAsync(d_lines_, call_lines_.data(), sizeof(int32_t) * call_lines_.size(),
                    cudaMemcpyHostToDevice, s);
    if (exact_) {
      ExactArgs ea = exact_args();
      ea.lines = d_lines_;
      ea.n_lines = static_cast<int>(call_lines_.size());
      ea.iter_nonzero = iter_nonzero;
      ea.zero_skipping = p_.zero_skipping;
      ea.stats = d_stat4_;
      ea.bf = 1;
      ea.bw = static_cast<const double*>(d_w_);
      ea.bsel = d_sel_;
      ea.n_sp = n_sp_;
      ea.bragg_t = bragg_t_;
      ea.bragg_delta = p_.bragg_delta;
      ea.mag = d_mag_;
      if ((rc = launch_exact_icd(ea, s))) return cuda_check(rc, "BF call (exact)");
    } else {
      RefOrderArgs a{};
      a.g = dg_;
      a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_,
                        d_lineok_};
      a.flt = flt_;
      a.x = d_x_;
      a.e = d_e_;
      a.lines = d_lines_;
      a.n_lines = static_cast<int>(call_lines_.size());
      a.iter_nonzero = iter_nonzero;
      a.zero_skipping = p_.zero_skipping;
      a.fp64 = fp64_;
      a.bf = 1;
      a.bfa = bfa;
      a.stats = d_stat4_;
      if ((rc = launch_ref_order(a, nb_, s))) return cuda_check(rc, "BF call (reference order)");
    }
  } else {
    SweepArgs a{};
    size_t smem = 0;
    if ((rc = bf_parallel_args(iter_nonzero, bfa, &a, &smem))) return rc;
    const int n0 = (g.n_y + 1) / 2;
    cudaEventRecord(static_cast<cudaEvent_t>(ev2_), s);
    for (int colour = 0; colour < 2; colour++) {
      a.colour = colour;
      a.n_slices = (g.n_y - colour + 1) / 2;
      a.stats = d_stats_ + (colour ? static_cast<size_t>(n0) * kStatSlots : 0);
      if (a.n_slices <= 0) continue;
      if ((rc = launch_sweep(a, nb_, smem, s))) return cuda_check(rc, "BF call launch");
    }
    cudaEventRecord(static_cast<cudaEvent_t>(ev3_), s);
    kernel_timed_ = true;
    if ((rc = launch_reduce_stats(d_stats_, g.n_y, kStatSlots, d_stat4_, s)))
      return cuda_check(rc, "stats reduce");
  }
  cudaEventRecord(static_cast<cudaEvent_t>(ev1_), s);
  if ((rc = bf_call_end())) return rc;
  double st[kStatSlots];
  cudaMemcpyAsync(st, d_stat4_, sizeof(st), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "BF call");
  bf_schedule_settle();
  if ((rc = check_device_error())) return rc;
  float ms = 0;
  cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev0_), static_cast<cudaEvent_t>(ev1_));
  icd_ms_ += ms;
  add_kernel_time();
  sweeps_done_++;
  visited_ += static_cast<int64_t>(st[2] + st[3]);
  updated_ += static_cast<int64_t>(st[3]);
  last_rel_ = st[1] > 0 ? st[0] / st[1] : 0.0;
  outer_ = outer;
  inner_ = inner;
  if (st4)
    for (int i = 0; i < 4; i++) st4[i] = st[i];
  return MBIR_OK;
}

// The launch arguments of a parallel-order call (the call's lines already chosen): row order
// of this sweep, the call's schedule (device colouring or dependency levels, or none for the
// row walk) and the launch's shared memory.
int Engine::bf_parallel_args(int iter_nonzero, const DevBF& bfa, SweepArgs* out, size_t* smem_out) {
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc;
  std::vector<int32_t> rows;
  row_order_for_sweep(sweeps_done_, rows);
  cudaMemcpyAsync(d_rows_, rows.data(), sizeof(int) * g.n_z, cudaMemcpyHostToDevice, s);
  SweepArgs& a = *out;
  a = SweepArgs{};
  a.g = dg_;
  a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_,
                    d_lineok_};
  a.flt = flt_;
  a.x = d_x_;
  a.e = d_e_;
  a.row_order = d_rows_;
  a.stride = stride_;
  a.mode = kModeICD;
  a.fp64 = fp64_;
  a.bf = 1;
  a.bfa = bfa;
  a.iter_nonzero = iter_nonzero;
  a.zero_skipping = p_.zero_skipping;
  a.smem_rows = stage_ ? 1 : 0;
  a.n_rs = stage_ ? n_rs_ : 0;
  a.err = d_err_;
  a.shape = shape_;
  if ((rc = bf_schedule(rows, a))) return rc;
  size_t smem = a.sched_lines != nullptr ? smem_sched_bytes_ : smem_bytes_;
  if (a.sched_lines != nullptr) {
    // room for the schedule itself (offsets and lines) after the layout, when it fits: the
    // class steps then read it from shared memory
    const size_t limit = static_cast<size_t>(smem_optin_limit()) - 2048;
    const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
    const size_t lines = p_.nhicd ? nl / kNumHomogeneous + kNumHomogeneous : nl;
    const size_t room = (lofs_cap() + 1 + lines) * sizeof(int);
    if (smem + room <= limit) smem += room;
  }
  *smem_out = smem;
  return MBIR_OK;
}

// BFForwardModel::jointEstimation (BFForwardModel.cpp:390-441) followed by updateSelector, as
// execute() pairs them (BFReconstructionEngine.cpp:836-838)
int Engine::bf_joint_estimation() {
  const int nt = g_.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const BfSino b = bf_sino();
  int rc = launch_bf_offset_sums(b, exact_ ? 1 : 0, bragg_t_, p_.bragg_delta, d_partial_,
                                 n_chunk_, d_vsum_, s);
  if (rc) return cuda_check(rc, "offset sums");
  std::vector<double> vs(static_cast<size_t>(nt) * 2), step(nt);
  cudaMemcpyAsync(vs.data(), d_vsum_, sizeof(double) * vs.size(), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "offset sums");
  for (int v = 0; v < nt; v++) {
    step[v] = vs[v * 2 + 0] / vs[v * 2 + 1];
    mu_[v] += step[v];
  }
  cudaMemcpyAsync(d_mu2_, step.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  if ((rc = launch_bf_offset_apply(b, d_mu2_, s))) return cuda_check(rc, "offset apply");
  if ((rc = launch_bf_selector(b, bragg_t_, s))) return cuda_check(rc, "selector");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "offset step");
  return upload_views();
}

// BFForwardModel::updateWeights (BFForwardModel.cpp:447-511) followed by updateSelector
// (BFReconstructionEngine.cpp:850-851)
int Engine::bf_update_weights() {
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const BfSino b = bf_sino();
  cudaMemcpyAsync(d_alpha_, alpha_.data(), sizeof(double) * g.n_theta, cudaMemcpyHostToDevice, s);
  int rc = launch_bf_variance_sums(b, exact_ ? 1 : 0, d_alpha_, d_bfpart_, d_bfout_, s);
  if (rc) return cuda_check(rc, "variance sums");
  double sums[2];
  cudaMemcpyAsync(sums, d_bfout_, sizeof(sums), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "variance sums");
  const double upd = (sums[0] + (p_.bragg_delta * bragg_t_) * sums[1]) /
                     (g.n_theta * g.n_r * g.n_t);
  for (int v = 0; v < g.n_theta; v++) alpha_[v] = upd;
  if ((rc = launch_bf_scale_weights(b, upd, s))) return cuda_check(rc, "weight scale");
  if ((rc = launch_bf_selector(b, bragg_t_, s))) return cuda_check(rc, "selector");
  cudaMemcpyAsync(d_alpha_, alpha_.data(), sizeof(double) * g.n_theta, cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "variance");
  return MBIR_OK;
}

// BFReconstructionEngine::computeCost (BFReconstructionEngine.cpp:1084-1097): forwardCost
// (data term over selected / rejected entries, halved, plus (N/2) log(alpha_0) with the
// reference's integer N/2) + QGGMRF::PriorModelCost
int Engine::bf_compute_cost(double* parts3, double* total) {
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc = launch_bf_cost_sums(bf_sino(), exact_ ? 1 : 0, bragg_t_, p_.bragg_delta, d_bfpart_,
                               d_bfout_, s);
  if (rc) return cuda_check(rc, "BF data term");
  double* prior_partial = d_partial_ + static_cast<size_t>(g.n_theta) * n_chunk_ * 6;
  rc = launch_prior_cost(d_x_, flt_, g.n_z, g.n_x, g.n_y, prior_partial, prior_blocks_, fp64_, s);
  if (rc) return cuda_check(rc, "cost prior term");
  double data = 0;
  std::vector<double> pp(prior_blocks_);
  cudaMemcpyAsync(&data, d_bfout_, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(pp.data(), prior_partial, sizeof(double) * prior_blocks_, cudaMemcpyDeviceToHost,
                  s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "BF cost");
  data /= 2;
  double prior = 0;
  for (double v : pp) prior += v;
  double noise = 0;
  if (p_.noise_estimation)
    noise = static_cast<double>((g.n_theta * g.n_r * g.n_t) / 2) * std::log(alpha_[0]);
  if (parts3) {
    parts3[0] = data;
    parts3[1] = prior;
    parts3[2] = noise;
  }
  last_cost_ = data + noise + prior;
  if (total) *total = last_cost_;
  return MBIR_OK;
}

int Engine::bf_roi_sum(int kind, double* out) {
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc = launch_roi_sum(dg_, exact_ ? 1 : 0, kind, d_mag_, d_x_, fp64_, d_bfpart_, d_bfout_, s);
  if (rc) return cuda_check(rc, "ROI sum");
  cudaMemcpyAsync(out, d_bfout_, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "ROI sum");
  return MBIR_OK;
}

// BFReconstructionEngine::execute outer/inner loops (BFReconstructionEngine.cpp:595-858):
// the Bragg threshold starts at DefBraggThreshold while the first outer iteration's inner
// calls run (when there is more than one) and is set to the requested T after them; the stop
// rule compares the ROI sum of the update-magnitude map with the ROI volume sum of the previous
// equivalent iteration (stopCriteria, _Extra.cpp:1217-1273); JE and variance updates follow
// each outer iteration when there is more than one.
int Engine::bf_run() {
  const int nl = g_.n_z * g_.n_x;
  (void)nl;
  int num_iter = p_.inner_iterations;
  double des_t = 0, temp_t;
  if (num_iter > 1) {
    des_t = p_.bragg_threshold;
    temp_t = kDefBragg;
  } else {
    temp_t = p_.bragg_threshold;
  }
  bragg_t_ = temp_t;
  double prev_mag = 0, stop = p_.stop_threshold;
  int rc;
  for (int outer = 0; outer < p_.outer_iterations; outer++) {
    if (outer > 0) {
      num_iter = 1;
      bragg_t_ = temp_t;
    }
    int status = 1;
    for (int inner = 0; inner < num_iter; inner++) {
      if (num_iter > 1 && inner == 0) bragg_t_ = kDefBragg;
      const uint32_t eff = bf_eff_;
      double st[4];
      if ((rc = bf_call(outer, inner, st))) return rc;
      if (p_.cost_every_sweep && (rc = bf_compute_cost(nullptr, nullptr))) return rc;
      status = 1;
      const bool check = p_.nhicd ? (eff % kNumNonHomogeneous == 0) : true;
      if (check && eff > 0 && prev_mag > 0) {
        double mag_sum = 0;
        if ((rc = bf_roi_sum(0, &mag_sum))) return rc;
        if (std::fabs(mag_sum) / std::fabs(prev_mag) < stop) {
          stop *= p_.threshold_reduction_factor;
          status = 0;
        }
      }
      if (!p_.nhicd || eff % kNumNonHomogeneous == 0)
        if ((rc = bf_roi_sum(1, &prev_mag))) return rc;
      if (cancel_.load()) return fail(MBIR_ECANCELLED, "cancelled");
      if (status == 0) break;
      if (inner == num_iter - 1 && inner != 0) {
        temp_t = des_t;
        bragg_t_ = temp_t;
      }
    }
    if (status == 0 && outer >= 1) {
      notify_iteration(outer);
      break;
    }
    if (p_.outer_iterations > 1) {
      if (p_.joint_estimation && (rc = bf_joint_estimation())) return rc;
      if (p_.noise_estimation && (rc = bf_update_weights())) return rc;
    }
    notify_iteration(outer);
  }
  return MBIR_OK;
}

int Engine::get_call_schedule(int32_t* lines, int32_t cap, int32_t* lofs, int32_t lofs_cap,
                              int32_t* n_lines, int32_t* n_levels) const {
  const bool sched = !sched_lofs_.empty() && n_levels_ > 0;
  const size_t nlev = sched ? sched_lofs_.size() - 1 : 0;
  if (n_lines) *n_lines = sched ? static_cast<int32_t>(sched_lines_.size()) : 0;
  if (n_levels) *n_levels = static_cast<int32_t>(nlev);
  if (!sched) return MBIR_OK;
  if (lines) {
    if (cap < static_cast<int32_t>(sched_lines_.size())) return MBIR_EINVAL;
    std::copy(sched_lines_.begin(), sched_lines_.end(), lines);
  }
  if (lofs) {
    if (lofs_cap < static_cast<int32_t>(sched_lofs_.size())) return MBIR_EINVAL;
    std::copy(sched_lofs_.begin(), sched_lofs_.end(), lofs);
  }
  return MBIR_OK;
}

int Engine::get_footprint_bins(int16_t* lo, uint16_t* mask, uint8_t* lineok) const {
  if (state_ < 2) return MBIR_ESTATE;
  int rc = const_cast<Engine*>(this)->host_footprint_bins();
  if (rc) return rc;
  if (acol_lo_.empty()) return MBIR_ENOTSUP;
  if (lo) std::copy(acol_lo_.begin(), acol_lo_.end(), lo);
  if (mask) std::copy(acol_mask_.begin(), acol_mask_.end(), mask);
  if (lineok) std::copy(tab_.line_nonempty.begin(), tab_.line_nonempty.end(), lineok);
  return MBIR_OK;
}

int Engine::get_call_lines(int32_t* lines, int32_t cap, int32_t* n) const {
  if (n) *n = static_cast<int32_t>(call_lines_.size());
  if (lines) {
    if (cap < static_cast<int32_t>(call_lines_.size())) return MBIR_EINVAL;
    std::copy(call_lines_.begin(), call_lines_.end(), lines);
  }
  return MBIR_OK;
}

int Engine::get_bf_state(uint8_t* sel, float* w, double* mag, double* filt, double* bragg) {
  if (state_ < 2) return fail(MBIR_ESTATE, "get_bf_state: call prepare first");
  if (!bf_) return fail(MBIR_EINVAL, "get_bf_state: not a bright-field engine");
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
  if (bragg) *bragg = bragg_t_;
  if (mag) cudaMemcpyAsync(mag, d_mag_, sizeof(double) * nl, cudaMemcpyDeviceToHost, s);
  if (filt) cudaMemcpyAsync(filt, d_filt_, sizeof(double) * nl, cudaMemcpyDeviceToHost, s);
  if (w) {
    int rc = launch_sino_to_host(d_w_, d_stage_, g.n_theta, g.n_r, n_rp_, g.n_t, fp64_, s);
    if (rc) return cuda_check(rc, "weights read-out");
    cudaMemcpyAsync(w, d_stage_, sizeof(float) * g.n_theta * g.n_r * g.n_t, cudaMemcpyDeviceToHost,
                    s);
  }
  if (sel) {
    std::vector<uint8_t> dev(static_cast<size_t>(g.n_t) * g.n_theta * n_sp_);
    cudaMemcpyAsync(dev.data(), d_sel_, dev.size(), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "selector");
    for (int th = 0; th < g.n_theta; th++)
      for (int r = 0; r < g.n_r; r++)
        for (int t = 0; t < g.n_t; t++)
          sel[(static_cast<size_t>(th) * g.n_r + r) * g.n_t + t] =
              dev[(static_cast<size_t>(t) * g.n_theta + th) * n_sp_ + r];
  }
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK : cuda_check(MBIR_EDEVICE, "BF state");
}

int Engine::set_bragg_threshold(double t) {
  if (!(t > 0)) return fail(MBIR_EINVAL, "Bragg threshold must be > 0");
  bragg_t_ = t;
  return MBIR_OK;
}

}  // namespace mbir
