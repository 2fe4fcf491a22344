// mbir_engine.cu -- host orchestration of one reconstruction on one GB300.
//
// The host code derives geometry and lookup tables in FP64 exactly as the reference does
// (these are O(n_theta * bins) setup values), then keeps every per-voxel and per-measurement
// array in HBM and drives the sm_103a kernels of mbir_kernels.cu.  The small per-view solves
// (Lagrange-constrained gains, variances: n_theta values) run on the host in FP64 from
// FP64 device reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>

#include "mbir_engine.h"

namespace mbir {

namespace {
constexpr double kPi = 3.14159265358979323846;

// prior weights [dy+1][dz+1][dx+1] (HAADF_ReconstructionEngine.cpp:266-294)
constexpr double kFilter[27] = {0.0302, 0.0370, 0.0302, 0.0370, 0.0523, 0.0370, 0.0302,
                                0.0370, 0.0302, 0.0370, 0.0523, 0.0370, 0.0523, 0.0000,
                                0.0523, 0.0370, 0.0523, 0.0370, 0.0302, 0.0370, 0.0302,
                                0.0370, 0.0523, 0.0370, 0.0302, 0.0370, 0.0302};

template <typename T>
int dmalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T)) == cudaSuccess ? 0 : MBIR_ENOMEM;
}
int dmalloc_bytes(void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  return cudaMalloc(p, bytes) == cudaSuccess ? 0 : MBIR_ENOMEM;
}
template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}
}  // namespace

// ---- MT19937 ------------------------------------------------------------------------------
void MT19937::seed(uint32_t s) {
  mt_[0] = s;
  for (int i = 1; i < 624; i++) mt_[i] = 1812433253u * (mt_[i - 1] ^ (mt_[i - 1] >> 30)) + i;
  idx_ = 624;
}
uint32_t MT19937::next() {
  if (idx_ >= 624) {
    for (int i = 0; i < 624; i++) {
      const uint32_t y = (mt_[i] & 0x80000000u) | (mt_[(i + 1) % 624] & 0x7fffffffu);
      mt_[i] = mt_[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    idx_ = 0;
  }
  uint32_t y = mt_[idx_++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

void reference_visit_order(uint32_t seed, int n_z, int n_x, std::vector<int32_t>& out) {
  int size = n_z * n_x;
  std::vector<int32_t> counter(size);
  for (int j = 0; j < size; j++) counter[j] = j;
  MT19937 gen(seed);
  out.clear();
  out.reserve(size);
  for (int j = 0; j < n_z; j++)
    for (int k = 0; k < n_x; k++) {
      const uint32_t index = gen.next() % static_cast<uint32_t>(size);
      out.push_back(counter[index]);
      counter[index] = counter[size - 1];
      size--;
    }
}

// ---- Engine -------------------------------------------------------------------------------
Engine::Engine(const mbir_params& p) : p_(p) {
  if (p_.qggmrf_q == 0.0) p_.qggmrf_q = p_.diffuseness + 1.0;
  fp64_ = p_.precision == MBIR_PRECISION_FP64 ? 1 : 0;
  exact_ = fp64_ && p_.order_mode == MBIR_ORDER_REFERENCE;
  bf_ = p_.modality == MBIR_MODALITY_BF;
  rb_ = fp64_ ? sizeof(double) : sizeof(float);
  bins_ = p_.detector_response_bins > 0 ? p_.detector_response_bins : 64;
}

Engine::~Engine() { release(); }

void Engine::release() {
  dfree(d_y_);
  dfree(d_e_);
  dfree(d_yest_);
  dfree(d_x_);
  dfree(d_stage_);
  dfree(d_H_);
  dfree(d_bx_);
  dfree(d_bxd_);
  dfree(d_u0_);
  dfree(d_bz_);
  dfree(d_gw_);
  dfree(d_tfirst_);
  dfree(d_tcount_);
  dfree(d_hval_);
  dfree(d_rows_);
  dfree(d_lineok_);
  dfree(d_cosv_);
  dfree(d_sinv_);
  dfree(d_Href_);
  dfree(d_lines_);
  dfree(d_stats_);
  dfree(d_stat4_);
  dfree(d_mu_);
  dfree(d_gain_);
  dfree(d_mu2_);
  dfree(d_gain2_);
  dfree(d_wv_);
  dfree(d_partial_);
  dfree(d_vsum_);
  dfree(d_err_);
  dfree(d_w_);
  dfree(d_sel_);
  dfree(d_magfx_);
  dfree(d_mag_);
  dfree(d_filt_);
  dfree(d_active_);
  dfree(d_bfpart_);
  dfree(d_bfout_);
  dfree(d_alpha_);
  dfree(d_stage64_);
  dfree(d_acol_);
  dfree(d_sched_);
  dfree(d_lofs_);
  dfree(d_packed_);
  dfree(d_vis_);
  dfree(d_conf_);
  dfree(d_colour_);
  dfree(d_bin_used_);
  dfree(d_line_used_);
  dfree(d_cfsets_);
  dfree(d_cflags_);
  dfree(d_sched_count_);
  dfree(d_hc_lines_);
  dfree(d_hc_lofs_);
  dfree(d_hc_count_);
  hc_valid_.clear();
  acol_lo_.clear();
  acol_mask_.clear();
  if (ev0_) cudaEventDestroy(static_cast<cudaEvent_t>(ev0_));
  if (ev1_) cudaEventDestroy(static_cast<cudaEvent_t>(ev1_));
  if (ev2_) cudaEventDestroy(static_cast<cudaEvent_t>(ev2_));
  if (ev3_) cudaEventDestroy(static_cast<cudaEvent_t>(ev3_));
  if (ev4_) cudaEventDestroy(static_cast<cudaEvent_t>(ev4_));
  if (ev5_) cudaEventDestroy(static_cast<cudaEvent_t>(ev5_));
  if (stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
  ev0_ = ev1_ = ev2_ = ev3_ = ev4_ = ev5_ = stream_ = nullptr;
}

// device time of the colour launches of the last sweep/call (events ev2_ -> ev3_)
void Engine::add_kernel_time() {
  if (!kernel_timed_) return;
  kernel_timed_ = false;
  float ms = 0;
  if (cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev2_), static_cast<cudaEvent_t>(ev3_)) ==
      cudaSuccess)
    kernel_ms_ += ms;
}

int Engine::fail(int code, const std::string& msg) {
  err_ = msg;
  if (p_.verbose) std::fprintf(stderr, "mbir: %s\n", msg.c_str());
  notify(err_, 100, MBIR_UPDATE_ERROR_MESSAGE);
  return code;
}

void Engine::notify(const std::string& msg, int progress, int aspect) const {
  if (observer_) observer_(msg.c_str(), progress, aspect, observer_user_);
}

// The run's metrics after outer iteration `outer`, as one JSON object: sweeps (ICD calls) so
// far, the last sweep's sum|dx| / sum|x| over the ROI, the last FP64 cost (null when none was
// computed), voxel updates and ICD device time so far
void Engine::notify_iteration(int outer) const {
  if (!observer_) return;
  char cost[40] = "null";
  if (std::isfinite(last_cost_)) std::snprintf(cost, sizeof cost, "%.17g", last_cost_);
  char buf[320];
  std::snprintf(buf, sizeof buf,
                "{\"outer\": %d, \"sweeps\": %d, \"rel_update\": %.9g, \"cost\": %s, "
                "\"voxels_updated\": %lld, \"icd_ms\": %.3f}",
                outer, sweeps_done_, last_rel_, cost, static_cast<long long>(updated_), icd_ms_);
  const int n = std::max(1, p_.outer_iterations);
  notify(buf, std::min(100, 100 * (outer + 1) / n), MBIR_UPDATE_PROGRESS_MESSAGE);
}

int Engine::cuda_check(int code, const char* what) {
  if (code == 0) return 0;
  cudaError_t e = cudaGetLastError();
  std::ostringstream ss;
  ss << what << ": " << (e != cudaSuccess ? cudaGetErrorString(e) : "failed");
  return fail(code == MBIR_ENOMEM ? MBIR_ENOMEM : (code == -7 ? MBIR_ENOTSUP : MBIR_EDEVICE),
              ss.str());
}

int Engine::set_sinogram(const float* counts, const float* tilts_deg, int n_theta, int n_r,
                         int n_t, double delta_r, double delta_t) {
  if (!counts || !tilts_deg || n_theta <= 0 || n_r <= 0 || n_t <= 0 || !(delta_r > 0) ||
      !(delta_t > 0))
    return fail(MBIR_EINVAL, "set_sinogram: bad arguments");
  if (n_theta > 32 * kMaxViewsPerLane)
    return fail(MBIR_ENOTSUP, "set_sinogram: more than 256 views");
  if (n_r > 65535 || n_t > 65535) return fail(MBIR_EINVAL, "set_sinogram: detector too large");
  g_ = Geometry();
  g_.n_theta = n_theta;
  g_.n_r = n_r;
  g_.n_t = n_t;
  g_.delta_r = delta_r;
  g_.delta_t = delta_t;
  counts_.assign(counts, counts + static_cast<size_t>(n_theta) * n_r * n_t);
  bfm_.clear();
  tilts_.resize(n_theta);
  for (int i = 0; i < n_theta; i++) tilts_[i] = tilts_deg[i];
  if (state_ >= 2) release();
  state_ = 1;
  host_ready_ = false;
  return MBIR_OK;
}

// initializeBrightFieldData (HAADF_ReconstructionEngine_Extra.cpp:84-176): a bright-field tilt
// series of the sinogram's size; each count plus BF_OFFSET (HAADFConstants.h:49) becomes the
// measurement's factor m.  HAADF only, before prepare.
int Engine::set_bright_field(const float* counts, int n_theta, int n_r, int n_t) {
  if (state_ < 1) return fail(MBIR_ESTATE, "set_bright_field: set the sinogram first");
  if (state_ >= 2) return fail(MBIR_ESTATE, "set_bright_field: before prepare");
  if (bf_) return fail(MBIR_EINVAL, "set_bright_field: HAADF reconstructions only");
  if (!counts) return fail(MBIR_EINVAL, "set_bright_field: null counts");
  if (n_theta != g_.n_theta || n_r != g_.n_r || n_t != g_.n_t)
    return fail(MBIR_EINVAL, "set_bright_field: The two file sizes are not matched");
  const size_t n = static_cast<size_t>(n_theta) * n_r * n_t;
  constexpr double kBfOffset = 32768.0;  // BF_OFFSET
  bfm_.resize(n);
  for (size_t i = 0; i < n; i++) bfm_[i] = static_cast<double>(counts[i]) + kBfOffset;
  return MBIR_OK;
}

// --initial_recon_file (InitialReconstructionBinReader.cpp:73-135): the starting volume, as
// doubles (the reference hands levels the doubles of ReconstructedObject.bin)
template <typename T>
int Engine::set_initial_volume_t(const T* vol, int64_t n) {
  if (!vol || n <= 0) return fail(MBIR_EINVAL, "set_initial_volume: bad arguments");
  if (!p_.interpolate_initial_recon) {
    init_vol_.assign(vol, vol + n);
    host_ready_ = false;
    return MBIR_OK;
  }
  // --interpolate_initial_recon (InitialReconstructionBinReader.cpp:101-131): the given volume
  // has half the voxels along each axis ([z][x][y] of N_z/2 x N_x/2 x N_y/2, integer halves);
  // each value fills its 2x2x2 block and the rest of the volume starts at zero
  if (state_ < 1) return fail(MBIR_ESTATE, "set_initial_volume: set the sinogram first");
  if (g_.n_y == 0) {
    int rc = build_geometry();
    if (rc) return rc;
  }
  const int hz = g_.n_z / 2, hx = g_.n_x / 2, hy = g_.n_y / 2;
  if (n != static_cast<int64_t>(hz) * hx * hy)
    return fail(MBIR_EINVAL, "set_initial_volume: the interpolated initial volume must hold "
                             "(N_z/2) x (N_x/2) x (N_y/2) voxels");
  init_vol_.assign(static_cast<size_t>(g_.n_z) * g_.n_x * g_.n_y, 0.0);
  for (int z = 0; z < hz; z++)
    for (int x = 0; x < hx; x++)
      for (int y = 0; y < hy; y++) {
        const double b = vol[(static_cast<size_t>(z) * hx + x) * hy + y];
        for (int a = 0; a < 2; a++)
          for (int c = 0; c < 2; c++)
            for (int r = 0; r < 2; r++)
              init_vol_[(static_cast<size_t>(2 * z + a) * g_.n_x + 2 * x + c) * g_.n_y + 2 * y +
                        r] = b;
      }
  host_ready_ = false;
  return MBIR_OK;
}

int Engine::set_initial_volume(const float* vol, int64_t n) {
  return set_initial_volume_t(vol, n);
}
int Engine::set_initial_volume_f64(const double* vol, int64_t n) {
  return set_initial_volume_t(vol, n);
}

int Engine::set_initial_nuisance(const double* g, const double* o, const double* v) {
  const int nt = g_.n_theta;
  if (state_ < 1) return fail(MBIR_ESTATE, "set_initial_nuisance: set the sinogram first");
  if (g) user_gain_.assign(g, g + nt);
  if (o) user_offset_.assign(o, o + nt);
  if (v) user_var_.assign(v, v + nt);
  host_ready_ = false;
  return MBIR_OK;
}

int Engine::build_geometry() {
  Geometry& g = g_;
  g.R0 = -(g.n_r * g.delta_r) / 2;
  g.RMax = (g.n_r * g.delta_r) / 2;
  g.T0 = -(g.n_t * g.delta_t) / 2;
  g.TMax = (g.n_t * g.delta_t) / 2;
  // HAADF_MultiResolutionReconstruction.cpp:233,349-350: interpolateFactor is the coarsest
  // voxel multiple; level i uses delta_xz = 2^(levels-1-i) * final_resolution detector pixels.
  const int levels = std::max(p_.num_resolutions, 1);
  const int lvl = (p_.level < 0 || p_.level >= levels) ? levels - 1 : p_.level;
  const double fres = std::max(p_.final_resolution, 1);
  const double interp = std::pow(2.0, levels - 1) * fres;
  g.delta_xz = g.delta_r * (std::pow(2.0, levels - 1 - lvl) * fres);
  g.delta_xy = g.delta_xz;
  double mx = 0;
  for (double a : tilts_) mx = std::max(mx, std::fabs(a));
  if (mx > 75.0) mx = 75.0;
  mx = mx * kPi / 180.0;
  double lz = p_.sample_thickness * p_.z_stretch;
  lz /= (interp * g.delta_r);
  lz = std::floor(lz + 0.5) * interp * g.delta_r;
  g.length_z = lz;
  g.length_x = g.n_r * g.delta_r;
  if (p_.extend_object) {
    double lx = p_.x_shrink_factor * ((g.n_r * g.delta_r) / std::cos(mx)) + lz * std::tan(mx);
    lx /= (interp * g.delta_r);
    g.length_x = std::floor(lx + 0.5) * interp * g.delta_r;
  }
  g.length_y = g.n_t * g.delta_t;
  g.n_x = static_cast<uint16_t>(std::floor(g.length_x / g.delta_xz));
  g.n_z = static_cast<uint16_t>(std::floor(lz / g.delta_xz));
  g.n_y = static_cast<uint16_t>(std::floor(g.length_y / g.delta_xy));
  g.x0 = -g.length_x / 2;
  g.z0 = -lz / 2;
  g.y0 = -g.length_y / 2;
  g.offset_r = ((g.delta_xz / std::sqrt(3.0)) + g.delta_r / 2) / bins_;
  g.offset_t = ((g.delta_xz / 2) + g.delta_t / 2) / bins_;
  if (g.n_x < 1 || g.n_y < 1 || g.n_z < 1) return fail(MBIR_EINVAL, "geometry: empty volume");
  return MBIR_OK;
}

int Engine::build_tables() {
  const Geometry& g = g_;
  const int nt = g.n_theta, PR = p_.profile_resolution, BR = p_.beam_resolution;
  tab_.cosv.assign(nt, 0);
  tab_.sinv.assign(nt, 0);
  std::vector<double> profile(static_cast<size_t>(nt) * PR);
  for (int i = 0; i < nt; i++) {
    const double rad = tilts_[i] * (kPi / 180.0);
    tab_.cosv[i] = std::cos(rad);
    tab_.sinv[i] = std::sin(rad);
    // calculateVoxelProfile (HAADF_ReconstructionEngine.cpp:957-1029); the HAADF engine
    // converts the angle to radians twice before the profile feeding DetectorResponse.
    double angle = p_.compat_double_angle ? rad * (kPi / 180.0) : rad;
    while (angle > kPi / 2) angle -= kPi / 2;
    while (angle < 0) angle += kPi / 2;
    const double mv =
        (angle <= kPi / 4) ? g.delta_xz / std::cos(angle) : g.delta_xz / std::cos(kPi / 2 - angle);
    const double tmp = std::cos(kPi / 4);
    const double d1 = tmp * std::cos((kPi / 4 - angle));
    const double d2 = tmp * std::fabs((std::cos((kPi / 4 + angle))));
    const double lc = 1 - d1, ln = 1 - d2, rn = 1 + d2, rc = 1 + d1;
    for (int j = 0; j < PR; j++) {
      const double t = 2.0 * j / PR;
      double v;
      if (t <= lc || t >= rc)
        v = 0;
      else if (t > rn)
        v = mv * (rc - t) / (rc - rn);
      else if (t >= ln)
        v = mv;
      else
        v = mv * (t - lc) / (ln - lc);
      profile[static_cast<size_t>(i) * PR + j] = v;
    }
  }
  // beam profile (DetectorParameters.cpp:78-100) and response (DetectorResponse.cpp:66-127)
  std::vector<double> beam(BR);
  double sum = 0;
  for (int i = 0; i < BR; i++) {
    beam[i] = 0.54 - 0.46 * std::cos((2.0 * kPi / BR) * i);
    sum += beam[i];
  }
  for (int i = 0; i < BR; i++) {
    beam[i] /= sum;
    beam[i] /= g.delta_t;
  }
  tab_.H.assign(static_cast<size_t>(nt) * bins_, 0.0);
  const double bw = g.delta_r, r0 = -bw / 2, step = bw / BR, tc = PR / (2 * g.delta_xz);
  host_parallel(nt, [&](int k_begin, int k_end) {
    for (int k = k_begin; k < k_end; k++)
      for (int i = 0; i < bins_; i++) {
        const double rmin = i * g.offset_r - g.delta_xz;
        double s = 0;
        for (int pp = 0; pp < BR; pp++) {
          const double r = r0 + pp * step;
          if (r < rmin) continue;
          int pi = static_cast<int>(std::floor((r - rmin) * tc));
          if (pi < 0) pi = 0;
          if (pi >= PR) pi = PR - 1;
          s += profile[static_cast<size_t>(k) * PR + pi] * beam[pp];
        }
        tab_.H[static_cast<size_t>(k) * bins_ + i] = s;
      }
  });
  // H_t (HAADF_ForwardModel.cpp:408-451)
  tab_.Ht.assign(bins_, 0.0);
  for (int i = 0; i < bins_; i++) {
    const double pct = i * g.offset_t;
    double v;
    if (g.delta_xy >= g.delta_t)
      v = (pct <= ((g.delta_xy / 2) - (g.delta_t / 2))) ? g.delta_t
                                                        : -1 * pct + (g.delta_xy / 2) + g.delta_t / 2;
    else
      v = (pct <= g.delta_t / 2 - g.delta_xy / 2) ? g.delta_xy
                                                  : -pct + (g.delta_xy / 2) + g.delta_t / 2;
    tab_.Ht[i] = v < 0 ? 0 : v;
  }
  // voxel-line response per slice (storeVoxelResponse, _Extra.cpp:329-404)
  tab_.t_first.assign(g.n_y, 0);
  tab_.t_count.assign(g.n_y, 0);
  tab_.hval.assign(static_cast<size_t>(g.n_y) * kMaxTRows, 0.0);
  t_rows_ = 1;
  for (int i = 0; i < g.n_y; i++) {
    const double t = ((double)i + 0.5) * g.delta_xy + g.y0;
    const double tmin = (t - g.delta_xy / 2) > g.T0 ? t - g.delta_xy / 2 : g.T0;
    const double tmax = (t + g.delta_xy / 2) <= g.TMax ? t + g.delta_xy / 2 : g.TMax;
    int smin = static_cast<int16_t>(static_cast<uint16_t>(std::floor((tmin - g.T0) / g.delta_t)));
    int smax = static_cast<int16_t>(static_cast<uint16_t>(std::floor((tmax - g.T0) / g.delta_t)));
    if (smin < 0) smin = 0;
    if (smax >= g.n_t) smax = g.n_t - 1;
    int cnt = 0, first = 0;
    for (int it = smin; it <= smax; it++) {
      const double ct = ((double)it + 0.5) * g.delta_t + g.T0;
      const double dt = std::fabs(ct - t);
      const int idt = static_cast<uint16_t>(std::floor(dt / g.offset_t));
      double pt = 0;
      if (idt < bins_) {
        const double w3 = dt - (double)idt * g.offset_t;
        const double w4 = ((double)idt + 1) * g.offset_t - dt;
        const int tt = idt + 1 < bins_ ? idt + 1 : bins_ - 1;
        pt = (w4 / g.offset_t) * tab_.Ht[idt] + (w3 / g.offset_t) * tab_.Ht[tt];
      }
      if (pt != 0) {
        if (cnt == 0) first = it;
        if (cnt >= kMaxTRows || first + cnt != it)
          return fail(MBIR_ENOTSUP, "voxel-line response wider than 4 detector rows");
        tab_.hval[static_cast<size_t>(i) * kMaxTRows + cnt] = pt;
        cnt++;
      }
    }
    tab_.t_first[i] = first;
    tab_.t_count[i] = cnt;
    t_rows_ = std::max(t_rows_, cnt);
  }
  // same-colour slices must touch disjoint detector rows
  for (int i = 0; i + 2 < g.n_y; i++)
    if (tab_.t_count[i] > 0 && tab_.t_count[i + 2] > 0 &&
        tab_.t_first[i] + tab_.t_count[i] > tab_.t_first[i + 2])
      return fail(MBIR_ENOTSUP, "voxel slices y and y+2 share detector rows");
  // empty A-columns (the reference zeroes those lines, HAADF_ReconstructionEngine.cpp:614-625)
  tab_.line_nonempty.assign(static_cast<size_t>(g.n_z) * g.n_x, 0);
  std::vector<int64_t> row_entries(g.n_z, 0);  // summed in row order below
  host_parallel(g.n_z, [&](int z_begin, int z_end) {
    for (int z = z_begin; z < z_end; z++)
      for (int x = 0; x < g.n_x; x++) {
        const double xc = g.x0 + ((double)x + 0.5) * g.delta_xz;
        const double zc = g.z0 + ((double)z + 0.5) * g.delta_xz;
        int64_t nnz = 0;
        for (int i = 0; i < nt; i++) {
          const double r = xc * tab_.cosv[i] - zc * tab_.sinv[i];
          const double rmin = r - g.delta_xz, rmax = r + g.delta_xz;
          if (rmax < g.R0 || rmin > g.RMax) continue;
          int imin = static_cast<int>(std::floor((rmin - g.R0) / g.delta_r));
          int imax = static_cast<int>(std::floor((rmax - g.R0) / g.delta_r));
          if (imax >= g.n_r) imax = g.n_r - 1;
          if (imin < 0) imin = 0;
          for (int j = imin; j <= imax; j++) {
            const double dr = std::fabs(r - (g.R0 + ((double)j + 0.5) * g.delta_r));
            const int idr = static_cast<int>(std::floor(dr / g.offset_r));
            if (idr < bins_) {
              const double w1 = dr - idr * g.offset_r, w2 = (idr + 1) * g.offset_r - dr;
              const int ii = idr + 1 < bins_ ? idr + 1 : bins_ - 1;
              const double f1 = (w2 / g.offset_r) * tab_.H[static_cast<size_t>(i) * bins_ + idr] +
                                (w1 / g.offset_r) * tab_.H[static_cast<size_t>(i) * bins_ + ii];
              if (f1 > 0) nnz++;
            }
          }
        }
        tab_.line_nonempty[static_cast<size_t>(z) * g.n_x + x] = nnz > 0 ? 1 : 0;
        row_entries[z] += nnz;
      }
  });
  footprint_entries_ = 0;
  for (int z = 0; z < g.n_z; z++) footprint_entries_ += row_entries[z];
  return MBIR_OK;
}

// Smallest x stride S such that voxels (z,x) and (z,x+S) never share a detector bin at any
// view (bin intervals [floor(u-d), floor(u+d)] widened by a rounding margin), and S >= 2 so
// that in-row prior neighbours are never updated together.
int Engine::compute_stride() {
  const Geometry& g = g_;
  const double d = g.delta_xz / g.delta_r, eps = 1e-4;
  int S = 2;
  for (; S < g.n_x; ++S) {
    // any conflict at this stride, searched over rows in parallel (a yes/no answer)
    std::atomic<bool> found{false};
    host_parallel(g.n_z, [&](int z_begin, int z_end) {
      bool conflict = false;
      for (int v = 0; v < g.n_theta && !conflict; ++v) {
        const double bxv = g.delta_xz * tab_.cosv[v] / g.delta_r;
        const double bzv = g.delta_xz * tab_.sinv[v] / g.delta_r;
        const double u0 = ((g.x0 + 0.5 * g.delta_xz) * tab_.cosv[v] -
                           (g.z0 + 0.5 * g.delta_xz) * tab_.sinv[v] - g.R0) /
                          g.delta_r;
        if (found.load(std::memory_order_relaxed)) break;
        for (int z = z_begin; z < z_end && !conflict; ++z) {
          for (int x = 0; x + S < g.n_x; ++x) {
            const double ua = u0 + x * bxv - z * bzv, ub = ua + S * bxv;
            double alo = std::floor(ua - d - eps), ahi = std::floor(ua + d + eps);
            double blo = std::floor(ub - d - eps), bhi = std::floor(ub + d + eps);
            alo = std::max(alo, 0.0);
            blo = std::max(blo, 0.0);
            ahi = std::min(ahi, (double)g.n_r - 1);
            bhi = std::min(bhi, (double)g.n_r - 1);
            if (alo > ahi || blo > bhi) continue;
            if (!(ahi < blo || bhi < alo)) {
              conflict = true;
              break;
            }
          }
        }
      }
      if (conflict) found.store(true);
    });
    if (!found.load()) break;
  }
  stride_ = std::max(2, std::min(S, std::max(g.n_x, 2)));
  return MBIR_OK;
}

int Engine::init_nuisance_host() {
  const int nt = g_.n_theta;
  // createInitialGainsData / OffsetsData / VariancesData (HAADF_ForwardModel.cpp:248-402)
  init_gain_.assign(nt, p_.target_gain);
  if (!user_gain_.empty()) init_gain_ = user_gain_;
  init_offset_.assign(nt, bf_ ? bf_default_offset() : p_.default_offset);
  if (!user_offset_.empty()) {
    init_offset_ = user_offset_;
  } else if (!p_.use_default_offset) {
    // ComputeInitialOffsets::execute (ComputeInitialOffsets.cpp:58-186): LS fit of the
    // per-view mean against [1/cos(theta), 1]; the constant term is every view's offset.
    std::vector<double> avg(nt), tg(nt);
    for (int th = 0; th < nt; th++) {
      double s = 0;
      for (int r = 0; r < g_.n_r; r++)
        for (int t = 0; t < g_.n_t; t++)
          s += counts_[(static_cast<size_t>(th) * g_.n_r + r) * g_.n_t + t];
      avg[th] = s / (g_.n_r * g_.n_t);
      tg[th] = 1.0 / std::cos(tilts_[th] * kPi / 180);
    }
    double pm[2][2] = {{0, 0}, {0, 0}};
    for (int k = 0; k < nt; k++) {
      const double a[2] = {tg[k], 1.0};
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) pm[i][j] += a[i] * a[j];
    }
    const double det = pm[0][0] * pm[1][1] - (pm[0][1] * pm[0][1]);
    const double inv10 = -pm[0][1] / det, inv11 = pm[0][0] / det;
    double tv0 = 0, tv1 = 0;
    for (int k = 0; k < nt; k++) {
      tv0 += tg[k] * avg[k];
      tv1 += avg[k];
    }
    const double est1 = inv10 * tv0 + inv11 * tv1;
    init_offset_.assign(nt, est1);
  }
  init_var_.assign(nt, p_.default_variance);
  if (!user_var_.empty()) init_var_ = user_var_;
  // gainAndOffsetInitialization (_Extra.cpp:280-307)
  I_ = init_gain_;
  mu_ = init_offset_;
  double s = 0;
  for (int k = 0; k < nt; k++) s += I_[k];
  s /= nt;
  if (s - p_.target_gain > 1e-5) {
    const double t = p_.target_gain / s;
    for (int k = 0; k < nt; k++) I_[k] = init_gain_[k] * t;
  }
  // calculateMeasurementWeight (_Extra.cpp:693-771), IDENTITY_NOISE_MODEL: w = 1 / alpha.
  // Bright field: per-entry weights (bf_upload); alpha starts at the initial variance when
  // NOISE_ESTIMATION is on (BFForwardModel.cpp:337-341).
  alpha_.assign(nt, 1.0);
  w_.assign(nt, 1.0);
  const bool per_view_var = bf_ ? p_.noise_estimation != 0 : p_.noise_model != 0;
  for (int k = 0; k < nt; k++) {
    if (per_view_var) {
      alpha_[k] = init_var_[k];
      if (!bf_) w_[k] = 1.0 / alpha_[k];
    }
  }
  return MBIR_OK;
}

int Engine::alloc_device() {
  cudaError_t ce = cudaSetDevice(p_.device);
  if (ce != cudaSuccess) return fail(MBIR_EDEVICE, std::string("cudaSetDevice: ") + cudaGetErrorString(ce));
  const Geometry& g = g_;
  n_rp_ = (g.n_r + 3) / 4 * 4;
  n_rs_ = (n_rp_ % 32 == 0) ? n_rp_ + 4 : n_rp_;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, p_.device);
  const bool bfa = bright_field_assisted();
  // the bright-field sweep (per-entry weights and selector) serves assisted HAADF as well
  n_sp_ = (bf_ || bfa) ? (g.n_r + 15) / 16 * 16 : 0;
  // a selector row stride of a multiple of 128 bytes would put every view's byte of a detector
  // bin into one shared-memory bank; 16 more bytes spread the views over eight banks
  if (n_sp_ > 0 && n_sp_ % 128 == 0) n_sp_ += 16;
  smem_bytes_ = sweep_smem_bytes(g.n_theta, g.n_x, n_rs_, t_rows_, bins_, fp64_, n_sp_);
  smem_sched_bytes_ = sweep_smem_bytes(g.n_theta, g.n_x, n_rs_, t_rows_, bins_, fp64_, n_sp_, true);
  // above 160 views the sweeps keep the slices in HBM (32 lanes x 8 views)
  stage_ = smem_bytes_ <= static_cast<size_t>(max_smem) && p_.slice_staging == 0 &&
           g.n_theta <= kMaxViewsShaped;
  if (!stage_) {
    smem_bytes_ = sweep_smem_bytes(g.n_theta, g.n_x, 0, t_rows_, bins_, fp64_, 0);
    smem_sched_bytes_ = sweep_smem_bytes(g.n_theta, g.n_x, 0, t_rows_, bins_, fp64_, 0, true);
  }
  const size_t ns = static_cast<size_t>(g.n_t) * g.n_theta * n_rp_;
  const size_t nh = static_cast<size_t>(g.n_theta) * g.n_r * g.n_t;
  const size_t nv = static_cast<size_t>(g.n_z) * g.n_x * g.n_y;
  int rc = 0;
  rc |= dmalloc_bytes(&d_y_, ns * rb_);
  rc |= dmalloc_bytes(&d_e_, ns * rb_);
  rc |= dmalloc_bytes(&d_yest_, ns * rb_);
  rc |= dmalloc_bytes(&d_x_, nv * rb_);
  rc |= dmalloc(&d_stage_, std::max(nh, nv));
  rc |= dmalloc_bytes(&d_H_, static_cast<size_t>(g.n_theta) * (bins_ + 1) * rb_);
  rc |= dmalloc(&d_bx_, g.n_theta);
  rc |= dmalloc(&d_bxd_, g.n_theta);
  rc |= dmalloc(&d_u0_, g.n_theta);
  rc |= dmalloc(&d_bz_, g.n_theta);
  rc |= dmalloc_bytes(&d_gw_, static_cast<size_t>(g.n_theta) * 2 * rb_);
  rc |= dmalloc(&d_tfirst_, g.n_y);
  rc |= dmalloc(&d_tcount_, g.n_y);
  rc |= dmalloc_bytes(&d_hval_, static_cast<size_t>(g.n_y) * kMaxTRows * rb_);
  rc |= dmalloc(&d_rows_, g.n_z);
  rc |= dmalloc(&d_lineok_, static_cast<size_t>(g.n_z) * g.n_x);
  rc |= dmalloc(&d_cosv_, g.n_theta);
  rc |= dmalloc(&d_sinv_, g.n_theta);
  rc |= dmalloc(&d_Href_, static_cast<size_t>(g.n_theta) * bins_);
  rc |= dmalloc(&d_lines_, static_cast<size_t>(g.n_z) * g.n_x);
  rc |= dmalloc(&d_stats_, static_cast<size_t>((g.n_y + 1) / 2 + 1) * kStatSlots * 2);
  rc |= dmalloc(&d_stat4_, kStatSlots);
  rc |= dmalloc(&d_mu_, g.n_theta);
  rc |= dmalloc(&d_gain_, g.n_theta);
  rc |= dmalloc(&d_mu2_, g.n_theta);
  rc |= dmalloc(&d_gain2_, g.n_theta);
  rc |= dmalloc(&d_wv_, g.n_theta);
  n_chunk_ = std::min(32, std::max(1, g.n_t));
  rc |= dmalloc(&d_partial_, static_cast<size_t>(g.n_theta) * n_chunk_ * 6 +
                                 static_cast<size_t>(prior_blocks_));
  rc |= dmalloc(&d_vsum_, static_cast<size_t>(g.n_theta) * 6);
  rc |= dmalloc(&d_err_, 1);
  if (bf_) {
    const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
    rc |= dmalloc_bytes(&d_w_, ns * rb_);
    rc |= dmalloc(&d_sel_, static_cast<size_t>(g.n_t) * g.n_theta * n_sp_);
    rc |= dmalloc(&d_magfx_, nl);
    rc |= dmalloc(&d_mag_, nl);
    rc |= dmalloc(&d_filt_, nl);
    rc |= dmalloc(&d_active_, nl);
    rc |= dmalloc(&d_bfpart_, 4096);
    rc |= dmalloc(&d_bfout_, 16);
    rc |= dmalloc(&d_alpha_, g.n_theta);
    rc |= dmalloc(&d_stage64_, nh);
  }
  if (bfa) {
    const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
    rc |= dmalloc_bytes(&d_w_, ns * rb_);
    rc |= dmalloc_bytes(&d_bfm_, ns * rb_);
    rc |= dmalloc(&d_sel_, static_cast<size_t>(g.n_t) * g.n_theta * n_sp_);
    rc |= dmalloc(&d_active_, nl);
    rc |= dmalloc(&d_stage64_, nh);
  }
  if (rc) return fail(MBIR_ENOMEM, "device allocation failed");
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return fail(MBIR_EDEVICE, "stream creation failed");
  stream_ = s;
  cudaEvent_t e0, e1, e2, e3, e4, e5;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  cudaEventCreate(&e3);
  cudaEventCreate(&e4);
  cudaEventCreate(&e5);
  ev0_ = e0;
  ev1_ = e1;
  ev2_ = e2;
  ev3_ = e3;
  ev4_ = e4;
  ev5_ = e5;
  cudaMemsetAsync(d_err_, 0, sizeof(int), s);
  return MBIR_OK;
}

int Engine::upload_views() {
  const int nt = g_.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  std::vector<float2> gw(nt);
  std::vector<double2> gwd(nt);
  for (int v = 0; v < nt; v++) {
    gw[v] = make_float2(static_cast<float>(I_[v]), static_cast<float>(w_[v]));
    gwd[v] = make_double2(I_[v], w_[v]);
  }
  if (fp64_)
    cudaMemcpyAsync(d_gw_, gwd.data(), sizeof(double2) * nt, cudaMemcpyHostToDevice, s);
  else
    cudaMemcpyAsync(d_gw_, gw.data(), sizeof(float2) * nt, cudaMemcpyHostToDevice, s);
  cudaStreamSynchronize(s);  // host vectors go out of scope
  cudaMemcpyAsync(d_mu_, mu_.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_gain_, I_.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_wv_, w_.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : cuda_check(MBIR_EDEVICE, "upload views");
}

int Engine::check_device_error() {
  int h = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  if (cudaMemcpyAsync(&h, d_err_, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return cuda_check(MBIR_EDEVICE, "device error check");
  if (h == 0) return 0;
  // reported once: the work a timed-out wait guarded was skipped, the state stays consistent
  cudaMemsetAsync(d_err_, 0, sizeof(int), s);
  if (h & 4)
    return fail(MBIR_ENOTSUP,
                "call schedule: the call needs more colours than the device colouring holds "
                "(use call_schedule 2)");
  return fail(MBIR_ETIMEOUT, "a bounded device wait timed out");
}

int Engine::build_host() {
  if (state_ < 1) return fail(MBIR_ESTATE, "no sinogram");
  int rc;
  if ((rc = build_geometry())) return rc;
  if ((rc = build_tables())) return rc;
  const double hw = g_.delta_xz / g_.delta_r;
  nb_ = 2 * static_cast<int>(std::ceil(hw)) + 1;
  if (nb_ != 3 && nb_ != 5 && nb_ != 9)
    return fail(MBIR_ENOTSUP, "voxel/detector size ratio must be 1, 2 or 4");
  if ((rc = compute_stride())) return rc;
  if ((rc = init_nuisance_host())) return rc;
  if (bf_ && (rc = bf_prepare_host())) return rc;
  host_ready_ = true;
  return MBIR_OK;
}

int Engine::prepare() {
  if (state_ < 1) return fail(MBIR_ESTATE, "prepare: no sinogram");
  if (state_ >= 2) release();
  if (p_.order_mode == MBIR_ORDER_REFERENCE && g_.n_theta > kMaxViewsShaped)
    return fail(MBIR_ENOTSUP, "prepare: the reference-order modes take at most 160 views");
  notify("Calculating A Matrix....", 0, MBIR_UPDATE_PROGRESS_MESSAGE);
  int rc;
  if ((rc = build_host())) return rc;
  if ((rc = alloc_device())) return rc;
  const double hw = g_.delta_xz / g_.delta_r;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);

  // tables
  std::vector<float> Hf(static_cast<size_t>(g.n_theta) * (bins_ + 1));
  std::vector<float2> bx(g.n_theta);
  std::vector<double> u0(g.n_theta), bz(g.n_theta);
  for (int v = 0; v < g.n_theta; v++) {
    for (int i = 0; i < bins_; i++)
      Hf[static_cast<size_t>(v) * (bins_ + 1) + i] =
          static_cast<float>(tab_.H[static_cast<size_t>(v) * bins_ + i]);
    Hf[static_cast<size_t>(v) * (bins_ + 1) + bins_] =
        static_cast<float>(tab_.H[static_cast<size_t>(v) * bins_ + bins_ - 1]);
    const double b = g.delta_xz * tab_.cosv[v] / g.delta_r;
    const float bh = static_cast<float>(b);
    bx[v] = make_float2(bh, static_cast<float>(b - static_cast<double>(bh)));
    u0[v] = ((g.x0 + 0.5 * g.delta_xz) * tab_.cosv[v] - (g.z0 + 0.5 * g.delta_xz) * tab_.sinv[v] -
             g.R0) /
            g.delta_r;
    bz[v] = g.delta_xz * tab_.sinv[v] / g.delta_r;
  }
  std::vector<float> hv(tab_.hval.size());
  for (size_t i = 0; i < hv.size(); i++) hv[i] = static_cast<float>(tab_.hval[i]);
  std::vector<double> Hd(Hf.size()), bxd(g.n_theta);
  for (int v = 0; v < g.n_theta; v++) {
    for (int i = 0; i <= bins_; i++)
      Hd[static_cast<size_t>(v) * (bins_ + 1) + i] =
          tab_.H[static_cast<size_t>(v) * bins_ + std::min(i, bins_ - 1)];
    bxd[v] = g.delta_xz * tab_.cosv[v] / g.delta_r;
  }
  if (fp64_) {
    cudaMemcpyAsync(d_H_, Hd.data(), sizeof(double) * Hd.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_hval_, tab_.hval.data(), sizeof(double) * tab_.hval.size(),
                    cudaMemcpyHostToDevice, s);
  } else {
    cudaMemcpyAsync(d_H_, Hf.data(), sizeof(float) * Hf.size(), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_hval_, hv.data(), sizeof(float) * hv.size(), cudaMemcpyHostToDevice, s);
  }
  cudaMemcpyAsync(d_bxd_, bxd.data(), sizeof(double) * bxd.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_bx_, bx.data(), sizeof(float2) * bx.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_u0_, u0.data(), sizeof(double) * u0.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_bz_, bz.data(), sizeof(double) * bz.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_tfirst_, tab_.t_first.data(), sizeof(int) * g.n_y, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_tcount_, tab_.t_count.data(), sizeof(int) * g.n_y, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_lineok_, tab_.line_nonempty.data(), tab_.line_nonempty.size(),
                  cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_cosv_, tab_.cosv.data(), sizeof(double) * g.n_theta, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_sinv_, tab_.sinv.data(), sizeof(double) * g.n_theta, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_Href_, tab_.H.data(), sizeof(double) * tab_.H.size(), cudaMemcpyHostToDevice, s);

  // measured sinogram -> [t][theta][r_pad]
  const size_t nh = static_cast<size_t>(g.n_theta) * g.n_r * g.n_t;
  if (bf_) {
    cudaMemcpyAsync(d_stage64_, ylog_.data(), sizeof(double) * nh, cudaMemcpyHostToDevice, s);
    if ((rc = launch_layout_from_double(d_stage64_, d_y_, g.n_theta, g.n_r, n_rp_, g.n_t, fp64_, s)))
      return cuda_check(rc, "sinogram upload");
  } else {
    cudaMemcpyAsync(d_stage_, counts_.data(), sizeof(float) * nh, cudaMemcpyHostToDevice, s);
    if ((rc = launch_sino_to_dev(d_stage_, d_y_, g.n_theta, g.n_r, n_rp_, g.n_t, fp64_, s)))
      return cuda_check(rc, "sinogram upload");
  }
  if (bright_field_assisted()) {
    cudaMemcpyAsync(d_stage64_, bfm_.data(), sizeof(double) * nh, cudaMemcpyHostToDevice, s);
    if ((rc = launch_layout_from_double(d_stage64_, d_bfm_, g.n_theta, g.n_r, n_rp_, g.n_t, fp64_,
                                        s)))
      return cuda_check(rc, "bright-field upload");
    // selector always on, every line in every sweep
    cudaMemsetAsync(d_sel_, 1, static_cast<size_t>(g.n_t) * g.n_theta * n_sp_, s);
    cudaMemsetAsync(d_active_, 1, static_cast<size_t>(g.n_z) * g.n_x, s);
  }

  // initial volume (InitialReconstructionInitializer::initializeData, :74-90)
  const size_t nv = static_cast<size_t>(g.n_z) * g.n_x * g.n_y;
  std::vector<double> vol(nv);
  if (!init_vol_.empty()) {
    if (init_vol_.size() != nv) return fail(MBIR_EINVAL, "initial volume size does not match");
    vol = init_vol_;
  } else {
    std::fill(vol.begin(), vol.end(), fp64_ ? p_.default_recon_value
                                            : static_cast<double>(static_cast<float>(
                                                  p_.default_recon_value)));
  }
  for (int z = 0; z < g.n_z; z++)
    for (int x = 0; x < g.n_x; x++)
      if (!tab_.line_nonempty[static_cast<size_t>(z) * g.n_x + x])
        for (int y = 0; y < g.n_y; y++) vol[(static_cast<size_t>(z) * g.n_x + x) * g.n_y + y] = 0.0;
  if (fp64_) {
    // the doubles as given (an FP64 engine starts exactly where the reference starts)
    double* tmp = nullptr;
    if (cudaMalloc(&tmp, sizeof(double) * nv) != cudaSuccess) {
      cudaGetLastError();
      return fail(MBIR_ENOMEM, "volume upload: device allocation failed");
    }
    cudaMemcpyAsync(tmp, vol.data(), sizeof(double) * nv, cudaMemcpyHostToDevice, s);
    rc = launch_vol64_to_dev(tmp, d_x_, g.n_z, g.n_x, g.n_y, fp64_, s);
    const bool ok = cudaStreamSynchronize(s) == cudaSuccess;
    cudaFree(tmp);
    if (rc) return cuda_check(rc, "volume upload");
    if (!ok) return cuda_check(MBIR_EDEVICE, "prepare sync");
  } else {
    std::vector<float> vf(vol.begin(), vol.end());
    cudaMemcpyAsync(d_stage_, vf.data(), sizeof(float) * nv, cudaMemcpyHostToDevice, s);
    if ((rc = launch_vol_to_dev(d_stage_, d_x_, g.n_z, g.n_x, g.n_y, fp64_, s)))
      return cuda_check(rc, "volume upload");
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "prepare sync");
  }

  // device geometry + prior constants
  dg_.n_theta = g.n_theta;
  dg_.n_r = g.n_r;
  dg_.n_rp = n_rp_;
  dg_.n_t = g.n_t;
  dg_.n_x = g.n_x;
  dg_.n_y = g.n_y;
  dg_.n_z = g.n_z;
  dg_.bins = bins_;
  dg_.kr = static_cast<float>(g.delta_r / g.offset_r);
  dg_.half_width = static_cast<float>(hw);
  // ROI mask (initializeROIMask, _Extra.cpp:227-248) as index ranges
  dg_.roi_x0 = g.n_x;
  dg_.roi_x1 = -1;
  for (int j = 0; j < g.n_x; j++) {
    const double x = g.x0 + ((double)j + 0.5) * g.delta_xz;
    if (x >= -(g.n_r * g.delta_r) / 2 && x <= (g.n_r * g.delta_r) / 2) {
      dg_.roi_x0 = std::min(dg_.roi_x0, j);
      dg_.roi_x1 = std::max(dg_.roi_x1, j);
    }
  }
  dg_.roi_z0 = g.n_z;
  dg_.roi_z1 = -1;
  for (int i = 0; i < g.n_z; i++) {
    const double z = g.z0 + ((double)i + 0.5) * g.delta_xz;
    if (z >= -g.length_z / 2 && z <= g.length_z / 2) {
      dg_.roi_z0 = std::min(dg_.roi_z0, i);
      dg_.roi_z1 = std::max(dg_.roi_z1, i);
    }
  }
  for (int i = 0; i < 27; i++) flt_.f[i] = kFilter[i];
  flt_.mrf_p = p_.qggmrf_p;
  flt_.mrf_q = p_.qggmrf_q;
  flt_.mrf_c = p_.qggmrf_c;
  flt_.mrf_alpha = p_.qggmrf_alpha;
  flt_.sig_p = std::pow(p_.sigma_x, p_.qggmrf_p);
  flt_.sig_pq = std::pow(p_.sigma_x, p_.qggmrf_p - p_.qggmrf_q);
  flt_.inv_sig_pq = 1.0 / flt_.sig_pq;

  if (resume_ && bright_field_assisted())
    return fail(MBIR_ENOTSUP, "checkpoint: HAADF without bright-field data only");
  if (resume_) {
    // the checkpoint's gains, offsets and variances exactly (no renormalisation); w = 1/alpha
    // holds for HAADF with and without the noise model
    I_ = resume_gain_;
    mu_ = resume_offset_;
    alpha_ = resume_var_;
    for (int k = 0; k < g.n_theta; k++) w_[k] = 1.0 / alpha_[k];
  }
  if ((rc = upload_views())) return rc;
  state_ = 2;
  sweeps_done_ = 0;
  outer_next_ = resume_ ? resume_outer_ : 0;
  stop_now_ = resume_ ? resume_stop_ : p_.stop_threshold;
  // voxel-group shape: the requested one when it covers the views, else the default
  shape_ = 0;
  if (((p_.lane_shape >= 1 && p_.lane_shape <= 4) ||
       (p_.lane_shape == 5 && g.n_theta > kMaxViewsShaped)) &&
      g.n_theta <= shape_max_views(p_.lane_shape))
    shape_ = p_.lane_shape;
  if (shape_ == 0) {
    const int d = lane_shape(g.n_theta);
    shape_ = d == 0 ? 1 : d + 2;
  }
  // forward projection + error sinogram (HAADF_ReconstructionEngine.cpp:636-691)
  notify("Starting Forward Projection", 10, MBIR_UPDATE_PROGRESS_VALUE_AND_MESSAGE);
  if ((rc = forward_project())) return rc;
  if (resume_) {
    // the checkpoint's error sinogram in place of the one the projection rebuilt (that one
    // differs in the last bits from the sweeps' running updates)
    const size_t bytes = static_cast<size_t>(g.n_t) * g.n_theta * n_rp_ * rb_;
    if (resume_e_.size() != bytes)
      return fail(MBIR_EINVAL, "checkpoint: error sinogram size does not match this engine");
    cudaMemcpyAsync(d_e_, resume_e_.data(), bytes, cudaMemcpyHostToDevice, s);
    sweeps_done_ = resume_sweeps_;
  }
  if (bf_ && (rc = bf_upload())) return rc;
  if (bf_ && (rc = bf_prepare_schedule())) return rc;
  if (p_.lane_shape == 0 && (rc = autotune_shape())) return rc;
  // everything prepare queued has run: another thread may hand the engine to a batch stream
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "prepare sync");
  return MBIR_OK;
}

int Engine::forward_project() {
  if (state_ < 2) return fail(MBIR_ESTATE, "forward_project: call prepare first");
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t ns = static_cast<size_t>(g.n_t) * g.n_theta * n_rp_;
  if (!stage_) cudaMemsetAsync(d_yest_, 0, rb_ * ns, s);
  std::vector<int32_t> rows(g.n_z);
  for (int i = 0; i < g.n_z; i++) rows[i] = i;
  cudaMemcpyAsync(d_rows_, rows.data(), sizeof(int) * g.n_z, cudaMemcpyHostToDevice, s);
  if (exact_) {
    int rc = launch_exact_project(exact_args(), static_cast<double*>(d_yest_), s);
    if (rc) return cuda_check(rc, "forward projection (exact)");
    rc = bright_field_assisted()
             ? launch_exact_bfa_error(exact_args(), static_cast<const double*>(d_y_),
                                      static_cast<const double*>(d_yest_), d_mu_, s)
             : launch_error_from_projection(d_y_, d_yest_, d_e_, d_mu_, g.n_theta, n_rp_, g.n_r,
                                            g.n_t, fp64_, s);
    if (rc) return cuda_check(rc, "error sinogram");
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "forward projection");
    return check_device_error();
  }
  SweepArgs a{};
  a.g = dg_;
  a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_, d_lineok_};
  a.flt = flt_;
  a.x = d_x_;
  a.e = d_yest_;
  a.row_order = d_rows_;
  a.stride = stride_;
  a.mode = kModeProject;
  a.fp64 = fp64_;
  a.smem_rows = stage_ ? 1 : 0;
  a.n_rs = stage_ ? n_rs_ : 0;
  a.shape = shape_;
  a.stats = nullptr;
  a.err = d_err_;
  for (int colour = 0; colour < 2; colour++) {
    a.colour = colour;
    a.n_slices = (g.n_y - colour + 1) / 2;
    if (a.n_slices <= 0) continue;
    int rc = launch_sweep(a, nb_, smem_bytes_, s);
    if (rc) return cuda_check(rc, "forward projection launch");
  }
  int rc;
  if (bright_field_assisted()) {
    // scaled error e / m and per-entry weights m^2 w (mbir_bfassist.cu)
    rc = launch_bfa_error(d_y_, d_yest_, d_bfm_, d_e_, d_mu_, g.n_theta, n_rp_, g.n_r, g.n_t,
                          fp64_, s);
    if (!rc) rc = launch_bfa_weights(d_bfm_, d_wv_, d_w_, g.n_theta, n_rp_, g.n_r, g.n_t, fp64_, s);
  } else {
    rc = launch_error_from_projection(d_y_, d_yest_, d_e_, d_mu_, g.n_theta, n_rp_, g.n_r, g.n_t,
                                      fp64_, s);
  }
  if (rc) return cuda_check(rc, "error sinogram");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "forward projection");
  return check_device_error();
}

// The bright-field sweep arguments of an assisted HAADF engine: per-entry weights m^2 w, the
// selector always on, every line, no magnitude map
DevBF Engine::bfa_sweep_args() const {
  DevBF b{};
  b.w = d_w_;
  b.sel = d_sel_;
  b.n_sp = n_sp_;
  b.active = d_active_;
  b.mag_fx = nullptr;
  b.bragg_t = 1.0e30;
  b.bragg_dt = 0.0;
  return b;
}

void Engine::row_order_for_sweep(int sweep, std::vector<int32_t>& order) const {
  const int nz = g_.n_z;
  order.resize(nz);
  for (int i = 0; i < nz; i++) order[i] = i;
  MT19937 gen(p_.seed * 2654435761u + static_cast<uint32_t>(sweep) * 40503u + 17u);
  for (int i = nz - 1; i > 0; --i) {
    const int j = static_cast<int>(gen.next() % static_cast<uint32_t>(i + 1));
    std::swap(order[i], order[j]);
  }
}

int Engine::sweep(int outer, int inner, double* stats4) {
  if (state_ < 2) return fail(MBIR_ESTATE, "sweep: call prepare first");
  if (cancel_.load()) return fail(MBIR_ECANCELLED, "cancelled");
  if (bf_) return bf_call(outer, inner, stats4);
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const int iter_nonzero = (inner > 0 || outer > 0) ? 1 : 0;
  int rc = 0;
  cudaEventRecord(static_cast<cudaEvent_t>(ev0_), s);
  if (p_.order_mode == MBIR_ORDER_REFERENCE) {
    // UpdateYSlice seeds its generator from the millisecond clock at every sweep
    // (HAADF_ReconstructionEngine_UpdateVoxels.cpp:161-162): a new order per sweep (seed + sweep
    // index), or the same order every sweep as with the clock frozen (MBIR_SEED_FIXED)
    const uint32_t sweep_seed = p_.seed_mode == MBIR_SEED_FIXED
                                    ? p_.seed
                                    : p_.seed + static_cast<uint32_t>(sweeps_done_);
    std::vector<int32_t> lines;
    reference_visit_order(sweep_seed, g.n_z, g.n_x, lines);
    call_lines_ = lines;
    cudaMemcpyAsync(d_lines_, lines.data(), sizeof(int32_t) * lines.size(), cudaMemcpyHostToDevice, s);
    if (exact_) {
      ExactArgs ea = exact_args();
      ea.lines = d_lines_;
      ea.n_lines = static_cast<int>(lines.size());
      ea.iter_nonzero = iter_nonzero;
      ea.zero_skipping = p_.zero_skipping;
      ea.stats = d_stat4_;
      if ((rc = launch_exact_icd(ea, s))) return cuda_check(rc, "reference-order sweep (exact)");
    } else {
    RefOrderArgs a{};
    a.g = dg_;
    a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_, d_lineok_};
    a.flt = flt_;
    a.x = d_x_;
    a.e = d_e_;
    a.lines = d_lines_;
    a.n_lines = static_cast<int>(lines.size());
    a.iter_nonzero = iter_nonzero;
    a.zero_skipping = p_.zero_skipping;
    a.fp64 = fp64_;
    a.stats = d_stat4_;
    if (bright_field_assisted()) {
      a.bf = 1;
      a.bfa = bfa_sweep_args();
    }
    if ((rc = launch_ref_order(a, nb_, s))) return cuda_check(rc, "reference-order sweep");
    }
  } else {
    std::vector<int32_t> rows;
    row_order_for_sweep(sweeps_done_, rows);
    cudaMemcpyAsync(d_rows_, rows.data(), sizeof(int) * g.n_z, cudaMemcpyHostToDevice, s);
    SweepArgs a{};
    a.g = dg_;
    a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_, d_lineok_};
    a.flt = flt_;
    a.x = d_x_;
    a.e = d_e_;
    a.row_order = d_rows_;
    a.stride = stride_;
    a.mode = kModeICD;
    a.fp64 = fp64_;
    a.iter_nonzero = iter_nonzero;
    a.zero_skipping = p_.zero_skipping;
    a.smem_rows = stage_ ? 1 : 0;
    a.n_rs = stage_ ? n_rs_ : 0;
    a.shape = shape_;
    a.err = d_err_;
    if (bright_field_assisted()) {
      a.bf = 1;
      a.bfa = bfa_sweep_args();
    }
    const int n0 = (g.n_y + 1) / 2;
    cudaEventRecord(static_cast<cudaEvent_t>(ev2_), s);
    for (int colour = 0; colour < 2; colour++) {
      a.colour = colour;
      a.n_slices = (g.n_y - colour + 1) / 2;
      a.stats = d_stats_ + (colour ? static_cast<size_t>(n0) * kStatSlots : 0);
      if (a.n_slices <= 0) continue;
      if ((rc = launch_sweep(a, nb_, smem_bytes_, s))) return cuda_check(rc, "ICD sweep launch");
    }
    cudaEventRecord(static_cast<cudaEvent_t>(ev3_), s);
    kernel_timed_ = true;
    if ((rc = launch_reduce_stats(d_stats_, g.n_y, kStatSlots, d_stat4_, s)))
      return cuda_check(rc, "stats reduce");
  }
  cudaEventRecord(static_cast<cudaEvent_t>(ev1_), s);
  double st[kStatSlots];
  cudaMemcpyAsync(st, d_stat4_, sizeof(st), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "ICD sweep");
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
  if (stats4)
    for (int i = 0; i < 4; i++) stats4[i] = st[i];
  return MBIR_OK;
}

ExactArgs Engine::exact_args() {
  const Geometry& g = g_;
  ExactArgs a{};
  a.g = dg_;
  a.flt = flt_;
  a.x0 = g.x0;
  a.z0 = g.z0;
  a.delta_xz = g.delta_xz;
  a.delta_r = g.delta_r;
  a.R0 = g.R0;
  a.RMax = g.RMax;
  a.offset_r = g.offset_r;
  a.cosv = d_cosv_;
  a.sinv = d_sinv_;
  a.H = d_Href_;
  a.gain = d_gain_;
  a.weight = d_wv_;
  a.t_first = d_tfirst_;
  a.t_count = d_tcount_;
  a.hval = static_cast<const double*>(d_hval_);
  a.lineok = d_lineok_;
  a.x = static_cast<double*>(d_x_);
  a.e = static_cast<double*>(d_e_);
  a.bfm = bright_field_assisted() ? static_cast<const double*>(d_bfm_) : nullptr;
  return a;
}

int Engine::batch_args(int outer, int inner, SweepArgs* out, size_t* smem_needed) {
  if (state_ < 2) return fail(MBIR_ESTATE, "batch: engine not prepared");
  if (fp64_ || p_.order_mode != MBIR_ORDER_PARALLEL)
    return fail(MBIR_ENOTSUP, "batch: FP32 parallel-order engines only");
  if (bright_field_assisted())
    return fail(MBIR_ENOTSUP, "batch: HAADF with bright-field data runs alone");
  if (g_.n_theta > kMaxViewsShaped)
    return fail(MBIR_ENOTSUP, "batch: series of at most 160 views");
  const Geometry& g = g_;
  std::vector<int32_t> rows;
  row_order_for_sweep(sweeps_done_, rows);
  if (cudaMemcpy(d_rows_, rows.data(), sizeof(int) * g.n_z, cudaMemcpyHostToDevice) != cudaSuccess)
    return cuda_check(MBIR_EDEVICE, "batch row order");
  SweepArgs a{};
  a.g = dg_;
  a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_, d_lineok_};
  a.flt = flt_;
  a.x = d_x_;
  a.e = d_e_;
  a.row_order = d_rows_;
  a.stride = stride_;
  a.mode = kModeICD;
  a.fp64 = 0;
  a.iter_nonzero = (inner > 0 || outer > 0) ? 1 : 0;
  a.zero_skipping = p_.zero_skipping;
  a.smem_rows = stage_ ? 1 : 0;
  a.n_rs = stage_ ? n_rs_ : 0;
  a.shape = shape_;
  a.err = d_err_;
  a.stats = d_stats_;
  a.colour = 0;
  if (bf_) {  // this call's NHICD list, active mask and magnitude reset, its level schedule
    int rc = bf_call_begin(outer, inner, &a.bfa);
    if (rc) return rc;
    a.bf = 1;
    if ((rc = bf_schedule(rows, a))) return rc;
    if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream_)) != cudaSuccess)
      return cuda_check(MBIR_EDEVICE, "batch schedule upload");
  }
  a.n_slices = (g.n_y + 1) / 2;
  *out = a;
  if (smem_needed) *smem_needed = smem_bytes_;
  return MBIR_OK;
}

int Engine::batch_finish(int outer, int inner, const double* st, double ms) {
  if (bf_) {
    int rc = bf_call_end();
    if (rc) return rc;
    if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream_)) != cudaSuccess)
      return cuda_check(MBIR_EDEVICE, "batch call end");
    bf_schedule_settle();
  }
  icd_ms_ += ms;
  sweeps_done_++;
  visited_ += static_cast<int64_t>(st[2] + st[3]);
  updated_ += static_cast<int64_t>(st[3]);
  last_rel_ = st[1] > 0 ? st[0] / st[1] : 0.0;
  outer_ = outer;
  inner_ = inner;
  return MBIR_OK;
}

// jointEstimation, gain + offset branch (HAADF_ReconstructionEngine_Extra.cpp:419-636)
int Engine::joint_estimation() {
  if (state_ < 2) return fail(MBIR_ESTATE, "joint_estimation: call prepare first");
  if (bf_) return bf_joint_estimation();
  if (bright_field_assisted()) return bfa_offsets();
  const Geometry& g = g_;
  const int nt = g.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc = exact_ ? launch_exact_view_sums(exact_args(), 0, static_cast<const double*>(d_y_), d_mu_,
                                           d_vsum_, s)
                 : launch_view_sums(0, d_y_, d_e_, d_mu_, d_gain_, d_wv_, d_partial_, d_vsum_, nt,
                                    n_rp_, g.n_r, g.n_t, n_chunk_, fp64_, s);
  if (rc) return cuda_check(rc, "joint estimation sums");
  std::vector<double> vs(static_cast<size_t>(nt) * 6);
  cudaMemcpyAsync(vs.data(), d_vsum_, sizeof(double) * vs.size(), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "joint estimation");
  std::vector<double> Q0(nt), Q1(nt), b0(nt), d1(nt), d2(nt);
  for (int v = 0; v < nt; v++) {
    const double num = vs[v * 6 + 0], den = vs[v * 6 + 1], a = vs[v * 6 + 2], b = vs[v * 6 + 3],
                 d = vs[v * 6 + 5];
    Q0[v] = d;
    Q1[v] = a;
    b0[v] = b;
    d1[v] = num / den;
    d2[v] = a / den;
  }
  double sum1 = 0, sum2 = 0;
  for (int v = 0; v < nt; v++) {
    sum1 += (1.0 / (Q0[v] - Q1[v] * d2[v]));
    sum2 += ((b0[v] - Q1[v] * d1[v]) / (Q0[v] - Q1[v] * d2[v]));
  }
  const double lm = (-nt * p_.target_gain + sum2) / sum1;
  std::vector<double> In(nt), Mn(nt);
  for (int v = 0; v < nt; v++) {
    In[v] = (-1 * lm - Q1[v] * d1[v] + b0[v]) / (Q0[v] - Q1[v] * d2[v]);
    Mn[v] = d1[v] - d2[v] * In[v];
  }
  cudaMemcpyAsync(d_mu2_, Mn.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_gain2_, In.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  rc = launch_rebuild_error(d_y_, d_e_, d_mu_, d_gain_, d_mu2_, d_gain2_, nt, n_rp_, g.n_r, g.n_t,
                            fp64_, s);
  if (rc) return cuda_check(rc, "rebuild error sinogram");
  I_ = In;
  mu_ = Mn;
  return upload_views();
}

// updateWeights (HAADF_ReconstructionEngine_Extra.cpp:795-881), IDENTITY_NOISE_MODEL
int Engine::update_weights() {
  if (state_ < 2) return fail(MBIR_ESTATE, "update_weights: call prepare first");
  if (bf_) return bf_update_weights();
  const Geometry& g = g_;
  const int nt = g.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const bool scaled = bright_field_assisted() && !exact_;  // e / m in d_e_
  int rc = exact_ ? launch_exact_view_sums(exact_args(), 1, static_cast<const double*>(d_y_), d_mu_,
                                           d_vsum_, s)
           : scaled ? launch_bfa_sums(1, d_bfm_, d_e_, d_partial_, d_vsum_, nt, n_rp_, g.n_r,
                                      g.n_t, n_chunk_, fp64_, s)
                    : launch_view_sums(1, d_y_, d_e_, d_mu_, d_gain_, d_wv_, d_partial_, d_vsum_,
                                       nt, n_rp_, g.n_r, g.n_t, n_chunk_, fp64_, s);
  if (rc) return cuda_check(rc, "variance sums");
  std::vector<double> vs(nt);
  cudaMemcpyAsync(vs.data(), d_vsum_, sizeof(double) * nt, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "update weights");
  for (int v = 0; v < nt; v++) {
    alpha_[v] = vs[v] / (g.n_r * g.n_t);
    w_[v] = 1.0 / alpha_[v];
  }
  if ((rc = upload_views())) return rc;
  if (scaled) {
    rc = launch_bfa_weights(d_bfm_, d_wv_, d_w_, nt, n_rp_, g.n_r, g.n_t, fp64_, s);
    if (rc) return cuda_check(rc, "bright-field weights");
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "update weights");
  }
  return MBIR_OK;
}

// jointEstimation with bright-field data (HAADF_ReconstructionEngine_Extra.cpp:429, :643-668):
// the offsets only, per view the weighted mean of the error taken off the error
int Engine::bfa_offsets() {
  const Geometry& g = g_;
  const int nt = g.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc;
  if (exact_) {
    cudaMemcpyAsync(d_mu2_, mu_.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
    if ((rc = launch_exact_bfa_offsets(exact_args(), d_mu2_, s)))
      return cuda_check(rc, "offset estimation (exact)");
    cudaMemcpyAsync(mu_.data(), d_mu2_, sizeof(double) * nt, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "offsets");
    return upload_views();
  }
  // the weights are one value per view, so the weighted mean is sum(m e') / (N_r N_t)
  if ((rc = launch_bfa_sums(0, d_bfm_, d_e_, d_partial_, d_vsum_, nt, n_rp_, g.n_r, g.n_t,
                            n_chunk_, fp64_, s)))
    return cuda_check(rc, "offset sums");
  std::vector<double> vs(nt);
  cudaMemcpyAsync(vs.data(), d_vsum_, sizeof(double) * nt, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "offsets");
  std::vector<double> step(nt);
  for (int v = 0; v < nt; v++) {
    step[v] = vs[v] / (static_cast<double>(g.n_r) * g.n_t);
    mu_[v] += step[v];
  }
  cudaMemcpyAsync(d_mu2_, step.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  if ((rc = launch_bfa_offset_apply(d_bfm_, d_e_, d_mu2_, nt, n_rp_, g.n_r, g.n_t, fp64_, s)))
    return cuda_check(rc, "offset step");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "offsets");
  return upload_views();
}

// computeCost (HAADF_ReconstructionEngine.cpp:1147-1364): data + prior + noise terms
int Engine::compute_cost(double* parts3, double* total) {
  if (state_ < 2) return fail(MBIR_ESTATE, "compute_cost: call prepare first");
  if (bf_) return bf_compute_cost(parts3, total);
  const Geometry& g = g_;
  const int nt = g.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc = (bright_field_assisted() && !exact_)
               ? launch_bfa_sums(1, d_bfm_, d_e_, d_partial_, d_vsum_, nt, n_rp_, g.n_r, g.n_t,
                                 n_chunk_, fp64_, s)
               : launch_view_sums(1, d_y_, d_e_, d_mu_, d_gain_, d_wv_, d_partial_, d_vsum_, nt,
                                  n_rp_, g.n_r, g.n_t, n_chunk_, fp64_, s);
  if (rc) return cuda_check(rc, "cost data term");
  double* prior_partial = d_partial_ + static_cast<size_t>(nt) * n_chunk_ * 6;
  rc = launch_prior_cost(d_x_, flt_, g.n_z, g.n_x, g.n_y, prior_partial, prior_blocks_, fp64_,
                         s);
  if (rc) return cuda_check(rc, "cost prior term");
  std::vector<double> vs(nt), pp(prior_blocks_);
  cudaMemcpyAsync(vs.data(), d_vsum_, sizeof(double) * nt, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(pp.data(), prior_partial, sizeof(double) * prior_blocks_, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "cost");
  double data = 0, prior = 0, noise = 0;
  for (int v = 0; v < nt; v++) data += vs[v] * w_[v];
  data /= 2;
  for (double x : pp) prior += x;
  if (p_.noise_model) {
    for (int v = 0; v < nt; v++)
      if (w_[v] != 0) noise += static_cast<double>(g.n_r) * g.n_t * std::log(2 * kPi * (1.0 / w_[v]));
    noise /= 2;
  }
  if (parts3) {
    parts3[0] = data;
    parts3[1] = prior;
    parts3[2] = noise;
  }
  const double c = data + prior + noise;
  if (total) *total = c;
  last_cost_ = c;
  return MBIR_OK;
}

// HAADF_ReconstructionEngine::execute outer/inner loop (HAADF_ReconstructionEngine.cpp:706-815)
int Engine::run() {
  const auto t0 = std::chrono::steady_clock::now();
  int rc = prepare();
  if (rc) return rc;
  state_ = 3;
  if (bf_) {
    if ((rc = bf_run())) return rc;
    state_ = 4;
    total_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    notify("Reconstruction Complete", 100, MBIR_UPDATE_PROGRESS_VALUE_AND_MESSAGE);
    return MBIR_OK;
  }
  // a resumed run continues at the checkpoint's outer iteration and stop threshold
  double stop = stop_now_;
  for (int outer = outer_next_; outer < p_.outer_iterations; outer++) {
    const int num_iter = outer == 0 ? p_.inner_iterations : 1;
    int status = 1;
    for (int inner = 0; inner < num_iter; inner++) {
      double st[4];
      if ((rc = sweep(outer, inner, st))) return rc;
      // the intermediate image of every inner iteration (HAADF_ReconstructionEngine.cpp:757-763)
      if (!interm_dir_.empty()) {
        const std::string image = interm_dir_ + "/" + std::to_string(outer) + "_" +
                                  std::to_string(inner) + "_ReconstructedVolume.rec";
        if ((rc = write_volume_mrc(image))) return rc;
        notify(image, 0, MBIR_UPDATE_INTERMEDIATE_IMAGE);
      }
      if (p_.cost_every_sweep && (rc = compute_cost(nullptr, nullptr))) return rc;
      status = 1;
      if (st[1] > 0 && (st[0] / st[1]) < stop) {
        stop *= p_.threshold_reduction_factor;
        status = 0;
        break;
      }
    }
    if (cancel_.load()) return fail(MBIR_ECANCELLED, "cancelled");
    if (p_.joint_estimation && (rc = joint_estimation())) return rc;
    if (p_.noise_model && (rc = update_weights())) return rc;
    outer_next_ = outer + 1;
    stop_now_ = stop;
    notify_iteration(outer);
    if (status == 0 && outer >= 1) break;
  }
  state_ = 4;
  total_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  notify("Reconstruction Complete", 100, MBIR_UPDATE_PROGRESS_VALUE_AND_MESSAGE);
  return MBIR_OK;
}

int Engine::dims(int32_t* d) const {
  if (state_ < 1) return MBIR_ESTATE;
  Engine* self = const_cast<Engine*>(this);
  if (g_.n_x == 0) {
    int rc = self->build_geometry();
    if (rc) return rc;
  }
  d[0] = g_.n_z;
  d[1] = g_.n_x;
  d[2] = g_.n_y;
  d[3] = g_.n_theta;
  d[4] = g_.n_r;
  d[5] = g_.n_t;
  return MBIR_OK;
}

int Engine::get_volume(float* out, int64_t n) {
  if (state_ < 2) return fail(MBIR_ESTATE, "get_volume: nothing reconstructed");
  const Geometry& g = g_;
  const size_t nv = static_cast<size_t>(g.n_z) * g.n_x * g.n_y;
  if (!out || n < static_cast<int64_t>(nv)) return fail(MBIR_EINVAL, "get_volume: buffer too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc = launch_vol_to_host(d_x_, d_stage_, g.n_z, g.n_x, g.n_y, fp64_, s);
  if (rc) return cuda_check(rc, "volume read-out");
  cudaMemcpyAsync(out, d_stage_, sizeof(float) * nv, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : cuda_check(MBIR_EDEVICE, "volume read-out");
}

// The volume as doubles, [z][x][y] (an FP64 engine's values exactly)
int Engine::get_volume_f64(double* out, int64_t n) {
  if (state_ < 2) return fail(MBIR_ESTATE, "get_volume: nothing reconstructed");
  const Geometry& g = g_;
  const size_t nv = static_cast<size_t>(g.n_z) * g.n_x * g.n_y;
  if (!out || n < static_cast<int64_t>(nv)) return fail(MBIR_EINVAL, "get_volume: buffer too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  std::vector<unsigned char> raw(nv * rb_);
  cudaMemcpyAsync(raw.data(), d_x_, raw.size(), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "volume read-out");
  for (int y = 0; y < g.n_y; y++)
    for (int z = 0; z < g.n_z; z++)
      for (int x = 0; x < g.n_x; x++) {
        const size_t i = (static_cast<size_t>(y) * g.n_z + z) * g.n_x + x;
        const double v = fp64_ ? reinterpret_cast<const double*>(raw.data())[i]
                               : static_cast<double>(reinterpret_cast<const float*>(raw.data())[i]);
        out[(static_cast<size_t>(z) * g.n_x + x) * g.n_y + y] = v;
      }
  return MBIR_OK;
}

static int sino_readout(Engine* eng, const void* dsrc, float* stage, float* out, int64_t n,
                        const Geometry& g, int n_rp, int fp64, void* stream) {
  const size_t nh = static_cast<size_t>(g.n_theta) * g.n_r * g.n_t;
  if (!out || n < static_cast<int64_t>(nh)) return eng->fail(MBIR_EINVAL, "buffer too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (launch_sino_to_host(dsrc, stage, g.n_theta, g.n_r, n_rp, g.n_t, fp64, s))
    return eng->fail(MBIR_EDEVICE, "sinogram read-out");
  cudaMemcpyAsync(out, stage, sizeof(float) * nh, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : eng->fail(MBIR_EDEVICE, "sinogram read-out");
}

int Engine::get_error(float* out, int64_t n) {
  if (state_ < 2) return fail(MBIR_ESTATE, "get_error: call prepare first");
  const int rc = sino_readout(this, d_e_, d_stage_, out, n, g_, n_rp_, fp64_, stream_);
  if (rc || !bright_field_assisted() || exact_) return rc;
  // the parallel engines keep e / m on the device (mbir_bfassist.cu)
  for (size_t i = 0; i < bfm_.size() && static_cast<int64_t>(i) < n; i++)
    out[i] = static_cast<float>(static_cast<double>(out[i]) * bfm_[i]);
  return MBIR_OK;
}
int Engine::get_projection(float* out, int64_t n) {
  if (state_ < 2) return fail(MBIR_ESTATE, "get_projection: call prepare first");
  return sino_readout(this, d_yest_, d_stage_, out, n, g_, n_rp_, fp64_, stream_);
}

int Engine::get_nuisance(double* gg, double* o, double* v) {
  if (!host_ready_) {
    const int rc = build_host();
    if (rc) return rc;
  }
  const int nt = g_.n_theta;
  if (gg) std::copy(I_.begin(), I_.begin() + nt, gg);
  if (o) std::copy(mu_.begin(), mu_.begin() + nt, o);
  if (v) std::copy(alpha_.begin(), alpha_.begin() + nt, v);
  return MBIR_OK;
}

int Engine::get_tables(double* H, double* Ht) {
  if (!host_ready_) {
    const int rc = build_host();
    if (rc) return rc;
  }
  if (H) std::copy(tab_.H.begin(), tab_.H.end(), H);
  if (Ht) std::copy(tab_.Ht.begin(), tab_.Ht.end(), Ht);
  return MBIR_OK;
}

int Engine::get_schedule(int sweep, int32_t* row_order, int32_t* stride) {
  if (!host_ready_) {
    const int rc = build_host();
    if (rc) return rc;
  }
  std::vector<int32_t> rows;
  row_order_for_sweep(sweep, rows);
  if (row_order) std::copy(rows.begin(), rows.end(), row_order);
  if (stride) *stride = stride_;
  return MBIR_OK;
}

int Engine::status(mbir_status* st) const {
  if (!st) return MBIR_EINVAL;
  st->state = state_;
  st->outer_iter = outer_;
  st->inner_iter = inner_;
  st->sweeps_done = sweeps_done_;
  st->last_cost = last_cost_;
  st->last_rel_update = last_rel_;
  st->icd_ms_total = icd_ms_;
  st->total_ms = total_ms_;
  st->voxels_visited = visited_;
  st->voxels_updated = updated_;
  st->footprint_entries = footprint_entries_;
  st->t_rows = t_rows_;
  st->stride = stride_;
  st->staged = stage_ ? 1 : 0;
  st->lane_shape = shape_;
  st->sched_levels = n_levels_;
  st->sched_ms_total = sched_ms_;
  st->kernel_ms_total = kernel_ms_;
  st->colour_ms_total = colour_ms_;
  return MBIR_OK;
}

int Engine::set_intermediate_dir(const char* dir) {
  interm_dir_ = dir ? dir : "";
  return MBIR_OK;
}

int Engine::set_observer(mbir_observer_fn fn, void* user) {
  observer_ = fn;
  observer_user_ = fn ? user : nullptr;
  return MBIR_OK;
}

namespace {
// Checkpoint.bin: this header, then the error sinogram's bytes in the engine's device layout
// ([t][theta][r padded to n_rp], FP32 or FP64)
struct CheckpointHeader {
  char magic[8];
  int32_t v[16];  // kCk* fields below
  double stop;
  uint64_t e_bytes;
};
constexpr char kCheckpointMagic[8] = {'M', 'B', 'I', 'R', 'C', 'K', 'P', '1'};
enum {
  kCkModality, kCkPrecision, kCkExact, kCkOrder, kCkNz, kCkNx, kCkNy, kCkNtheta, kCkNr, kCkNt,
  kCkNrp, kCkElem, kCkOuterNext, kCkSweeps, kCkFields
};

bool read_doubles(const std::string& path, std::vector<double>& out, size_t n) {
  out.assign(n, 0.0);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  const size_t got = std::fread(out.data(), sizeof(double), n, f);
  const bool at_end = std::fgetc(f) == EOF;
  std::fclose(f);
  return got == n && at_end;
}
}  // namespace

// Writes the run's state to dir: ReconstructedObject.bin, Final{Gain,Offset}Parameters.bin,
// FinalVariances.bin (the reference's level hand-off files, read back the way
// HAADF_MultiResolutionReconstruction.cpp:212-222 reads them) and Checkpoint.bin (outer
// iterations done, sweeps done, stop threshold, error sinogram).
int Engine::write_checkpoint(const char* dir) {
  if (state_ < 2) return fail(MBIR_ESTATE, "write_checkpoint: call prepare first");
  if (bf_ || bright_field_assisted())
    return fail(MBIR_ENOTSUP, "write_checkpoint: HAADF without bright-field data only");
  int rc = write_outputs(dir, nullptr);
  if (rc) return rc;
  const Geometry& g = g_;
  const size_t bytes = static_cast<size_t>(g.n_t) * g.n_theta * n_rp_ * rb_;
  std::vector<unsigned char> e(bytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  cudaMemcpyAsync(e.data(), d_e_, bytes, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "checkpoint read-out");
  CheckpointHeader h{};
  std::memcpy(h.magic, kCheckpointMagic, sizeof h.magic);
  const int32_t fields[kCkFields] = {
      bf_ ? MBIR_MODALITY_BF : MBIR_MODALITY_HAADF, fp64_ ? 1 : 0, exact_ ? 1 : 0,
      p_.order_mode, g.n_z, g.n_x, g.n_y, g.n_theta, g.n_r, g.n_t, n_rp_,
      static_cast<int32_t>(rb_), outer_next_, sweeps_done_};
  std::memcpy(h.v, fields, sizeof fields);
  h.stop = stop_now_;
  h.e_bytes = bytes;
  const std::string path = std::string(dir ? dir : ".") + "/Checkpoint.bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return fail(MBIR_EIO, "cannot write " + path);
  const bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 &&
                  std::fwrite(e.data(), 1, bytes, f) == bytes;
  if (std::fclose(f) != 0 || !ok) return fail(MBIR_EIO, "cannot write " + path);
  return MBIR_OK;
}

// Reads a checkpoint written by an engine of the same configuration and series; every later
// prepare starts from it (volume, gains, offsets, variances, error sinogram, sweep count) and
// mbir_run continues at its outer iteration.
int Engine::read_checkpoint(const char* dir) {
  if (state_ < 1) return fail(MBIR_ESTATE, "read_checkpoint: set the sinogram first");
  if (bf_ || bright_field_assisted())
    return fail(MBIR_ENOTSUP, "read_checkpoint: HAADF without bright-field data only");
  int rc;
  if (g_.n_y == 0 && (rc = build_geometry())) return rc;
  const Geometry& g = g_;
  const std::string d = dir ? dir : ".";
  const std::string path = d + "/Checkpoint.bin";
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(MBIR_EIO, "cannot read " + path);
  CheckpointHeader h{};
  const bool got = std::fread(&h, sizeof h, 1, f) == 1;
  int32_t v[kCkFields];
  std::memcpy(v, h.v, sizeof v);
  const int32_t want[kCkNrp] = {
      MBIR_MODALITY_HAADF, fp64_ ? 1 : 0, exact_ ? 1 : 0, p_.order_mode, g.n_z, g.n_x, g.n_y,
      g.n_theta, g.n_r, g.n_t};
  if (!got || std::memcmp(h.magic, kCheckpointMagic, sizeof h.magic) != 0) {
    std::fclose(f);
    return fail(MBIR_EIO, path + " is not a checkpoint");
  }
  // the error sinogram's size follows from the series: rows padded as alloc_device pads them
  const int32_t n_rp = (g.n_r + 3) / 4 * 4;
  const uint64_t e_bytes = static_cast<uint64_t>(g.n_t) * g.n_theta * n_rp * rb_;
  if (std::memcmp(v, want, sizeof want) != 0 || v[kCkElem] != static_cast<int32_t>(rb_) ||
      v[kCkNrp] != n_rp || v[kCkOuterNext] < 0 || v[kCkSweeps] < 0 || h.e_bytes != e_bytes) {
    std::fclose(f);
    return fail(MBIR_EINVAL, "checkpoint: written by an engine of another configuration or series");
  }
  std::vector<unsigned char> e(static_cast<size_t>(h.e_bytes));
  const bool got_e = std::fread(e.data(), 1, e.size(), f) == e.size();
  std::fclose(f);
  if (!got_e) return fail(MBIR_EIO, path + " is truncated");
  const size_t nv = static_cast<size_t>(g.n_z) * g.n_x * g.n_y;
  std::vector<double> yxz, gain, offset, var;
  if (!read_doubles(d + "/ReconstructedObject.bin", yxz, nv) ||
      !read_doubles(d + "/FinalGainParameters.bin", gain, g.n_theta) ||
      !read_doubles(d + "/FinalOffsetParameters.bin", offset, g.n_theta) ||
      !read_doubles(d + "/FinalVariances.bin", var, g.n_theta))
    return fail(MBIR_EIO, "checkpoint: a .bin file is missing or of the wrong size in " + d);
  // ReconstructedObject.bin is y-x-z; the engine's initial volume [z][x][y], taken as it is
  // (no 2x2x2 interpolation)
  init_vol_.assign(nv, 0.0);
  size_t k = 0;
  for (int y = 0; y < g.n_y; ++y)
    for (int x = 0; x < g.n_x; ++x)
      for (int z = 0; z < g.n_z; ++z) init_vol_[(static_cast<size_t>(z) * g.n_x + x) * g.n_y + y] = yxz[k++];
  resume_e_ = std::move(e);
  resume_gain_ = std::move(gain);
  resume_offset_ = std::move(offset);
  resume_var_ = std::move(var);
  resume_outer_ = v[kCkOuterNext];
  resume_sweeps_ = v[kCkSweeps];
  resume_stop_ = h.stop;
  resume_ = true;
  host_ready_ = false;
  return MBIR_OK;
}

// computeOriginalXDims (_Extra.cpp:252-275): the columns whose centres lie on the detector
static void original_x_dims(const Geometry& g, int& crop_start, int& crop_end) {
  crop_start = 0;
  crop_end = g.n_x;
  for (int j = 0; j < g.n_x; j++) {
    const double x = g.x0 + ((double)j + 0.5) * g.delta_xz;
    if (x >= -(g.n_r * g.delta_r) / 2 && x <= (g.n_r * g.delta_r) / 2) {
      crop_start = j;
      break;
    }
  }
  for (int j = g.n_x - 1; j >= 0; j--) {
    const double x = g.x0 + ((double)j + 0.5) * g.delta_xz;
    if (x >= -(g.n_r * g.delta_r) / 2 && x <= (g.n_r * g.delta_r) / 2) {
      crop_end = j;
      break;
    }
  }
}

// writeMRCFile(path, cropStart, cropEnd) of the current volume (HAADF_ForwardModel.cpp:176-245)
int Engine::write_volume_mrc(const std::string& path) {
  const Geometry& g = g_;
  std::vector<float> vol(static_cast<size_t>(g.n_z) * g.n_x * g.n_y);
  int rc = get_volume(vol.data(), static_cast<int64_t>(vol.size()));
  if (rc) return rc;
  int crop_start = 0, crop_end = g.n_x;
  original_x_dims(g, crop_start, crop_end);
  std::string err;
  if (mrc_write_volume(path, vol.data(), g.n_z, g.n_x, g.n_y, crop_start, crop_end + 1,
                       g.length_x, err))
    return fail(MBIR_EIO, err);
  return MBIR_OK;
}

int Engine::write_outputs(const char* dir, const char* mrc_path, const char* vtk_path,
                          const char* avizo_path) {
  if (state_ < 2) return fail(MBIR_ESTATE, "write_outputs: nothing reconstructed");
  const Geometry& g = g_;
  const size_t nv = static_cast<size_t>(g.n_z) * g.n_x * g.n_y;
  std::vector<float> vol(nv);
  int rc = get_volume(vol.data(), static_cast<int64_t>(nv));
  if (rc) return rc;
  std::string d = dir ? dir : ".";
  // ReconstructedObject.bin: doubles in y-x-z order (RawGeometryWriter.cpp:83-91), an FP64
  // engine's values exactly
  {
    std::vector<double> v64(nv);
    if ((rc = get_volume_f64(v64.data(), static_cast<int64_t>(nv)))) return rc;
    FILE* f = std::fopen((d + "/ReconstructedObject.bin").c_str(), "wb");
    if (!f) return fail(MBIR_EIO, "cannot write ReconstructedObject.bin");
    std::vector<double> buf;
    buf.reserve(nv);
    for (int y = 0; y < g.n_y; ++y)
      for (int x = 0; x < g.n_x; ++x)
        for (int z = 0; z < g.n_z; z++) buf.push_back(v64[(static_cast<size_t>(z) * g.n_x + x) * g.n_y + y]);
    std::fwrite(buf.data(), sizeof(double), buf.size(), f);
    std::fclose(f);
  }
  // nuisance parameters: raw double[N_theta] (NuisanceParamWriter.cpp:136)
  const char* names[3] = {"/FinalGainParameters.bin", "/FinalOffsetParameters.bin",
                          "/FinalVariances.bin"};
  const std::vector<double>* vecs[3] = {&I_, &mu_, &alpha_};
  for (int i = 0; i < 3; i++) {
    FILE* f = std::fopen((d + names[i]).c_str(), "wb");
    if (!f) return fail(MBIR_EIO, std::string("cannot write ") + names[i]);
    std::fwrite(vecs[i]->data(), sizeof(double), g.n_theta, f);
    std::fclose(f);
  }
  // ReconstructedSinogram.bin: (y - e) * I + mu per entry, [theta][r][t] doubles, y the
  // measurements the engine works on (bright field: after -log) (execute :861-875,
  // SinogramBinWriter.cpp:115-126)
  {
    const size_t ns = static_cast<size_t>(g.n_theta) * g.n_r * g.n_t;
    std::vector<float> e(ns);
    if ((rc = get_error(e.data(), static_cast<int64_t>(ns)))) return rc;
    FILE* f = std::fopen((d + "/ReconstructedSinogram.bin").c_str(), "wb");
    if (!f) return fail(MBIR_EIO, "cannot write ReconstructedSinogram.bin");
    std::vector<double> buf(static_cast<size_t>(g.n_r) * g.n_t);
    for (int th = 0; th < g.n_theta; ++th) {
      for (size_t k = 0; k < buf.size(); ++k) {
        const size_t i = static_cast<size_t>(th) * buf.size() + k;
        const double y = bf_ ? ylog_[i] : static_cast<double>(counts_[i]);
        buf[k] = (y - static_cast<double>(e[i])) * I_[th] + mu_[th];
      }
      std::fwrite(buf.data(), sizeof(double), buf.size(), f);
    }
    std::fclose(f);
  }
  // the VTK file takes [start, end) of the original x dims, the MRC and Avizo files
  // [start, end] (execute :879-901)
  int crop_start = 0, crop_end = g.n_x;
  original_x_dims(g, crop_start, crop_end);
  std::string err;
  if (vtk_path && vtk_path[0] &&
      vtk_write_volume(vtk_path, vol.data(), g.n_z, g.n_x, g.n_y, crop_start, crop_end, err))
    return fail(MBIR_EIO, err);
  if (mrc_path && mrc_path[0] &&
      mrc_write_volume(mrc_path, vol.data(), g.n_z, g.n_x, g.n_y, crop_start, crop_end + 1,
                       g.length_x, err))
    return fail(MBIR_EIO, err);
  if (avizo_path && avizo_path[0] &&
      avizo_write_volume(avizo_path, vol.data(), g.n_z, g.n_x, g.n_y, crop_start, crop_end + 1,
                         g.delta_xy, g.delta_xz, err))
    return fail(MBIR_EIO, err);
  return MBIR_OK;
}

// Autotuner of the FP32 voxel-group shape (lanes per voxel x views per lane).  When more than one
// shape covers the view count, each candidate runs one trial ICD pass (both colours, every
// line, the current state) on a snapshot of the volume, error sinogram and selector; the state
// is restored after every trial and the fastest candidate is kept.  Choices are cached per
// (views, x, z, y, footprint bins, modality, staging) for the life of the process, so engines of
// the same geometry tune once.
namespace {
std::mutex g_tune_mu;
std::map<std::vector<int>, int> g_tune_cache;
}  // namespace

int Engine::autotune_shape() {
  if (fp64_ || p_.order_mode != MBIR_ORDER_PARALLEL || bright_field_assisted()) return MBIR_OK;
  const Geometry& g = g_;
  std::vector<int> cands;
  for (int sh = 1; sh <= 4; sh++)
    if (g.n_theta <= shape_max_views(sh) && (sh == 1 || sh == 2 || g.n_theta > shape_max_views(sh - 1)))
      cands.push_back(sh);
  if (nb_ == 9 || cands.size() < 2) return MBIR_OK;
  const std::vector<int> key = {g.n_theta, g.n_x, g.n_z, g.n_y, nb_, bf_ ? 1 : 0, stage_ ? 1 : 0};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      shape_ = it->second;
      return MBIR_OK;
    }
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nvb = static_cast<size_t>(g.n_z) * g.n_x * g.n_y * rb_;
  const size_t neb = static_cast<size_t>(g.n_t) * g.n_theta * n_rp_ * rb_;
  const size_t nsb = bf_ ? static_cast<size_t>(g.n_t) * g.n_theta * n_sp_ : 0;
  const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
  void *sx = nullptr, *se = nullptr, *ss = nullptr, *sm = nullptr;
  if (cudaMalloc(&sx, nvb) != cudaSuccess || cudaMalloc(&se, neb) != cudaSuccess ||
      (nsb && cudaMalloc(&ss, nsb) != cudaSuccess) ||
      (bf_ && cudaMalloc(&sm, nl * sizeof(unsigned long long)) != cudaSuccess)) {
    cudaFree(sx);
    cudaFree(se);
    cudaFree(ss);
    cudaFree(sm);
    cudaGetLastError();
    return MBIR_OK;  // no room for a snapshot: keep the default shape
  }
  cudaMemcpyAsync(sx, d_x_, nvb, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(se, d_e_, neb, cudaMemcpyDeviceToDevice, s);
  if (nsb) cudaMemcpyAsync(ss, d_sel_, nsb, cudaMemcpyDeviceToDevice, s);
  if (bf_) {
    cudaMemcpyAsync(sm, d_magfx_, nl * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(d_active_, 1, nl, s);
  }
  std::vector<int32_t> rows(g.n_z);
  for (int i = 0; i < g.n_z; i++) rows[i] = i;
  cudaMemcpyAsync(d_rows_, rows.data(), sizeof(int) * g.n_z, cudaMemcpyHostToDevice, s);
  SweepArgs a{};
  a.g = dg_;
  a.tab = DevTables{d_H_, d_bx_, d_bxd_, d_u0_, d_bz_, d_gw_, d_tfirst_, d_tcount_, d_hval_, d_lineok_};
  a.flt = flt_;
  a.x = d_x_;
  a.e = d_e_;
  a.row_order = d_rows_;
  a.stride = stride_;
  a.mode = kModeICD;
  a.fp64 = 0;
  a.iter_nonzero = 0;
  a.zero_skipping = p_.zero_skipping;
  a.smem_rows = stage_ ? 1 : 0;
  a.n_rs = stage_ ? n_rs_ : 0;
  a.err = d_err_;
  if (bf_) {
    a.bf = 1;
    a.bfa.w = d_w_;
    a.bfa.sel = d_sel_;
    a.bfa.n_sp = n_sp_;
    a.bfa.active = d_active_;
    a.bfa.mag_fx = d_magfx_;
    a.bfa.bragg_t = bragg_t_;
    a.bfa.bragg_dt = p_.bragg_delta * bragg_t_;
  }
  const int n0 = (g.n_y + 1) / 2;
  int best = shape_;
  float best_ms = 0;
  int rc = MBIR_OK;
  // two rounds over the candidates, the best time of each kept: the first launch of a kernel
  // instantiation also loads its module, which must not count against the shape tried first
  std::vector<int> trials;
  for (int rep = 0; rep < 2; rep++) trials.insert(trials.end(), cands.begin(), cands.end());
  for (int sh : trials) {
    a.shape = sh;
    cudaEventRecord(static_cast<cudaEvent_t>(ev0_), s);
    for (int colour = 0; colour < 2 && rc == MBIR_OK; colour++) {
      a.colour = colour;
      a.n_slices = (g.n_y - colour + 1) / 2;
      a.stats = d_stats_ + (colour ? static_cast<size_t>(n0) * kStatSlots : 0);
      if (a.n_slices > 0) rc = launch_sweep(a, nb_, smem_bytes_, s);
    }
    cudaEventRecord(static_cast<cudaEvent_t>(ev1_), s);
    // restore the state for the next candidate (and for the reconstruction itself)
    cudaMemcpyAsync(d_x_, sx, nvb, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(d_e_, se, neb, cudaMemcpyDeviceToDevice, s);
    if (nsb) cudaMemcpyAsync(d_sel_, ss, nsb, cudaMemcpyDeviceToDevice, s);
    if (bf_) cudaMemcpyAsync(d_magfx_, sm, nl * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s);
    if (rc != MBIR_OK || cudaStreamSynchronize(s) != cudaSuccess) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev0_), static_cast<cudaEvent_t>(ev1_));
    if (best_ms == 0 || ms < best_ms) {
      best_ms = ms;
      best = sh;
    }
  }
  cudaFree(sx);
  cudaFree(se);
  cudaFree(ss);
  cudaFree(sm);
  if (rc != MBIR_OK) return cuda_check(rc, "shape autotune");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "shape autotune");
  if ((rc = check_device_error())) return rc;
  shape_ = best;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_cache[key] = best;
  return MBIR_OK;
}

}  // namespace mbir

