// mbir_shard.cu -- y-slab sharding of one reconstruction over several engines (one per GPU).
//
// Voxel slice y touches only its own detector rows, so a contiguous slab of slices [y0, y1)
// owns a contiguous block of the error sinogram: ICD needs no sinogram exchange between slabs.
// The prior couples neighbouring slices, so after each colour phase a slab's boundary planes
// go to its neighbours (host-mediated: get_planes / set_planes), and the per-view sums of the
// gain/offset and variance estimates are summed over slabs before the host solves them.  Bright
// field the same way, one NHICD call at a time: the call's lines come from the magnitude map,
// which the host keeps identical on every slab by summing each call's per-line magnitudes over
// the slabs; the offset and variance sums and the stop rule's volume sum are summed too.  Each
// engine holds the whole problem; only its slab is updated and summed.
#include <algorithm>
#include <vector>

#include "mbir_engine.h"

namespace mbir {

int Engine::set_slab(int y0, int y1) {
  if (state_ < 1) return fail(MBIR_ESTATE, "set_slab: no sinogram");
  if (bright_field_assisted() && !(y0 == 0 && y1 == 0))
    return fail(MBIR_ENOTSUP, "set_slab: HAADF with bright-field data runs unsharded");
  if (g_.n_y == 0) {
    int rc = build_geometry();
    if (rc) return rc;
  }
  if (y0 == 0 && y1 == 0) {
    slab_y0_ = slab_y1_ = 0;
    return MBIR_OK;
  }
  if (y0 < 0 || y1 > g_.n_y || y0 >= y1) return fail(MBIR_EINVAL, "set_slab: bad slice range");
  slab_y0_ = y0;
  slab_y1_ = y1;
  return slab_rows_owned();
}

// A slab owns its detector rows only when its edge slices share no row with the slices just
// outside it (at delta_xy = delta_t every slice has its own row; other pixel shapes let slices
// y and y+1 share one, and two slab engines would then update their own copies of that row).
// Checked once the voxel-line response exists (set_slab after prepare, or the first sweep).
int Engine::slab_rows_owned() {
  if (slab_y1_ <= 0 || static_cast<int>(tab_.t_first.size()) != g_.n_y) return MBIR_OK;
  auto shared = [&](int a, int b) {
    return tab_.t_count[a] > 0 && tab_.t_count[b] > 0 &&
           tab_.t_first[a] + tab_.t_count[a] > tab_.t_first[b];
  };
  if ((slab_y0_ > 0 && shared(slab_y0_ - 1, slab_y0_)) ||
      (slab_y1_ < g_.n_y && shared(slab_y1_ - 1, slab_y1_)))
    return fail(MBIR_ENOTSUP, "set_slab: an edge slice of the slab shares detector rows with "
                              "the slice next to it outside the slab");
  return MBIR_OK;
}

// One colour of a parallel-order sweep over the slab's slices of that colour.  Both colours of
// sweep k use the row order of sweep k; the sweep is counted after colour 1.  Bright field: one
// colour of the call opened by bf_slab_begin (its lines, schedule and row order).
int Engine::sweep_colour(int colour, int outer, int inner, double* st4) {
  if (state_ < 2) return fail(MBIR_ESTATE, "sweep_colour: call prepare first");
  if (p_.order_mode != MBIR_ORDER_PARALLEL || exact_)
    return fail(MBIR_ENOTSUP, "sweep_colour: parallel order only");
  if (bf_ && !slab_call_open_)
    return fail(MBIR_ESTATE, "sweep_colour: open a bright-field call first (bf_call_begin)");
  if (colour != 0 && colour != 1) return fail(MBIR_EINVAL, "sweep_colour: colour is 0 or 1");
  if (int rc = slab_rows_owned()) return rc;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const int y0 = slab_y1_ > 0 ? slab_y0_ : 0, y1 = slab_y1_ > 0 ? slab_y1_ : g.n_y;
  const int first = y0 + ((y0 & 1) != colour ? 1 : 0);
  const int n = first < y1 ? (y1 - first + 1) / 2 : 0;
  if (colour == 0 && !bf_) {
    std::vector<int32_t> rows;
    row_order_for_sweep(sweeps_done_, rows);
    cudaMemcpyAsync(d_rows_, rows.data(), sizeof(int) * g.n_z, cudaMemcpyHostToDevice, s);
  }
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
  a.iter_nonzero = (inner > 0 || outer > 0) ? 1 : 0;
  a.zero_skipping = p_.zero_skipping;
  a.smem_rows = stage_ ? 1 : 0;
  a.n_rs = stage_ ? n_rs_ : 0;
  a.shape = shape_;
  a.err = d_err_;
  size_t smem = smem_bytes_;
  if (bf_) {
    a = slab_args_;
    smem = slab_smem_;
  }
  a.colour = colour;
  a.y_first = first;
  a.y_end = y1;
  a.n_slices = n;
  a.stats = d_stats_;
  double st[kStatSlots] = {0, 0, 0, 0};
  int rc;
  cudaEventRecord(static_cast<cudaEvent_t>(ev0_), s);
  if (n > 0) {
    if ((rc = launch_sweep(a, nb_, smem, s))) return cuda_check(rc, "slab sweep launch");
    if ((rc = launch_reduce_stats(d_stats_, n, kStatSlots, d_stat4_, s)))
      return cuda_check(rc, "stats reduce");
    cudaMemcpyAsync(st, d_stat4_, sizeof(st), cudaMemcpyDeviceToHost, s);
  }
  cudaEventRecord(static_cast<cudaEvent_t>(ev1_), s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "slab sweep");
  if ((rc = check_device_error())) return rc;
  float ms = 0;
  cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev0_), static_cast<cudaEvent_t>(ev1_));
  icd_ms_ += ms;
  visited_ += static_cast<int64_t>(st[2] + st[3]);
  updated_ += static_cast<int64_t>(st[3]);
  if (colour == 1 && !bf_) {  // a bright-field call counts at bf_slab_end
    sweeps_done_++;
    outer_ = outer;
    inner_ = inner;
  }
  if (st4)
    for (int i = 0; i < 4; i++) st4[i] = st[i];
  return MBIR_OK;
}

int Engine::get_planes(int y, int n, float* out) {
  if (state_ < 2) return fail(MBIR_ESTATE, "get_planes: call prepare first");
  if (fp64_) return fail(MBIR_ENOTSUP, "get_planes: FP32 engines only");
  if (!out || y < 0 || n < 0 || y + n > g_.n_y) return fail(MBIR_EINVAL, "get_planes: bad range");
  const size_t plane = static_cast<size_t>(g_.n_z) * g_.n_x;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  cudaMemcpyAsync(out, static_cast<float*>(d_x_) + static_cast<size_t>(y) * plane,
                  sizeof(float) * plane * n, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK : cuda_check(MBIR_EDEVICE, "get_planes");
}

int Engine::set_planes(int y, int n, const float* in) {
  if (state_ < 2) return fail(MBIR_ESTATE, "set_planes: call prepare first");
  if (fp64_) return fail(MBIR_ENOTSUP, "set_planes: FP32 engines only");
  if (!in || y < 0 || n < 0 || y + n > g_.n_y) return fail(MBIR_EINVAL, "set_planes: bad range");
  const size_t plane = static_cast<size_t>(g_.n_z) * g_.n_x;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  cudaMemcpyAsync(static_cast<float*>(d_x_) + static_cast<size_t>(y) * plane, in,
                  sizeof(float) * plane * n, cudaMemcpyHostToDevice, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK : cuda_check(MBIR_EDEVICE, "set_planes");
}

// kind 0: the six jointEstimation sums per view ([theta][6]); kind 1: sum e^2 per view; over
// the detector rows of the slab's slices
int Engine::view_sums(int kind, double* out) {
  if (state_ < 2) return fail(MBIR_ESTATE, "view_sums: call prepare first");
  if (bf_) return fail(MBIR_ENOTSUP, "view_sums: HAADF only");
  if (kind != 0 && kind != 1) return fail(MBIR_EINVAL, "view_sums: kind is 0 or 1");
  const Geometry& g = g_;
  const int y0 = slab_y1_ > 0 ? slab_y0_ : 0, y1 = slab_y1_ > 0 ? slab_y1_ : g.n_y;
  int t0 = g.n_t, t1 = 0;
  for (int y = y0; y < y1; y++)
    if (tab_.t_count[y] > 0) {
      t0 = std::min(t0, tab_.t_first[y]);
      t1 = std::max(t1, tab_.t_first[y] + tab_.t_count[y]);
    }
  const int nt = g.n_theta, K = kind == 0 ? 6 : 1;
  if (t0 >= t1) {
    for (int i = 0; i < nt * K; i++) out[i] = 0.0;
    return MBIR_OK;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  int rc = launch_view_sums_rows(kind, d_y_, d_e_, d_mu_, d_gain_, d_wv_, d_partial_, d_vsum_, nt,
                                 n_rp_, g.n_r, t0, t1, n_chunk_, fp64_, s);
  if (rc) return cuda_check(rc, "view sums");
  cudaMemcpyAsync(out, d_vsum_, sizeof(double) * nt * K, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK : cuda_check(MBIR_EDEVICE, "view sums");
}

// New gain/offset (with the jointEstimation error rebuild, _Extra.cpp:600-612) and/or variance
// (w = 1 / alpha); null arrays leave those parameters unchanged
int Engine::apply_nuisance(const double* gain, const double* offset, const double* variance) {
  if (state_ < 2) return fail(MBIR_ESTATE, "apply_nuisance: call prepare first");
  if (bf_) return fail(MBIR_ENOTSUP, "apply_nuisance: HAADF only");
  const Geometry& g = g_;
  const int nt = g.n_theta;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  if (gain && offset) {
    cudaMemcpyAsync(d_mu2_, offset, sizeof(double) * nt, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_gain2_, gain, sizeof(double) * nt, cudaMemcpyHostToDevice, s);
    int rc = launch_rebuild_error(d_y_, d_e_, d_mu_, d_gain_, d_mu2_, d_gain2_, nt, n_rp_, g.n_r,
                                  g.n_t, fp64_, s);
    if (rc) return cuda_check(rc, "rebuild error sinogram");
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "apply nuisance");
    I_.assign(gain, gain + nt);
    mu_.assign(offset, offset + nt);
  }
  if (variance) {
    for (int v = 0; v < nt; v++) {
      alpha_[v] = variance[v];
      w_[v] = 1.0 / alpha_[v];
    }
  }
  return upload_views();
}

// Detector rows [t0, t1) of the slab's slices (of every slice without a slab); t0 >= t1: none.
void Engine::slab_rows(int* t0, int* t1) const {
  const Geometry& g = g_;
  const int y0 = slab_y1_ > 0 ? slab_y0_ : 0, y1 = slab_y1_ > 0 ? slab_y1_ : g.n_y;
  *t0 = g.n_t;
  *t1 = 0;
  for (int y = y0; y < y1; y++)
    if (tab_.t_count[y] > 0) {
      *t0 = std::min(*t0, tab_.t_first[y]);
      *t1 = std::max(*t1, tab_.t_first[y] + tab_.t_count[y]);
    }
}

// The bright-field sinogram arrays from detector row t0 on, t1 - t0 rows ([t][theta][r] layout:
// a row range is one contiguous block of each array).
BfSino Engine::bf_sino_rows(int t0, int t1) const {
  BfSino b = bf_sino();
  const size_t plane = static_cast<size_t>(g_.n_theta) * n_rp_;
  b.e = static_cast<char*>(b.e) + static_cast<size_t>(t0) * plane * rb_;
  b.w = static_cast<char*>(b.w) + static_cast<size_t>(t0) * plane * rb_;
  b.sel += static_cast<size_t>(t0) * g_.n_theta * n_sp_;
  b.n_t = t1 - t0;
  return b;
}

// Opens an NHICD call on the slab (BFReconstructionEngine.cpp:610-646): the call's lines (the
// next homogeneous sub-list, or the non-homogeneous list from the magnitude map, which every
// slab holds summed over all slabs), its schedule and row order.  The slab's colours follow
// with sweep_colour; bf_slab_end closes the call.
int Engine::bf_slab_begin(int outer, int inner) {
  if (state_ < 2) return fail(MBIR_ESTATE, "bf_call_begin: call prepare first");
  if (!bf_) return fail(MBIR_EINVAL, "bf_call_begin: not a bright-field engine");
  if (p_.order_mode != MBIR_ORDER_PARALLEL || exact_)
    return fail(MBIR_ENOTSUP, "bf_call_begin: parallel order only");
  if (slab_call_open_) return fail(MBIR_ESTATE, "bf_call_begin: a call is open");
  if (int rc = slab_rows_owned()) return rc;
  DevBF bfa{};
  int rc = bf_call_begin(outer, inner, &bfa);
  if (rc) return rc;
  const int iter_nonzero = (inner > 0 || outer > 0) ? 1 : 0;
  if ((rc = bf_parallel_args(iter_nonzero, bfa, &slab_args_, &slab_smem_))) return rc;
  slab_call_open_ = true;
  outer_ = outer;
  inner_ = inner;
  return MBIR_OK;
}

// The open call's update magnitude per line (sum |dx| over this slab's slices, fixed point
// 2^-32), after both colours.
int Engine::bf_slab_magnitudes(unsigned long long* out) {
  if (!slab_call_open_) return fail(MBIR_ESTATE, "bf_call_magnitudes: no open call");
  if (!out) return fail(MBIR_EINVAL, "bf_call_magnitudes: null output");
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nl = static_cast<size_t>(g_.n_z) * g_.n_x;
  cudaMemcpyAsync(out, d_magfx_, sizeof(unsigned long long) * nl, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK
                                                 : cuda_check(MBIR_EDEVICE, "call magnitudes");
}

// Closes the call: the magnitude map takes the call's magnitudes (mag: summed over all slabs,
// so every slab holds the same map; null: this slab's own), and the call is counted.
int Engine::bf_slab_end(const unsigned long long* mag) {
  if (!slab_call_open_) return fail(MBIR_ESTATE, "bf_call_end: no open call");
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const size_t nl = static_cast<size_t>(g_.n_z) * g_.n_x;
  if (mag)
    cudaMemcpyAsync(d_magfx_, mag, sizeof(unsigned long long) * nl, cudaMemcpyHostToDevice, s);
  slab_call_open_ = false;
  int rc = bf_call_end();
  if (rc) return rc;
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "call end");
  bf_schedule_settle();
  if ((rc = check_device_error())) return rc;
  sweeps_done_++;
  return MBIR_OK;
}

// Partial sums over the slab's detector rows, for the host to sum over slabs.  kind 2: the
// offset step's numerator and denominator per view (jointEstimation, BFForwardModel.cpp:
// 390-441), [theta][2]; kind 3: the variance sums over selected and rejected entries
// (updateWeights, :447-511) and the number of entries they cover, [3], after scaling the slab's
// weights by the current variance as updateWeights does (once per update, then
// bf_slab_apply(3)).
int Engine::bf_slab_sums(int kind, double* out) {
  if (state_ < 2) return fail(MBIR_ESTATE, "bf_slab_sums: call prepare first");
  if (!bf_ || exact_) return fail(MBIR_ENOTSUP, "bf_slab_sums: bright field, parallel order");
  if (kind != 2 && kind != 3) return fail(MBIR_EINVAL, "bf_slab_sums: kind is 2 or 3");
  if (!out) return fail(MBIR_EINVAL, "bf_slab_sums: null output");
  const int nt = g_.n_theta, K = kind == 2 ? 2 * nt : 3;
  int t0, t1;
  slab_rows(&t0, &t1);
  if (t0 >= t1) {
    for (int i = 0; i < K; i++) out[i] = 0.0;
    return MBIR_OK;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const BfSino b = bf_sino_rows(t0, t1);
  int rc;
  if (kind == 2) {
    rc = launch_bf_offset_sums(b, 0, bragg_t_, p_.bragg_delta, d_partial_, n_chunk_, d_vsum_, s);
    if (rc) return cuda_check(rc, "offset sums");
    cudaMemcpyAsync(out, d_vsum_, sizeof(double) * K, cudaMemcpyDeviceToHost, s);
  } else {
    cudaMemcpyAsync(d_alpha_, alpha_.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
    rc = launch_bf_variance_sums(b, 0, d_alpha_, d_bfpart_, d_bfout_, s);
    if (rc) return cuda_check(rc, "variance sums");
    cudaMemcpyAsync(out, d_bfout_, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
    out[2] = static_cast<double>(nt) * g_.n_r * (t1 - t0);
  }
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK : cuda_check(MBIR_EDEVICE, "slab sums");
}

// Applies the sums of bf_slab_sums added over all slabs to the slab's rows: kind 2, the offset
// step num / den per view (e -= step, mu += step); kind 3, the common variance (the two sums
// over the entries they cover; weights divided by it); then the Bragg selector
// (updateSelector, BFForwardModel.cpp:517-531).
int Engine::bf_slab_apply(int kind, const double* sums) {
  if (state_ < 2) return fail(MBIR_ESTATE, "bf_slab_apply: call prepare first");
  if (!bf_ || exact_) return fail(MBIR_ENOTSUP, "bf_slab_apply: bright field, parallel order");
  if (kind != 2 && kind != 3) return fail(MBIR_EINVAL, "bf_slab_apply: kind is 2 or 3");
  if (!sums) return fail(MBIR_EINVAL, "bf_slab_apply: null sums");
  const Geometry& g = g_;
  const int nt = g.n_theta;
  int t0, t1;
  slab_rows(&t0, &t1);
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const BfSino b = bf_sino_rows(t0, std::max(t0, t1));
  int rc;
  if (kind == 2) {
    std::vector<double> step(nt);
    for (int v = 0; v < nt; v++) {
      step[v] = sums[v * 2 + 0] / sums[v * 2 + 1];
      mu_[v] += step[v];
    }
    if (b.n_t > 0) {
      cudaMemcpyAsync(d_mu2_, step.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
      if ((rc = launch_bf_offset_apply(b, d_mu2_, s))) return cuda_check(rc, "offset apply");
    }
  } else {
    const double upd = (sums[0] + (p_.bragg_delta * bragg_t_) * sums[1]) / sums[2];
    for (int v = 0; v < nt; v++) alpha_[v] = upd;
    if (b.n_t > 0 && (rc = launch_bf_scale_weights(b, upd, s))) return cuda_check(rc, "weights");
    cudaMemcpyAsync(d_alpha_, alpha_.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  }
  if (b.n_t > 0 && (rc = launch_bf_selector(b, bragg_t_, s))) return cuda_check(rc, "selector");
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_check(MBIR_EDEVICE, "slab apply");
  return kind == 2 ? upload_views() : MBIR_OK;
}

// The stop rule's two ROI sums (stopCriteria / roiVolumeSum, BFReconstructionEngine_Extra.cpp:
// 1200-1248): [0] over the magnitude map (the same on every slab), [1] over the volume of the
// slab's slices (summed over slabs by the host).
int Engine::roi_sums(double* out2) {
  if (state_ < 2) return fail(MBIR_ESTATE, "roi_sums: call prepare first");
  if (!bf_) return fail(MBIR_EINVAL, "roi_sums: bright field only");
  if (!out2) return fail(MBIR_EINVAL, "roi_sums: null output");
  int rc = bf_roi_sum(0, &out2[0]);
  if (rc) return rc;
  const int y0 = slab_y1_ > 0 ? slab_y0_ : 0, y1 = slab_y1_ > 0 ? slab_y1_ : g_.n_y;
  DevGeom gs = dg_;
  gs.n_y = y1 - y0;
  const size_t plane = static_cast<size_t>(g_.n_z) * g_.n_x;
  const void* xs = static_cast<const char*>(d_x_) + static_cast<size_t>(y0) * plane * rb_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  rc = launch_roi_sum(gs, exact_ ? 1 : 0, 1, d_mag_, xs, fp64_, d_bfpart_, d_bfout_, s);
  if (rc) return cuda_check(rc, "ROI sum");
  cudaMemcpyAsync(&out2[1], d_bfout_, sizeof(double), cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? MBIR_OK : cuda_check(MBIR_EDEVICE, "ROI sums");
}

}  // namespace mbir
