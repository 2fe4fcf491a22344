// mbir_shard.cu -- y-slab sharding of one reconstruction over several engines (one per GPU).
//
// Voxel slice y touches only its own detector rows, so a contiguous slab of slices [y0, y1)
// owns a contiguous block of the error sinogram: ICD needs no sinogram exchange between slabs.
// The prior couples neighbouring slices, so after each colour phase a slab's boundary planes
// go to its neighbours (host-mediated: get_planes / set_planes), and the per-view sums of the
// gain/offset and variance estimates are summed over slabs before the host solves them.  Each
// engine holds the whole problem; only its slab is updated and summed.
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
// sweep k use the row order of sweep k; the sweep is counted after colour 1.
int Engine::sweep_colour(int colour, int outer, int inner, double* st4) {
  if (state_ < 2) return fail(MBIR_ESTATE, "sweep_colour: call prepare first");
  if (bf_ || p_.order_mode != MBIR_ORDER_PARALLEL)
    return fail(MBIR_ENOTSUP, "sweep_colour: HAADF parallel order only");
  if (colour != 0 && colour != 1) return fail(MBIR_EINVAL, "sweep_colour: colour is 0 or 1");
  if (int rc = slab_rows_owned()) return rc;
  const Geometry& g = g_;
  cudaStream_t s = static_cast<cudaStream_t>(stream_);
  const int y0 = slab_y1_ > 0 ? slab_y0_ : 0, y1 = slab_y1_ > 0 ? slab_y1_ : g.n_y;
  const int first = y0 + ((y0 & 1) != colour ? 1 : 0);
  const int n = first < y1 ? (y1 - first + 1) / 2 : 0;
  if (colour == 0) {
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
  a.colour = colour;
  a.y_first = first;
  a.y_end = y1;
  a.n_slices = n;
  a.stats = d_stats_;
  double st[kStatSlots] = {0, 0, 0, 0};
  int rc;
  cudaEventRecord(static_cast<cudaEvent_t>(ev0_), s);
  if (n > 0) {
    if ((rc = launch_sweep(a, nb_, smem_bytes_, s))) return cuda_check(rc, "slab sweep launch");
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
  if (colour == 1) {
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

}  // namespace mbir
