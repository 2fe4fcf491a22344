// mbir_capi.cpp -- extern "C" boundary over mbir::Engine.  No C++ exception crosses it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mbir_batch.h"
#include "mbir_server.h"
#include "mbir_engine.h"

struct mbir_engine {
  mbir::Engine* impl;
};
struct mbir_batch {
  mbir::Batch* impl;
};
struct mbir_server {
  mbir::Server* impl;
};

namespace {
thread_local std::string g_create_error;

template <typename F>
int32_t guarded(mbir_engine* e, F&& f) {
  if (!e || !e->impl) return MBIR_EINVAL;
  try {
    return f(*e->impl);
  } catch (const std::bad_alloc&) {
    return e->impl->fail(MBIR_ENOMEM, "host allocation failed");
  } catch (const std::exception& ex) {
    return e->impl->fail(MBIR_EINVAL, ex.what());
  } catch (...) {
    return e->impl->fail(MBIR_EINVAL, "unknown error");
  }
}
}  // namespace

extern "C" {

const char* mbir_version(void) { return "mbir-gb300 0.1 (sm_103a)"; }

// InitializeAdvancedParams (HAADF_ReconstructionEngine.cpp:244-259), the TCLAP defaults of
// HAADFReconstructionArgsParser.cpp:143-211 and the QGGMRF constants of
// HAADF_QGGMRFPriorModel.cpp:10-21 / BF_QGGMRFPriorModel.cpp:49-67.
void mbir_params_default(mbir_params* p, int32_t modality) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->struct_size = static_cast<int32_t>(sizeof(mbir_params));
  p->modality = modality;
  p->sample_thickness = 0.0;
  p->diffuseness = 0.2;
  p->sigma_x = 1.0;
  p->stop_threshold = 0.005;
  p->num_resolutions = 3;
  p->final_resolution = 1;
  p->level = -1;
  p->target_gain = 1.0;
  p->outer_iterations = 30;
  p->inner_iterations = 10;
  p->default_offset = 0.0;
  p->default_variance = 1.0;
  p->default_recon_value = 0.0;
  p->default_pixel_size = 1.0;
  p->x_shrink_factor = 0.6;
  p->z_stretch = 2;
  p->detector_response_bins = 64;
  p->profile_resolution = 1536;
  p->beam_resolution = 512;
  p->joint_estimation = 1;
  p->zero_skipping = 1;
  p->noise_model = 1;
  p->noise_estimation = 0;
  p->estimate_prior = 0;
  p->threshold_reduction_factor = 1.0;
  p->qggmrf_p = 2.0;
  p->qggmrf_q = 0.0;
  p->qggmrf_c = modality == MBIR_MODALITY_BF ? 0.01 : 0.001;
  p->qggmrf_alpha = 1.5;
  p->bragg_threshold = 5e10;
  p->bragg_delta = 0.5;
  p->bf_offset = 0.0;
  p->default_dosage = 0.0;
  p->order_mode = MBIR_ORDER_PARALLEL;
  p->seed = 1u;
  p->compat_double_angle = modality == MBIR_MODALITY_BF ? 0 : 1;
  p->cost_every_sweep = 0;
  p->device = 0;
  p->slice_staging = 0;
  p->nhicd = 0;
  if (modality == MBIR_MODALITY_BF) {
    // BFReconstructionArgsParser.cpp:143-226 and BFReconstructionEngine.cpp:246-260
    p->stop_threshold = 0.001;
    p->outer_iterations = 600;
    p->inner_iterations = 100;
    p->bragg_threshold = 3.0;
    p->bragg_delta = 0.5;
    p->noise_estimation = 1;
    p->noise_model = 0;
    p->nhicd = 1;  // NHICD is defined in BFConstants.h
  }
}

namespace {
// The reference's multi-resolution pipeline keeps these parameters in float members
// (HAADF_MultiResolutionReconstruction.h:76-89, BFMultiResolutionReconstruction.h:76-107) and
// evaluates p = diffuseness + 1 in float (HAADF_MultiResolutionReconstruction.cpp:333); the BF
// command line stores -log(dosage + bf_offset) in such a member (BFReconstructionArgsParser.cpp:
// 272-274).  float_params = 1 applies the same roundings, so that results equal the reference
// run from its command line (the rounding is idempotent; the BF offset is rounded where the
// engine computes it, Engine::bf_default_offset).
mbir_params with_float_params(const mbir_params& in) {
  mbir_params p = in;
  if (!p.float_params) return p;
  auto f = [](double v) { return static_cast<double>(static_cast<float>(v)); };
  if (p.qggmrf_q == 0.0)
    p.qggmrf_q = static_cast<double>(static_cast<float>(p.diffuseness) + 1.0f);
  p.diffuseness = f(p.diffuseness);
  p.sample_thickness = f(p.sample_thickness);
  p.target_gain = f(p.target_gain);
  p.stop_threshold = f(p.stop_threshold);
  p.sigma_x = f(p.sigma_x);
  p.default_offset = f(p.default_offset);
  p.default_variance = f(p.default_variance);
  p.default_recon_value = f(p.default_recon_value);
  p.bragg_threshold = f(p.bragg_threshold);
  p.bragg_delta = f(p.bragg_delta);
  p.bf_offset = f(p.bf_offset);
  return p;
}
}  // namespace

mbir_engine* mbir_create(const mbir_params* p) {
  if (!p || p->struct_size != static_cast<int32_t>(sizeof(mbir_params))) {
    g_create_error = "mbir_create: params missing or struct_size mismatch";
    return nullptr;
  }
  if (p->modality != MBIR_MODALITY_HAADF && p->modality != MBIR_MODALITY_BF) {
    g_create_error = "mbir_create: unknown modality";
    return nullptr;
  }
  if (p->modality == MBIR_MODALITY_BF &&
      (!(p->bragg_threshold > 0) || !(p->bragg_delta >= 0) ||
       (p->use_default_offset && !(p->default_dosage + p->bf_offset > 0)))) {
    g_create_error = "mbir_create: invalid bright-field parameter";
    return nullptr;
  }
  if (p->estimate_prior) {
    // ESTIMATE_PRIOR (HAADF_ReconstructionEngine.cpp:807-812): the sigma_x re-estimate between
    // outer iterations is not built; refuse rather than run a different algorithm
    g_create_error = "mbir_create: estimate_prior is not supported by this build";
    return nullptr;
  }
  if (!(p->sigma_x > 0) || p->num_resolutions < 1 || p->final_resolution < 1 ||
      !(p->qggmrf_c > 0) || !(p->qggmrf_p > 0) ||
      (p->seed_mode != MBIR_SEED_PER_CALL && p->seed_mode != MBIR_SEED_FIXED)) {
    g_create_error = "mbir_create: invalid parameter value";
    return nullptr;
  }
  try {
    auto* e = new mbir_engine;
    e->impl = new mbir::Engine(with_float_params(*p));
    return e;
  } catch (...) {
    g_create_error = "mbir_create: allocation failed";
    return nullptr;
  }
}

void mbir_destroy(mbir_engine* e) {
  if (!e) return;
  delete e->impl;
  delete e;
}

const char* mbir_last_error(const mbir_engine* e) {
  if (!e || !e->impl) return g_create_error.c_str();
  return e->impl->last_error();
}

int32_t mbir_set_sinogram(mbir_engine* e, const float* counts, const float* tilts_deg,
                          int32_t n_theta, int32_t n_r, int32_t n_t, double delta_r,
                          double delta_t) {
  return guarded(e, [&](mbir::Engine& m) {
    return m.set_sinogram(counts, tilts_deg, n_theta, n_r, n_t, delta_r, delta_t);
  });
}
int32_t mbir_load_sinogram_mrc(mbir_engine* e, const char* path) {
  return guarded(e, [&](mbir::Engine& m) { return m.load_mrc(path); });
}
int32_t mbir_set_bright_field(mbir_engine* e, const float* counts, int32_t n_theta, int32_t n_r,
                              int32_t n_t) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_bright_field(counts, n_theta, n_r, n_t); });
}
int32_t mbir_set_intermediate_dir(mbir_engine* e, const char* dir) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_intermediate_dir(dir); });
}
int32_t mbir_set_observer(mbir_engine* e, mbir_observer_fn fn, void* user) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_observer(fn, user); });
}
int32_t mbir_write_checkpoint(mbir_engine* e, const char* dir) {
  return guarded(e, [&](mbir::Engine& m) { return m.write_checkpoint(dir); });
}
int32_t mbir_read_checkpoint(mbir_engine* e, const char* dir) {
  return guarded(e, [&](mbir::Engine& m) { return m.read_checkpoint(dir); });
}
int32_t mbir_load_bright_field_mrc(mbir_engine* e, const char* path) {
  return guarded(e, [&](mbir::Engine& m) { return m.load_bright_field_mrc(path); });
}
int32_t mbir_set_initial_volume(mbir_engine* e, const float* vol, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_initial_volume(vol, n); });
}
int32_t mbir_set_initial_volume_f64(mbir_engine* e, const double* vol, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_initial_volume_f64(vol, n); });
}
int32_t mbir_get_volume_f64(mbir_engine* e, double* out, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_volume_f64(out, n); });
}
int32_t mbir_set_initial_nuisance(mbir_engine* e, const double* g, const double* o,
                                  const double* v) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_initial_nuisance(g, o, v); });
}
int32_t mbir_get_dims(mbir_engine* e, int32_t* dims) {
  if (!dims) return MBIR_EINVAL;
  return guarded(e, [&](mbir::Engine& m) { return m.dims(dims); });
}
int32_t mbir_run(mbir_engine* e) {
  return guarded(e, [&](mbir::Engine& m) { return m.run(); });
}
int32_t mbir_prepare(mbir_engine* e) {
  return guarded(e, [&](mbir::Engine& m) { return m.prepare(); });
}
int32_t mbir_sweep(mbir_engine* e, int32_t outer, int32_t inner, double* stats4) {
  return guarded(e, [&](mbir::Engine& m) { return m.sweep(outer, inner, stats4); });
}
int32_t mbir_joint_estimation(mbir_engine* e) {
  return guarded(e, [&](mbir::Engine& m) { return m.joint_estimation(); });
}
int32_t mbir_update_weights(mbir_engine* e) {
  return guarded(e, [&](mbir::Engine& m) { return m.update_weights(); });
}
int32_t mbir_compute_cost(mbir_engine* e, double* parts3, double* total) {
  return guarded(e, [&](mbir::Engine& m) { return m.compute_cost(parts3, total); });
}
int32_t mbir_forward_project(mbir_engine* e) {
  return guarded(e, [&](mbir::Engine& m) { return m.forward_project(); });
}
int32_t mbir_get_volume(mbir_engine* e, float* out, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_volume(out, n); });
}
int32_t mbir_get_error_sinogram(mbir_engine* e, float* out, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_error(out, n); });
}
int32_t mbir_get_projection(mbir_engine* e, float* out, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_projection(out, n); });
}
int32_t mbir_get_nuisance(mbir_engine* e, double* g, double* o, double* v) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_nuisance(g, o, v); });
}
int32_t mbir_get_tables(mbir_engine* e, double* H, double* Ht) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_tables(H, Ht); });
}
int32_t mbir_get_schedule(mbir_engine* e, int32_t sweep, int32_t* rows, int32_t* stride) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_schedule(sweep, rows, stride); });
}
int32_t mbir_get_call_lines(mbir_engine* e, int32_t* lines, int32_t cap, int32_t* n) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_call_lines(lines, cap, n); });
}
int32_t mbir_get_call_schedule(mbir_engine* e, int32_t* lines, int32_t cap, int32_t* lofs,
                               int32_t lofs_cap, int32_t* n_lines, int32_t* n_levels) {
  return guarded(e, [&](mbir::Engine& m) {
    return m.get_call_schedule(lines, cap, lofs, lofs_cap, n_lines, n_levels);
  });
}
int32_t mbir_get_footprint_bins(mbir_engine* e, int16_t* lo, uint16_t* mask, uint8_t* lineok) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_footprint_bins(lo, mask, lineok); });
}
int32_t mbir_get_bf_state(mbir_engine* e, uint8_t* selector, float* weights, double* mag,
                          double* filtered_mag, double* bragg_t) {
  return guarded(e, [&](mbir::Engine& m) {
    return m.get_bf_state(selector, weights, mag, filtered_mag, bragg_t);
  });
}
int32_t mbir_set_bragg_threshold(mbir_engine* e, double t) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_bragg_threshold(t); });
}
int32_t mbir_set_slab(mbir_engine* e, int32_t y0, int32_t y1) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_slab(y0, y1); });
}
int32_t mbir_sweep_colour(mbir_engine* e, int32_t colour, int32_t outer, int32_t inner,
                          double* stats4) {
  return guarded(e, [&](mbir::Engine& m) { return m.sweep_colour(colour, outer, inner, stats4); });
}
int32_t mbir_get_planes(mbir_engine* e, int32_t y, int32_t n, float* out) {
  return guarded(e, [&](mbir::Engine& m) { return m.get_planes(y, n, out); });
}
int32_t mbir_set_planes(mbir_engine* e, int32_t y, int32_t n, const float* in) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_planes(y, n, in); });
}
int32_t mbir_view_sums(mbir_engine* e, int32_t kind, double* out) {
  return guarded(e, [&](mbir::Engine& m) { return m.view_sums(kind, out); });
}
int32_t mbir_apply_nuisance(mbir_engine* e, const double* gain, const double* offset,
                            const double* variance) {
  return guarded(e, [&](mbir::Engine& m) { return m.apply_nuisance(gain, offset, variance); });
}
int32_t mbir_bf_call_begin(mbir_engine* e, int32_t outer, int32_t inner) {
  return guarded(e, [&](mbir::Engine& m) { return m.bf_slab_begin(outer, inner); });
}
int32_t mbir_bf_call_magnitudes(mbir_engine* e, uint64_t* out) {
  static_assert(sizeof(uint64_t) == sizeof(unsigned long long), "64-bit magnitudes");
  return guarded(e, [&](mbir::Engine& m) {
    return m.bf_slab_magnitudes(reinterpret_cast<unsigned long long*>(out));
  });
}
int32_t mbir_bf_call_end(mbir_engine* e, const uint64_t* magnitudes) {
  return guarded(e, [&](mbir::Engine& m) {
    return m.bf_slab_end(reinterpret_cast<const unsigned long long*>(magnitudes));
  });
}
int32_t mbir_bf_slab_sums(mbir_engine* e, int32_t kind, double* out) {
  return guarded(e, [&](mbir::Engine& m) { return m.bf_slab_sums(kind, out); });
}
int32_t mbir_bf_slab_apply(mbir_engine* e, int32_t kind, const double* sums) {
  return guarded(e, [&](mbir::Engine& m) { return m.bf_slab_apply(kind, sums); });
}
int32_t mbir_roi_sums(mbir_engine* e, double* out2) {
  return guarded(e, [&](mbir::Engine& m) { return m.roi_sums(out2); });
}
int32_t mbir_status_get(mbir_engine* e, mbir_status* st) {
  return guarded(e, [&](mbir::Engine& m) { return m.status(st); });
}
void mbir_cancel(mbir_engine* e) {
  if (e && e->impl) e->impl->cancel();
}
int32_t mbir_write_outputs(mbir_engine* e, const char* dir, const char* mrc_path) {
  return guarded(e, [&](mbir::Engine& m) { return m.write_outputs(dir, mrc_path); });
}
int32_t mbir_estimate_sigma_x(const char* mrc_path, double sample_thickness, double target_gain,
                              int32_t use_bf_offset, double bf_offset, const float* tilts_deg,
                              int32_t n_tilts, const int32_t* x_range, const int32_t* y_range,
                              double* sigma_x) {
  if (!mrc_path || !sigma_x || (n_tilts > 0 && !tilts_deg) || n_tilts < 0) return MBIR_EINVAL;
  try {
    std::vector<float> tilts(tilts_deg, tilts_deg + n_tilts);
    if (n_tilts == 0) {  // the a-tilts of the FEI extended header
      mbir::MrcVolume hdr;
      std::string err;
      if (mbir::mrc_read(mrc_path, nullptr, nullptr, hdr, true, err)) return MBIR_EIO;
      tilts = hdr.a_tilt;
    }
    std::string err;
    return mbir::estimate_sigma_x(mrc_path, sample_thickness, target_gain, use_bf_offset != 0,
                                  bf_offset, tilts.data(), static_cast<int>(tilts.size()),
                                  x_range, y_range, sigma_x, err);
  } catch (...) {
    return MBIR_ENOMEM;
  }
}

int32_t mbir_write_outputs_ex(mbir_engine* e, const char* dir, const char* mrc_path,
                              const char* vtk_path, const char* avizo_path) {
  return guarded(
      e, [&](mbir::Engine& m) { return m.write_outputs(dir, mrc_path, vtk_path, avizo_path); });
}

// HAADF_MultiResolutionReconstruction::execute (HAADF_MultiResolutionReconstruction.cpp:175-485):
// per level i: sigma_x * 2^((levels-1-i)(1-3/p)), NumIter = 1 after the first level,
// stop threshold x2 from level 2, the previous level's volume replicated 2x in every
// direction (InitialReconstructionBinReader.cpp:104-135) and its nuisance vectors handed on.
int32_t mbir_run_multires(const mbir_params* p, const float* counts, const float* tilts_deg,
                          int32_t n_theta, int32_t n_r, int32_t n_t, double delta_r,
                          double delta_t, float* out, int64_t n, int32_t* dims_out) {
  if (!p || !counts || !tilts_deg) return MBIR_EINVAL;
  if (p->estimate_prior) return MBIR_ENOTSUP;
  const mbir_params top = with_float_params(*p);
  p = &top;
  const int levels = p->num_resolutions > 0 ? p->num_resolutions : 1;
  std::vector<double> prev;
  int pdims[3] = {0, 0, 0};
  std::vector<double> g(n_theta), o(n_theta), v(n_theta);
  bool have_nuis = false;
  try {
    for (int i = 0; i < levels; ++i) {
      mbir_params q = *p;
      q.level = i;
      const double pq = (p->qggmrf_q != 0.0) ? p->qggmrf_q : p->diffuseness + 1.0;
      q.qggmrf_q = pq;
      q.sigma_x = std::pow(2.0, (levels - 1 - i) * (1 - 3 / pq)) * p->sigma_x;
      if (i > 0) q.inner_iterations = 1;
      if (i >= 2) q.stop_threshold = p->stop_threshold * 2.0f;
      mbir::Engine eng(q);
      int rc = eng.set_sinogram(counts, tilts_deg, n_theta, n_r, n_t, delta_r, delta_t);
      if (rc) return rc;
      int32_t d[6];
      if ((rc = eng.dims(d))) return rc;
      if (have_nuis && (rc = eng.set_initial_nuisance(g.data(), o.data(), v.data()))) return rc;
      if (i > 0) {
        // 2x voxel replication of the previous level (InterpFlag = 1), in FP64 as the
        // reference reads ReconstructedObject.bin
        std::vector<double> up(static_cast<size_t>(d[0]) * d[1] * d[2], 0.0);
        const int ze = d[0] / 2, xe = d[1] / 2, ye = d[2] / 2;
        for (int y = 0; y < ye && y < pdims[2]; y++)
          for (int x = 0; x < xe && x < pdims[1]; x++)
            for (int z = 0; z < ze && z < pdims[0]; z++) {
              const double b = prev[(static_cast<size_t>(z) * pdims[1] + x) * pdims[2] + y];
              for (int a = 0; a < 2; a++)
                for (int c = 0; c < 2; c++)
                  for (int r = 0; r < 2; r++)
                    up[(static_cast<size_t>(2 * z + a) * d[1] + 2 * x + c) * d[2] + 2 * y + r] = b;
            }
        if ((rc = eng.set_initial_volume_f64(up.data(), static_cast<int64_t>(up.size()))))
          return rc;
      }
      if ((rc = eng.run())) return rc;
      prev.assign(static_cast<size_t>(d[0]) * d[1] * d[2], 0.0);
      if ((rc = eng.get_volume_f64(prev.data(), static_cast<int64_t>(prev.size())))) return rc;
      pdims[0] = d[0];
      pdims[1] = d[1];
      pdims[2] = d[2];
      eng.get_nuisance(g.data(), o.data(), v.data());
      have_nuis = true;
    }
  } catch (...) {
    return MBIR_ENOMEM;
  }
  const size_t nv = static_cast<size_t>(pdims[0]) * pdims[1] * pdims[2];
  if (dims_out) {
    dims_out[0] = pdims[0];
    dims_out[1] = pdims[1];
    dims_out[2] = pdims[2];
  }
  if (out) {
    if (n < static_cast<int64_t>(nv)) return MBIR_EINVAL;
    for (size_t i = 0; i < nv; i++) out[i] = static_cast<float>(prev[i]);
  }
  return MBIR_OK;
}

mbir_batch* mbir_batch_create(int32_t device) {
  try {
    auto* b = new mbir_batch;
    b->impl = new mbir::Batch(device);
    return b;
  } catch (...) {
    return nullptr;
  }
}
void mbir_batch_destroy(mbir_batch* b) {
  if (!b) return;
  delete b->impl;
  delete b;
}
int32_t mbir_batch_add(mbir_batch* b, mbir_engine* e) {
  if (!b || !e || !e->impl) return MBIR_EINVAL;
  try {
    return b->impl->add(e->impl);
  } catch (...) {
    return MBIR_ENOMEM;
  }
}
int32_t mbir_batch_remove(mbir_batch* b, mbir_engine* e) {
  if (!b || !e || !e->impl) return MBIR_EINVAL;
  return b->impl->remove(e->impl);
}
int32_t mbir_batch_size(const mbir_batch* b) {
  return b ? static_cast<int32_t>(b->impl->size()) : 0;
}
int32_t mbir_batch_set_threads(mbir_batch* b, int32_t threads) {
  return b ? b->impl->set_threads(threads) : MBIR_EINVAL;
}
int32_t mbir_batch_get_threads(mbir_batch* b) { return b ? b->impl->threads() : MBIR_EINVAL; }
int32_t mbir_batch_set_wait_limit(mbir_batch* b, double seconds) {
  return b ? b->impl->set_wait_limit(seconds) : MBIR_EINVAL;
}
int32_t mbir_batch_sweep(mbir_batch* b, int32_t outer, double* stats) {
  if (!b) return MBIR_EINVAL;
  try {
    std::vector<std::pair<int, int>> it(b->impl->size(), std::make_pair(outer, 0));
    return b->impl->sweep(it, stats);
  } catch (...) {
    return b->impl->fail(MBIR_ENOMEM, "host allocation failed");
  }
}
int32_t mbir_batch_run(mbir_batch* b, int32_t max_outer, double tol, int32_t* outer_done,
                       double* final_cost) {
  if (!b || max_outer < 0) return MBIR_EINVAL;
  try {
    std::vector<int> od(b->impl->size());
    int rc = b->impl->run(max_outer, tol, od.data(), final_cost);
    if (outer_done)
      for (size_t i = 0; i < od.size(); i++) outer_done[i] = od[i];
    return rc;
  } catch (...) {
    return b->impl->fail(MBIR_ENOMEM, "host allocation failed");
  }
}
double mbir_batch_last_ms(const mbir_batch* b) { return b ? b->impl->last_ms() : 0.0; }
double mbir_batch_total_ms(const mbir_batch* b) { return b ? b->impl->total_ms() : 0.0; }
const char* mbir_batch_last_error(const mbir_batch* b) {
  return b ? b->impl->last_error() : "null batch";
}

mbir_server* mbir_server_create(int32_t device, int64_t budget, int32_t max_active) {
  try {
    auto* s = new mbir_server;
    s->impl = new mbir::Server(device, budget, max_active);
    return s;
  } catch (...) {
    return nullptr;
  }
}
void mbir_server_destroy(mbir_server* s) {
  if (!s) return;
  delete s->impl;
  delete s;
}
int64_t mbir_server_submit(mbir_server* s, const mbir_params* p, const float* counts,
                           const float* tilts, int32_t n_theta, int32_t n_r, int32_t n_t,
                           double dr, double dt, int32_t max_outer, double tol) {
  if (!s || !p || !counts || !tilts) return MBIR_EINVAL;
  if (p->struct_size != static_cast<int32_t>(sizeof(mbir_params))) return MBIR_EINVAL;
  if (p->estimate_prior) return MBIR_ENOTSUP;
  if (p->modality != MBIR_MODALITY_HAADF && p->modality != MBIR_MODALITY_BF) return MBIR_EINVAL;
  try {
    return s->impl->submit(*p, counts, tilts, n_theta, n_r, n_t, dr, dt, max_outer, tol);
  } catch (...) {
    return MBIR_ENOMEM;
  }
}
int32_t mbir_server_poll(mbir_server* s, int64_t id, int32_t* state, double* latency_ms,
                         int32_t* outer_done, double* cost) {
  if (!s) return MBIR_EINVAL;
  int st = 0, od = 0;
  int rc = s->impl->poll(id, &st, latency_ms, &od, cost);
  if (state) *state = st;
  if (outer_done) *outer_done = od;
  return rc;
}
int32_t mbir_server_wait(mbir_server* s, int64_t id, double timeout_s) {
  return s ? s->impl->wait(id, timeout_s) : MBIR_EINVAL;
}
int32_t mbir_server_result(mbir_server* s, int64_t id, float* out, int64_t n, int32_t* dims) {
  return s ? s->impl->result(id, out, n, dims) : MBIR_EINVAL;
}
int32_t mbir_server_release(mbir_server* s, int64_t id) {
  return s ? s->impl->release(id) : MBIR_EINVAL;
}
int32_t mbir_server_get_stats(mbir_server* s, mbir_server_stats* st) {
  if (!s || !st) return MBIR_EINVAL;
  mbir::ServerStats x;
  int rc = s->impl->stats(&x);
  st->submitted = x.submitted;
  st->completed = x.completed;
  st->failed = x.failed;
  st->active = x.active;
  st->queued = x.queued;
  st->p50_ms = x.p50_ms;
  st->p99_ms = x.p99_ms;
  st->mean_ms = x.mean_ms;
  st->voxel_updates = x.voxel_updates;
  st->busy_s = x.busy_s;
  st->batched_sweep_ms = x.batched_sweep_ms;
  st->batched_sweeps = x.batched_sweeps;
  st->budget_bytes = x.budget_bytes;
  st->peak_bytes = x.peak_bytes;
  st->peak_active = x.peak_active;
  st->reserved = 0;
  st->admitted = x.admitted;
  st->admitted_out_of_order = x.admitted_out_of_order;
  return rc;
}
const char* mbir_server_last_error(const mbir_server* s) {
  return s ? s->impl->last_error() : "null server";
}

int32_t mbir_level_schedule(int32_t n_z, int32_t n_x, int32_t n_theta, int32_t n_r, int32_t nb,
                            int32_t stride, const int32_t* rows, const uint8_t* lineok,
                            const uint8_t* active, const int16_t* lo, const uint16_t* mask,
                            int32_t* lines, int32_t lines_cap, int32_t* lofs, int32_t lofs_cap,
                            int32_t* n_lines, int32_t* n_levels) {
  if (!rows || !lineok || !lo || !mask || !lines || !lofs || !n_lines || !n_levels)
    return MBIR_EINVAL;
  if (n_z <= 0 || n_x <= 0 || n_theta <= 0 || n_r <= 0 || nb <= 0 || nb > 16 || stride <= 0)
    return MBIR_EINVAL;
  const size_t nl = static_cast<size_t>(n_z) * n_x;
  for (size_t i = 0; i < nl * n_theta; ++i) {
    if (!mask[i]) continue;
    if (mask[i] >> nb) return MBIR_EINVAL;
    for (int b = 0; b < nb; ++b)
      if (((mask[i] >> b) & 1u) && (lo[i] + b < 0 || lo[i] + b >= n_r)) return MBIR_EINVAL;
  }
  try {
    mbir::LevelScheduleIn in{n_z, n_x, n_theta, n_r, nb, stride, rows, lineok, active, lo, mask};
    mbir::LevelScheduleWork w;
    std::vector<int32_t> out, ofs;
    const int levels = mbir::level_schedule(in, w, out, ofs);
    if (levels < 0) return MBIR_EINVAL;
    if (static_cast<int64_t>(out.size()) > lines_cap ||
        static_cast<int64_t>(ofs.size()) > lofs_cap)
      return MBIR_EINVAL;
    std::copy(out.begin(), out.end(), lines);
    std::copy(ofs.begin(), ofs.end(), lofs);
    *n_lines = static_cast<int32_t>(out.size());
    *n_levels = levels;
    return MBIR_OK;
  } catch (...) {
    return MBIR_ENOMEM;
  }
}

int32_t mbir_colour_schedule(int32_t n_z, int32_t n_x, int32_t n_theta, int32_t n_r, int32_t nb,
                             int32_t max_colours, int32_t class_cap, const uint8_t* lineok,
                             const uint8_t* active,
                             const int16_t* lo, const uint16_t* mask, int32_t* lines,
                             int32_t lines_cap, int32_t* lofs, int32_t lofs_cap, int32_t* n_lines,
                             int32_t* n_colours) {
  if (!lineok || !lo || !mask || !lines || !lofs || !n_lines || !n_colours) return MBIR_EINVAL;
  if (n_z <= 0 || n_x <= 0 || n_theta <= 0 || n_r <= 0 || nb <= 0 || nb > 16 ||
      max_colours <= 0 || max_colours > 4096 || class_cap < 0)
    return MBIR_EINVAL;
  const size_t nl = static_cast<size_t>(n_z) * n_x;
  for (size_t i = 0; i < nl * n_theta; ++i) {
    if (!mask[i]) continue;
    if (mask[i] >> nb) return MBIR_EINVAL;
    for (int b = 0; b < nb; ++b)
      if (((mask[i] >> b) & 1u) && (lo[i] + b < 0 || lo[i] + b >= n_r)) return MBIR_EINVAL;
  }
  try {
    mbir::LevelScheduleIn in{n_z, n_x, n_theta, n_r, nb, 1, nullptr, lineok, active, lo, mask};
    mbir::LevelScheduleWork w;
    std::vector<int32_t> out, ofs;
    const int colours = mbir::colour_schedule(in, max_colours, class_cap, w, out, ofs);
    if (colours < 0) return MBIR_EINVAL;
    if (static_cast<int64_t>(out.size()) > lines_cap ||
        static_cast<int64_t>(ofs.size()) > lofs_cap)
      return MBIR_EINVAL;
    std::copy(out.begin(), out.end(), lines);
    std::copy(ofs.begin(), ofs.end(), lofs);
    *n_lines = static_cast<int32_t>(out.size());
    *n_colours = colours;
    return MBIR_OK;
  } catch (...) {
    return MBIR_ENOMEM;
  }
}

}  // extern "C"
