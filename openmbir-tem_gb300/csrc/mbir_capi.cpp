// mbir_capi.cpp -- extern "C" boundary over mbir::Engine.  No C++ exception crosses it.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mbir_engine.h"

struct mbir_engine {
  mbir::Engine* impl;
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
}

mbir_engine* mbir_create(const mbir_params* p) {
  if (!p || p->struct_size != static_cast<int32_t>(sizeof(mbir_params))) {
    g_create_error = "mbir_create: params missing or struct_size mismatch";
    return nullptr;
  }
  if (p->modality != MBIR_MODALITY_HAADF) {
    g_create_error = "mbir_create: only the HAADF modality is built";
    return nullptr;
  }
  if (!(p->sigma_x > 0) || p->num_resolutions < 1 || p->final_resolution < 1 ||
      !(p->qggmrf_c > 0) || !(p->qggmrf_p > 0)) {
    g_create_error = "mbir_create: invalid parameter value";
    return nullptr;
  }
  try {
    auto* e = new mbir_engine;
    e->impl = new mbir::Engine(*p);
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
int32_t mbir_set_initial_volume(mbir_engine* e, const float* vol, int64_t n) {
  return guarded(e, [&](mbir::Engine& m) { return m.set_initial_volume(vol, n); });
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
int32_t mbir_status_get(mbir_engine* e, mbir_status* st) {
  return guarded(e, [&](mbir::Engine& m) { return m.status(st); });
}
void mbir_cancel(mbir_engine* e) {
  if (e && e->impl) e->impl->cancel();
}
int32_t mbir_write_outputs(mbir_engine* e, const char* dir, const char* mrc_path) {
  return guarded(e, [&](mbir::Engine& m) { return m.write_outputs(dir, mrc_path); });
}

// HAADF_MultiResolutionReconstruction::execute (HAADF_MultiResolutionReconstruction.cpp:175-485):
// per level i: sigma_x * 2^((levels-1-i)(1-3/p)), NumIter = 1 after the first level,
// stop threshold x2 from level 2, the previous level's volume replicated 2x in every
// direction (InitialReconstructionBinReader.cpp:104-135) and its nuisance vectors handed on.
int32_t mbir_run_multires(const mbir_params* p, const float* counts, const float* tilts_deg,
                          int32_t n_theta, int32_t n_r, int32_t n_t, double delta_r,
                          double delta_t, float* out, int64_t n, int32_t* dims_out) {
  if (!p || !counts || !tilts_deg) return MBIR_EINVAL;
  const int levels = p->num_resolutions > 0 ? p->num_resolutions : 1;
  std::vector<float> prev;
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
        // 2x voxel replication of the previous level (InterpFlag = 1)
        std::vector<float> up(static_cast<size_t>(d[0]) * d[1] * d[2], 0.f);
        const int ze = d[0] / 2, xe = d[1] / 2, ye = d[2] / 2;
        for (int y = 0; y < ye && y < pdims[2]; y++)
          for (int x = 0; x < xe && x < pdims[1]; x++)
            for (int z = 0; z < ze && z < pdims[0]; z++) {
              const float b = prev[(static_cast<size_t>(z) * pdims[1] + x) * pdims[2] + y];
              for (int a = 0; a < 2; a++)
                for (int c = 0; c < 2; c++)
                  for (int r = 0; r < 2; r++)
                    up[(static_cast<size_t>(2 * z + a) * d[1] + 2 * x + c) * d[2] + 2 * y + r] = b;
            }
        if ((rc = eng.set_initial_volume(up.data(), static_cast<int64_t>(up.size())))) return rc;
      }
      if ((rc = eng.run())) return rc;
      prev.assign(static_cast<size_t>(d[0]) * d[1] * d[2], 0.f);
      if ((rc = eng.get_volume(prev.data(), static_cast<int64_t>(prev.size())))) return rc;
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
    std::memcpy(out, prev.data(), nv * sizeof(float));
  }
  return MBIR_OK;
}

}  // extern "C"
