// compat_classes.cpp -- test program for the C++ classes of include/mbir_gb300.hpp, driven by
// tests/test_cpp_classes.py.  Prints one "key value" line per checked quantity.
//
//   compat_classes errors <scratch dir>
//       error paths that need no GPU: an engine without a sinogram, results read before a load,
//       a pipeline whose output directory cannot be made, a pipeline cancelled before it runs
//   compat_classes run <counts.f32> <tilts.f32> n_theta n_r n_t thickness <out.f32>
//       a HAADF reconstruction through HAADF_ReconstructionEngine from arrays, executed twice
//       on the same object; writes the first volume ([z][x][y] float32) and says whether the
//       second equals it and how many "Reconstruction Complete" messages the observer saw
//   compat_classes cancel <counts.f32> <tilts.f32> n_theta n_r n_t thickness
//       setCancel(true) from another thread once the first sweep is done
//   compat_classes levels
//       the per-level parameters of a three-level pipeline
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "mbir_gb300.hpp"

namespace {

template <typename T>
bool read_file(const char* path, std::vector<T>& out, size_t n) {
  out.assign(n, T());
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  const size_t got = std::fread(out.data(), sizeof(T), n, f);
  std::fclose(f);
  return got == n;
}

// the parameters of the tests' small HAADF case (five outer iterations, fixed voxel-group shape)
void small_case_params(mbir_params& p, double thickness) {
  p.sample_thickness = thickness;
  p.diffuseness = 0.1;
  p.sigma_x = 0.2;
  p.num_resolutions = 1;
  p.outer_iterations = 5;
  p.inner_iterations = 1;
  p.stop_threshold = 0.0;
  p.lane_shape = 1;
  p.seed_mode = MBIR_SEED_FIXED;
}

int errors(const std::string& dir) {
  {
    mbir_gb300::HAADF_ReconstructionEngine::Pointer e = mbir_gb300::HAADF_ReconstructionEngine::New();
    std::vector<float> vol;
    std::printf("volume_before_load %d\n", e->getVolume(vol));
    const int rc = e->execute();
    std::printf("no_sinogram %d %d %d\n", rc, e->getErrorCondition(),
                e->getErrorMessage().empty() ? 0 : 1);
  }
  {
    // a regular file where the output directory should go
    const std::string blocker = dir + "/not_a_directory";
    if (FILE* f = std::fopen(blocker.c_str(), "wb")) std::fclose(f);
    mbir_gb300::HAADF_MultiResolutionReconstruction m;
    std::string seen;
    m.setMessageHandler([&](const std::string& s) { seen += s; });
    m.setInputFile(dir + "/missing.mrc");
    m.setOutputFile(blocker + "/out/recon.mrc");
    const int rc = m.execute();
    std::printf("output_dir %d %d %d\n", rc, m.getErrorCondition(),
                seen.find("Error creating the output directory") != std::string::npos ? 1 : 0);
  }
  {
    mbir_gb300::BFMultiResolutionReconstruction m;
    m.setInputFile(dir + "/missing.mrc");
    m.setOutputFile(dir + "/bf/recon.mrc");
    m.setCancel(true);
    const int rc = m.execute();
    std::printf("cancel_before %d %d\n", rc, m.getCancel() ? 1 : 0);
  }
  return 0;
}

int levels() {
  mbir_gb300::HAADF_MultiResolutionReconstruction m;
  m.setNumberResolutions(3);
  m.setFinalResolution(2);
  m.setSigmaX(0.3);
  m.setMRFShapeParameter(0.2);
  m.setStopThreshold(0.005);
  m.setInnerIterations(10);
  m.setOuterIterations(7);
  m.setDefaultVariance(2.0);
  m.setInitialReconstructionValue(0.5);
  m.setDefaultOffsetValue(0.1);
  m.setUseDefaultOffset(true);
  m.setInterpolateInitialReconstruction(false);
  for (int i = 0; i < m.numberOfLevels(); ++i) {
    const mbir_params q = m.levelParams(i);
    std::printf("level%d %d %d %d %d %d %d %d\n", i, q.level, m.levelFactor(i), q.inner_iterations,
                q.outer_iterations, q.use_default_offset, q.interpolate_initial_recon,
                q.float_params);
    std::printf("level%d_f %.17g %.17g %.17g %.17g %.17g %.17g\n", i, q.sigma_x, q.qggmrf_q,
                q.stop_threshold, q.default_recon_value, q.default_variance, q.default_offset);
  }
  return 0;
}

int run(char** argv, bool cancel) {
  const int n_theta = std::atoi(argv[4]), n_r = std::atoi(argv[5]), n_t = std::atoi(argv[6]);
  const double thickness = std::atof(argv[7]);
  std::vector<float> counts, tilts;
  if (!read_file(argv[2], counts, static_cast<size_t>(n_theta) * n_r * n_t) ||
      !read_file(argv[3], tilts, n_theta)) {
    std::printf("input_error 1\n");
    return 1;
  }
  mbir_gb300::HAADF_ReconstructionEngine e;
  small_case_params(e.params(), thickness);
  e.setSinogram(counts.data(), tilts.data(), n_theta, n_r, n_t, 1.0, 1.0);
  if (!cancel) {
    int complete = 0;
    e.setObserver([&](const std::string& m, int progress, int aspect) {
      if (m == "Reconstruction Complete" && progress == 100 &&
          aspect == MBIR_UPDATE_PROGRESS_VALUE_AND_MESSAGE)
        ++complete;
    });
    const int rc = e.execute();
    std::printf("execute %d\n", rc);
    std::vector<float> vol, vol2;
    if (rc != MBIR_OK || e.getVolume(vol) != MBIR_OK) return 1;
    const int32_t* d = e.getDims();
    std::printf("dims %d %d %d %d %d %d\n", d[0], d[1], d[2], d[3], d[4], d[5]);
    std::vector<double> g, o, v;
    std::printf("nuisance %d %zu\n", e.getNuisance(g, o, v), g.size());
    std::printf("execute_again %d\n", e.execute());
    if (e.getVolume(vol2) != MBIR_OK) return 1;
    std::printf("same_volume %d\n", vol == vol2 ? 1 : 0);
    std::printf("complete %d\n", complete);
    FILE* f = std::fopen(argv[8], "wb");
    if (!f) return 1;
    std::fwrite(vol.data(), sizeof(float), vol.size(), f);
    std::fclose(f);
    return 0;
  }
  // many iterations, cancelled from this thread while execute() runs on another
  e.params().outer_iterations = 100000;
  if (e.load() != MBIR_OK) {
    std::printf("load %d\n", e.getErrorCondition());
    return 1;
  }
  int rc = 1;
  std::thread worker([&] { rc = e.execute(); });
  mbir_status st{};
  const auto t0 = std::chrono::steady_clock::now();
  while (std::chrono::steady_clock::now() - t0 < std::chrono::seconds(60)) {
    if (mbir_status_get(e.handle(), &st) == MBIR_OK && st.sweeps_done >= 1) break;
    std::this_thread::sleep_for(std::chrono::milliseconds(1));
  }
  e.setCancel(true);
  worker.join();
  mbir_status_get(e.handle(), &st);
  std::printf("cancel %d %d %d\n", rc, e.getErrorCondition(), st.sweeps_done < 100000 ? 1 : 0);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 3 && std::strcmp(argv[1], "errors") == 0) return errors(argv[2]);
  if (argc >= 2 && std::strcmp(argv[1], "levels") == 0) return levels();
  if (argc >= 9 && std::strcmp(argv[1], "run") == 0) return run(argv, false);
  if (argc >= 8 && std::strcmp(argv[1], "cancel") == 0) return run(argv, true);
  std::fprintf(stderr, "usage: compat_classes errors|levels|run|cancel ...\n");
  return 2;
}
