/*
 * mbir_gb300.hpp -- C++ classes over the C ABI (mbir_gb300.h) in the shape of the reference's
 * engine and pipeline classes, so code written against the reference's classes moves over with
 * its setter / execute() / getErrorCondition() pattern.  Header only; link libmbir_gb300.so.
 *
 *   ReconstructionEngine (HAADF_ReconstructionEngine / BFReconstructionEngine)
 *     reference: Code/MBIRLib/HAADF/HAADF_ReconstructionEngine.h:67-99,
 *                Code/MBIRLib/BrightField/BFReconstructionEngine.h; setCancel / getCancel /
 *                getErrorCondition / getErrorMessage of Code/MBIRLib/Common/AbstractFilter.h:46-82
 *   MultiResolutionReconstruction (HAADF_MultiResolutionReconstruction /
 *                                  BFMultiResolutionReconstruction)
 *     reference: Code/MBIRLib/HAADF/HAADF_MultiResolutionReconstruction.h:55-103 (properties),
 *                HAADF_MultiResolutionReconstruction.cpp:175-485 (execute),
 *                Code/MBIRLib/BrightField/BFMultiResolutionReconstruction.h:66-107
 *
 * The reference's TomoInputs / Sinogram / Geometry / AdvancedParameters structs are one
 * mbir_params here (params()); the engine reads its inputs from arrays or an MRC file instead of
 * a filled Sinogram.  Messages the reference sends to its observers (Observable::notify) go to
 * the handler given to setMessageHandler.  No exception leaves these classes except
 * std::bad_alloc from the host vectors that hold copies of the inputs.
 *
 * Threading: execute() blocks; setCancel(true) may be called from another thread while it runs
 * (the engine stops at its next check and execute() ends with MBIR_ECANCELLED, the reference's
 * -999).  A cancel set before execute() makes it end with MBIR_ECANCELLED without running.
 */
#ifndef MBIR_GB300_HPP_
#define MBIR_GB300_HPP_

#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "mbir_gb300.h"

namespace mbir_gb300 {

using MessageHandler = std::function<void(const std::string&)>;
/* an engine's messages: text, progress (0-100) and MBIR_UPDATE_* aspect (mbir_set_observer) */
using Observer = std::function<void(const std::string& msg, int progress, int aspect)>;

namespace detail {

inline std::string parent_path(const std::string& f) {
  const size_t k = f.find_last_of('/');
  return k == std::string::npos ? "." : (k == 0 ? "/" : f.substr(0, k));
}
inline std::string stem(const std::string& f) {
  const size_t k = f.find_last_of('/');
  std::string b = k == std::string::npos ? f : f.substr(k + 1);
  const size_t d = b.find_last_of('.');
  return d == std::string::npos ? b : b.substr(0, d);
}
// creates every missing directory of d (mkdir -p)
inline bool make_dirs(const std::string& d) {
  std::string acc;
  for (size_t i = 0; i <= d.size(); ++i) {
    if (i == d.size() || d[i] == '/') {
      if (!acc.empty()) {
        struct stat st;
        if (stat(acc.c_str(), &st) != 0 && mkdir(acc.c_str(), 0755) != 0) return false;
      }
    }
    if (i < d.size()) acc.push_back(d[i]);
  }
  return true;
}
// an initial reconstruction file: doubles in y-x-z order (InitialReconstructionBinReader.cpp:
// 101-155), returned as [z][x][y] of the given size
inline bool read_object_bin(const std::string& path, int n_z, int n_x, int n_y,
                            std::vector<double>& out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::vector<double> buf(static_cast<size_t>(n_z) * n_x * n_y);
  const size_t got = std::fread(buf.data(), sizeof(double), buf.size(), f);
  std::fclose(f);
  if (got != buf.size()) return false;
  out.assign(buf.size(), 0.0);
  size_t k = 0;
  for (int y = 0; y < n_y; ++y)
    for (int x = 0; x < n_x; ++x)
      for (int z = 0; z < n_z; ++z) out[(static_cast<size_t>(z) * n_x + x) * n_y + y] = buf[k++];
  return true;
}
inline bool file_exists(const std::string& path) {
  struct stat st;
  return stat(path.c_str(), &st) == 0;
}

}  // namespace detail

/* One reconstruction at one resolution level.  Set the parameters and the inputs, then
 * execute(); the results stay readable until the next execute() or destruction. */
class ReconstructionEngine {
 public:
  using Pointer = std::shared_ptr<ReconstructionEngine>;
  static Pointer New(int32_t modality) { return Pointer(new ReconstructionEngine(modality)); }

  explicit ReconstructionEngine(int32_t modality) { mbir_params_default(&p_, modality); }
  virtual ~ReconstructionEngine() { release(); }
  ReconstructionEngine(const ReconstructionEngine&) = delete;
  ReconstructionEngine& operator=(const ReconstructionEngine&) = delete;

  /* TomoInputs, Geometry and AdvancedParameters in one struct; edits apply at the next load */
  mbir_params& params() { return p_; }
  const mbir_params& params() const { return p_; }
  void setParams(const mbir_params& p) { p_ = p; }

  /* the tilt series, copied: counts[theta][r][t] (t fastest), tilts in degrees, pitch in nm */
  void setSinogram(const float* counts, const float* tilts_deg, int32_t n_theta, int32_t n_r,
                   int32_t n_t, double delta_r, double delta_t) {
    sino_file_.clear();
    counts_.assign(counts, counts + static_cast<size_t>(n_theta) * n_r * n_t);
    tilts_.assign(tilts_deg, tilts_deg + n_theta);
    n_theta_ = n_theta;
    n_r_ = n_r;
    n_t_ = n_t;
    delta_r_ = delta_r;
    delta_t_ = delta_t;
    loaded_ = false;
  }
  /* ... or an MRC tilt series, read with params().subvolume / tilt_selection / excluded views */
  void setSinogramFile(const std::string& mrc_path) {
    sino_file_ = mrc_path;
    counts_.clear();
    tilts_.clear();
    loaded_ = false;
  }
  /* HAADF: the bright-field series of the same views (setUseBrightFieldData + setBFSinogram) */
  void setBrightField(const float* counts, int32_t n_theta, int32_t n_r, int32_t n_t) {
    bf_file_.clear();
    bf_counts_.assign(counts, counts + static_cast<size_t>(n_theta) * n_r * n_t);
    bf_dims_[0] = n_theta;
    bf_dims_[1] = n_r;
    bf_dims_[2] = n_t;
    loaded_ = false;
  }
  void setBrightFieldFile(const std::string& mrc_path) {
    bf_file_ = mrc_path;
    bf_counts_.clear();
    loaded_ = false;
  }
  /* initial volume [z][x][y] in FP64 (half size per axis with interpolate_initial_recon) */
  void setInitialVolume(std::vector<double> zxy) { init_ = std::move(zxy); }
  /* initial gains, offsets and variances, one of each per view */
  void setInitialNuisance(std::vector<double> g, std::vector<double> o, std::vector<double> v) {
    init_g_ = std::move(g);
    init_o_ = std::move(o);
    init_v_ = std::move(v);
  }
  /* HAADF: write <dir>/<outer>_<inner>_ReconstructedVolume.rec after every inner iteration */
  void setIntermediateDir(const std::string& dir) { inter_dir_ = dir; }
  /* the engine's progress, intermediate-image and error messages (the reference's observers);
   * takes effect at the next load */
  void setObserver(Observer o) { observer_ = std::move(o); }
  /* HAADF: resume from a checkpoint directory (mbir_read_checkpoint) at every load; an initial
   * volume or nuisance set here as well would replace the checkpoint's.  "" turns it off. */
  void setResumeCheckpoint(const std::string& dir) {
    resume_dir_ = dir;
    loaded_ = false;
  }

  void setCancel(bool v) {
    cancel_.store(v);
    std::lock_guard<std::mutex> lk(mu_);
    if (v && e_) mbir_cancel(e_);
  }
  bool getCancel() const { return cancel_.load(); }
  int getErrorCondition() const { return err_; }
  const std::string& getErrorMessage() const { return msg_; }

  /* Creates the engine and reads the inputs: the volume and sinogram sizes are known after it
   * (getDims).  execute() calls it when it has not run since the last input change. */
  int load() {
    release();
    mbir_engine* e = mbir_create(&p_);
    if (!e) return fail(MBIR_EDEVICE, mbir_last_error(nullptr));
    {
      std::lock_guard<std::mutex> lk(mu_);
      e_ = e;
    }
    if (observer_) mbir_set_observer(e_, &ReconstructionEngine::forward_message, this);
    int rc;
    if (!sino_file_.empty())
      rc = mbir_load_sinogram_mrc(e_, sino_file_.c_str());
    else if (!counts_.empty())
      rc = mbir_set_sinogram(e_, counts_.data(), tilts_.data(), n_theta_, n_r_, n_t_, delta_r_,
                             delta_t_);
    else
      return fail(MBIR_ESTATE, "no sinogram set");
    if (rc == MBIR_OK && !bf_file_.empty())
      rc = mbir_load_bright_field_mrc(e_, bf_file_.c_str());
    else if (rc == MBIR_OK && !bf_counts_.empty())
      rc = mbir_set_bright_field(e_, bf_counts_.data(), bf_dims_[0], bf_dims_[1], bf_dims_[2]);
    if (rc == MBIR_OK && !resume_dir_.empty()) rc = mbir_read_checkpoint(e_, resume_dir_.c_str());
    if (rc == MBIR_OK) rc = mbir_get_dims(e_, dims_);
    if (rc != MBIR_OK) return fail(rc, mbir_last_error(e_));
    loaded_ = true;
    return ok();
  }

  /* Runs the reconstruction (HAADF_ReconstructionEngine::execute); the result is also
   * getErrorCondition(): MBIR_OK, MBIR_ECANCELLED or another MBIR_E* code */
  int execute() {
    if (!loaded_ && load() != MBIR_OK) return err_;
    loaded_ = false;  // a second execute() starts again from the inputs
    int rc = MBIR_OK;
    if (!init_.empty())
      rc = mbir_set_initial_volume_f64(e_, init_.data(), static_cast<int64_t>(init_.size()));
    if (rc == MBIR_OK && !init_g_.empty()) {
      if (init_g_.size() != static_cast<size_t>(dims_[3]) || init_o_.size() != init_g_.size() ||
          init_v_.size() != init_g_.size())
        return fail(MBIR_EINVAL, "initial nuisance: one gain, offset and variance per view");
      rc = mbir_set_initial_nuisance(e_, init_g_.data(), init_o_.data(), init_v_.data());
    }
    if (rc == MBIR_OK && !inter_dir_.empty())
      rc = mbir_set_intermediate_dir(e_, inter_dir_.c_str());
    if (rc == MBIR_OK && cancel_.load()) mbir_cancel(e_);
    if (rc == MBIR_OK) rc = mbir_run(e_);
    if (rc != MBIR_OK) return fail(rc, mbir_last_error(e_));
    return ok();
  }

  /* dims[0..2] = N_z, N_x, N_y; dims[3..5] = N_theta, N_r, N_t (after load or execute) */
  const int32_t* getDims() const { return dims_; }
  int64_t voxelCount() const { return static_cast<int64_t>(dims_[0]) * dims_[1] * dims_[2]; }
  int getVolume(std::vector<float>& out) {
    if (!e_) return not_loaded();
    out.assign(static_cast<size_t>(voxelCount()), 0.0f);
    return check(mbir_get_volume(e_, out.data(), voxelCount()));
  }
  int getVolumeF64(std::vector<double>& out) {
    if (!e_) return not_loaded();
    out.assign(static_cast<size_t>(voxelCount()), 0.0);
    return check(mbir_get_volume_f64(e_, out.data(), voxelCount()));
  }
  int getNuisance(std::vector<double>& g, std::vector<double>& o, std::vector<double>& v) {
    if (!e_) return not_loaded();
    g.assign(dims_[3], 0.0);
    o.assign(dims_[3], 0.0);
    v.assign(dims_[3], 0.0);
    return check(mbir_get_nuisance(e_, g.data(), o.data(), v.data()));
  }
  int getStatus(mbir_status& st) {
    if (!e_) return not_loaded();
    return check(mbir_status_get(e_, &st));
  }
  /* HAADF: the run's state in dir, for setResumeCheckpoint (mbir_write_checkpoint) */
  int writeCheckpoint(const std::string& dir) {
    if (!e_) return not_loaded();
    return check(mbir_write_checkpoint(e_, dir.c_str()));
  }
  /* the reference's output files in dir, and the MRC / VTK / Avizo volumes where a path is set */
  int writeOutputs(const std::string& dir, const std::string& mrc = std::string(),
                   const std::string& vtk = std::string(), const std::string& am = std::string()) {
    if (!e_) return not_loaded();
    auto c = [](const std::string& s) { return s.empty() ? nullptr : s.c_str(); };
    return check(mbir_write_outputs_ex(e_, dir.c_str(), c(mrc), c(vtk), c(am)));
  }
  /* the C ABI handle, for the step-wise entry points (NULL before load) */
  mbir_engine* handle() { return e_; }

 private:
  static void forward_message(const char* msg, int32_t progress, int32_t aspect, void* self) {
    try {
      static_cast<ReconstructionEngine*>(self)->observer_(msg ? msg : "", progress, aspect);
    } catch (...) {
      // an observer's exception must not cross the C ABI
    }
  }
  int ok() {
    err_ = MBIR_OK;
    msg_.clear();
    return MBIR_OK;
  }
  int fail(int rc, const char* m) {
    err_ = rc;
    msg_ = m ? m : "";
    return rc;
  }
  int not_loaded() { return fail(MBIR_ESTATE, "engine not loaded: call load() or execute()"); }
  int check(int rc) { return rc == MBIR_OK ? ok() : fail(rc, mbir_last_error(e_)); }
  void release() {
    std::lock_guard<std::mutex> lk(mu_);
    if (e_) mbir_destroy(e_);
    e_ = nullptr;
    loaded_ = false;
  }

  mbir_params p_{};
  std::string sino_file_, bf_file_, inter_dir_, resume_dir_;
  std::vector<float> counts_, tilts_, bf_counts_;
  int32_t n_theta_ = 0, n_r_ = 0, n_t_ = 0, bf_dims_[3] = {0, 0, 0};
  double delta_r_ = 1.0, delta_t_ = 1.0;
  std::vector<double> init_, init_g_, init_o_, init_v_;
  int32_t dims_[6] = {0, 0, 0, 0, 0, 0};
  Observer observer_;
  mbir_engine* e_ = nullptr;
  bool loaded_ = false;
  std::mutex mu_;  // guards e_ against a concurrent setCancel
  std::atomic<bool> cancel_{false};
  int err_ = MBIR_OK;
  std::string msg_;
};

class HAADF_ReconstructionEngine : public ReconstructionEngine {
 public:
  using Pointer = std::shared_ptr<HAADF_ReconstructionEngine>;
  static Pointer New() { return Pointer(new HAADF_ReconstructionEngine()); }
  HAADF_ReconstructionEngine() : ReconstructionEngine(MBIR_MODALITY_HAADF) {}
};

class BFReconstructionEngine : public ReconstructionEngine {
 public:
  using Pointer = std::shared_ptr<BFReconstructionEngine>;
  static Pointer New() { return Pointer(new BFReconstructionEngine()); }
  BFReconstructionEngine() : ReconstructionEngine(MBIR_MODALITY_BF) {}
};

/* The coarse-to-fine pipeline from an MRC tilt series (HAADF_MultiResolutionReconstruction::
 * execute, HAADF_MultiResolutionReconstruction.cpp:175-485; BFMultiResolutionReconstruction.cpp:
 * 175-520).  Per level i of L: voxels of 2^(L-1-i) * final_resolution detector pixels,
 * sigma_x * 2^((L-1-i)(1-3/p)) with p = diffuseness + 1 in float, one inner iteration after the
 * first level, the stop threshold doubled from the third level, the previous level's volume
 * replicated 2x2x2 and its gains, offsets and variances handed on.  Each level writes
 * ReconstructedObject.bin, Final*Parameters.bin, FinalVariances.bin and
 * ReconstructedSinogram.bin to <dir of OutputFile>/<factor>x/ (and, HAADF, the intermediate
 * <outer>_<inner>_ReconstructedVolume.rec images); the last level writes OutputFile (MRC) and,
 * beside it, <stem>.vtk and <stem>.am.  Float properties are rounded as the reference's float
 * members round them (mbir_params.float_params = 1). */
class MultiResolutionReconstruction {
 public:
  explicit MultiResolutionReconstruction(int32_t modality) {
    mbir_params_default(&p_, modality);
    p_.float_params = 1;
    p_.use_subvolume = 1;  // the reference always hands the engine a subvolume (zeros: all)
    if (modality == MBIR_MODALITY_BF) p_.extend_object = 1;  // the BF pipeline's default
  }
  virtual ~MultiResolutionReconstruction() = default;

  void setInputFile(const std::string& v) { input_ = v; }
  const std::string& getInputFile() const { return input_; }
  void setOutputFile(const std::string& v) { output_ = v; }
  const std::string& getOutputFile() const { return output_; }
  /* the level directories go under the output file's directory, as the reference's programs set
   * TempDir; a TempDir set here takes their place */
  void setTempDir(const std::string& v) { temp_dir_ = v; }
  const std::string& getTempDir() const { return temp_dir_; }
  void setBrightFieldFile(const std::string& v) { bright_field_ = v; }
  void setInitialReconstructionFile(const std::string& v) { initial_file_ = v; }
  void setDeleteTempFiles(bool v) { delete_temp_ = v; }
  void setNumberResolutions(int v) { p_.num_resolutions = v; }
  void setSampleThickness(double v) { p_.sample_thickness = v; }
  void setTargetGain(double v) { p_.target_gain = v; }
  void setStopThreshold(double v) { p_.stop_threshold = v; }
  void setOuterIterations(int v) { p_.outer_iterations = v; }
  void setInnerIterations(int v) { p_.inner_iterations = v; }
  void setSigmaX(double v) { p_.sigma_x = v; }
  /* the --diffuseness value (the prior's q is this + 1) */
  void setMRFShapeParameter(double v) { p_.diffuseness = v; }
  void setDefaultOffsetValue(double v) { p_.default_offset = v; }
  void setUseDefaultOffset(bool v) { p_.use_default_offset = v ? 1 : 0; }
  void setFinalResolution(int v) { p_.final_resolution = v; }
  void setExtendObject(bool v) { p_.extend_object = v ? 1 : 0; }
  void setInterpolateInitialReconstruction(bool v) { interpolate_ = v; }
  void setDefaultVariance(double v) { p_.default_variance = v; }
  void setInitialReconstructionValue(double v) { p_.default_recon_value = v; }
  void setDefaultPixelSize(double v) { p_.default_pixel_size = v; }
  /* 0: the FEI header's a-tilts, 1: its b-tilts (the reference's programs pick the tilts this way
   * before they call setTilts) */
  void setTiltSelection(int v) { p_.tilt_selection = v; }
  /* xmin, ymin, zmin, xmax, ymax, zmax; six zeros (the default) read the whole file */
  void setSubvolume(const std::vector<int>& v) {
    for (int i = 0; i < 6; ++i) p_.subvolume[i] = i < static_cast<int>(v.size()) ? v[i] : 0;
  }
  /* indices of the views to leave out (the reference's ViewMasks); at most 256 */
  bool setViewMasks(const std::vector<int>& v) {
    if (v.size() > 256) return false;
    p_.n_excluded_views = static_cast<int32_t>(v.size());
    for (size_t i = 0; i < v.size(); ++i) p_.excluded_views[i] = v[i];
    return true;
  }
  /* every other field (advanced parameters, precision, order, device); the level-dependent
   * fields are set per level by execute() */
  mbir_params& params() { return p_; }

  void setMessageHandler(MessageHandler h) { notify_ = std::move(h); }
  /* the running level's engine messages (ReconstructionEngine::setObserver) */
  void setObserver(Observer o) { observer_ = std::move(o); }
  void setCancel(bool v) {
    cancel_.store(v);
    std::lock_guard<std::mutex> lk(mu_);
    if (v && current_) current_->setCancel(true);
  }
  bool getCancel() const { return cancel_.load(); }
  int getErrorCondition() const { return err_; }
  const std::string& getErrorMessage() const { return msg_; }

  /* Runs every level; MBIR_OK or the failing level's MBIR_E* code (getErrorMessage says why) */
  int execute() {
    err_ = MBIR_OK;
    msg_.clear();
    const std::string out_dir = temp_dir_.empty() ? detail::parent_path(output_) : temp_dir_;
    if (!detail::make_dirs(out_dir))
      return fail(MBIR_EIO, "Error creating the output directory '" + out_dir +
                                "'\n   Exiting Now.");
    const bool bf = p_.modality == MBIR_MODALITY_BF;
    const int levels = numberOfLevels();
    std::vector<double> prev, g, o, v;
    std::vector<std::string> temp_files;
    for (int i = 0; i < levels; ++i) {
      if (cancel_.load()) return fail(MBIR_ECANCELLED, "cancelled");
      const mbir_params q = levelParams(i);
      const std::string level_dir = out_dir + "/" + std::to_string(levelFactor(i)) + "x";
      if (!detail::make_dirs(level_dir)) return fail(MBIR_EIO, "Could not create path: " + level_dir);
      auto eng = std::make_shared<ReconstructionEngine>(q.modality);
      eng->setParams(q);
      if (observer_) eng->setObserver(observer_);
      eng->setSinogramFile(input_);
      if (!bf && !bright_field_.empty()) eng->setBrightFieldFile(bright_field_);
      {
        std::lock_guard<std::mutex> lk(mu_);
        current_ = eng;
      }
      if (cancel_.load()) eng->setCancel(true);  // a cancel that came before current_ was set
      int rc = eng->load();
      const int32_t* d = eng->getDims();
      if (rc == MBIR_OK && i == 0 && !initial_file_.empty()) {
        const int f = q.interpolate_initial_recon ? 2 : 1;
        std::vector<double> init;
        if (!detail::read_object_bin(initial_file_, d[0] / f, d[1] / f, d[2] / f, init))
          return fail(MBIR_EIO, "Error opening Input file '" + initial_file_ + "'");
        eng->setInitialVolume(std::move(init));
      }
      if (rc == MBIR_OK && i > 0) {
        eng->setInitialVolume(prev);
        eng->setInitialNuisance(g, o, v);
      }
      if (rc == MBIR_OK)
        message(std::to_string(levelFactor(i)) + "x: reconstructing " + std::to_string(d[0]) +
                " x " + std::to_string(d[1]) + " x " + std::to_string(d[2]) +
                " voxels (z, x, y) from " + std::to_string(d[3]) + " views");
      // the HAADF program's intermediate images, <outer>_<inner>_ReconstructedVolume.rec
      if (rc == MBIR_OK && !bf) eng->setIntermediateDir(level_dir);
      if (rc == MBIR_OK) rc = eng->execute();
      if (rc == MBIR_OK) {
        const bool last = i == levels - 1;
        const std::string base = detail::parent_path(output_) + "/" + detail::stem(output_);
        rc = last ? eng->writeOutputs(level_dir, output_, base + ".vtk", base + ".am")
                  : eng->writeOutputs(level_dir);
        for (const char* n : {"ReconstructedObject.bin", "FinalGainParameters.bin",
                              "FinalOffsetParameters.bin", "FinalVariances.bin",
                              "ReconstructedSinogram.bin"})
          temp_files.push_back(level_dir + "/" + n);
        for (int it = 0; it < q.outer_iterations; ++it)
          for (int k = 0; k < std::max(1, q.inner_iterations); ++k) {
            const std::string rec = level_dir + "/" + std::to_string(it) + "_" +
                                    std::to_string(k) + "_ReconstructedVolume.rec";
            if (detail::file_exists(rec)) temp_files.push_back(rec);
          }
      }
      if (rc == MBIR_OK) rc = eng->getVolumeF64(prev);
      if (rc == MBIR_OK) rc = eng->getNuisance(g, o, v);
      if (rc != MBIR_OK)
        return fail(rc, eng->getErrorMessage() + "\nError Reconstructing the Data");
      for (int k = 0; k < 3; ++k) dims_[k] = d[k];
      mbir_status st{};
      eng->getStatus(st);
      message(std::to_string(levelFactor(i)) + "x: " + std::to_string(st.sweeps_done) +
              " ICD calls, " + std::to_string(static_cast<long long>(st.voxels_updated)) +
              " voxel updates, ICD device time " + fixed1(st.icd_ms_total) + " ms");
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      current_.reset();
    }
    if (delete_temp_)
      for (const std::string& f : temp_files) std::remove(f.c_str());
    final_ = std::move(prev);
    gains_ = std::move(g);
    offsets_ = std::move(o);
    variances_ = std::move(v);
    return MBIR_OK;
  }

  /* the levels execute() runs, and the parameters of level i (0 = coarsest): the settings
   * above with the per-level rules of HAADF_MultiResolutionReconstruction.cpp:318-357 */
  int numberOfLevels() const { return p_.num_resolutions > 0 ? p_.num_resolutions : 1; }
  /* voxel size of level i in detector pixels, the name of its directory (<factor>x) */
  int levelFactor(int i) const {
    return ((1 << (numberOfLevels() - 1)) * std::max(1, p_.final_resolution)) >> i;
  }
  mbir_params levelParams(int i) const {
    const int levels = numberOfLevels();
    // p = diffuseness + 1 in float, as the pipeline computes it
    const double pq = static_cast<double>(static_cast<float>(p_.diffuseness) + 1.0f);
    mbir_params q = p_;
    q.level = i;
    q.qggmrf_q = pq;
    q.sigma_x = std::pow(2.0, (levels - 1 - i) * (1 - 3 / pq)) *
                static_cast<double>(static_cast<float>(p_.sigma_x));
    if (i > 0) {
      q.inner_iterations = 1;
      // later levels take the nuisance and the volume from the level before
      q.default_recon_value = 0.0;
      q.default_variance = 1.0;
      q.use_default_offset = 0;
      q.default_offset = 0.0;
    }
    if (i >= 2) q.stop_threshold = static_cast<float>(p_.stop_threshold) * 2.0f;
    q.interpolate_initial_recon = i == 0 ? (interpolate_ ? 1 : 0) : 1;
    return q;
  }

  /* after execute(): N_z, N_x, N_y of the final level, its volume [z][x][y] and nuisance */
  const int32_t* getDims() const { return dims_; }
  const std::vector<double>& getVolume() const { return final_; }
  const std::vector<double>& getGains() const { return gains_; }
  const std::vector<double>& getOffsets() const { return offsets_; }
  const std::vector<double>& getVariances() const { return variances_; }

 protected:
  mbir_params p_{};

 private:
  static std::string fixed1(double x) {
    char b[64];
    std::snprintf(b, sizeof b, "%.1f", x);
    return b;
  }
  void message(const std::string& m) {
    if (notify_) notify_(m);
  }
  int fail(int rc, const std::string& m) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      current_.reset();
    }
    err_ = rc;
    msg_ = m;
    message(m);
    return rc;
  }

  std::string input_, output_, temp_dir_, bright_field_, initial_file_;
  bool delete_temp_ = false, interpolate_ = false;
  MessageHandler notify_;
  Observer observer_;
  std::mutex mu_;  // guards current_ against a concurrent setCancel
  std::shared_ptr<ReconstructionEngine> current_;
  std::atomic<bool> cancel_{false};
  int err_ = MBIR_OK;
  std::string msg_;
  int32_t dims_[3] = {0, 0, 0};
  std::vector<double> final_, gains_, offsets_, variances_;
};

class HAADF_MultiResolutionReconstruction : public MultiResolutionReconstruction {
 public:
  HAADF_MultiResolutionReconstruction() : MultiResolutionReconstruction(MBIR_MODALITY_HAADF) {}
};

class BFMultiResolutionReconstruction : public MultiResolutionReconstruction {
 public:
  BFMultiResolutionReconstruction() : MultiResolutionReconstruction(MBIR_MODALITY_BF) {}
  void setBraggThreshold(double v) { p_.bragg_threshold = v; }
  void setBraggDelta(double v) { p_.bragg_delta = v; }
  void setBfOffset(double v) { p_.bf_offset = v; }
  /* --default_dosage and --use_default_dosage (the engine's default offset switch) */
  void setDefaultDosage(double v) { p_.default_dosage = v; }
  void setUseDefaultDosage(bool v) { p_.use_default_offset = v ? 1 : 0; }
};

}  // namespace mbir_gb300

#endif  // MBIR_GB300_HPP_
