// mbir_reconstruct.cpp -- the reference's two reconstruction programs, HAADFReconstruction and
// BFReconstruction, over this library's C ABI.
//
// Built twice (MBIR_CLI_BF = 0 / 1) into openmbir-tem_gb300/bin/.  Each program accepts the flag
// set of the reference program of the same name (Code/Applications/HAADFReconstruction/
// HAADFReconstructionArgsParser.cpp:143-211, Code/Applications/BFReconstruction/
// BFReconstructionArgsParser.cpp:145-226) and runs the multi-resolution pipeline the way
// HAADF_MultiResolutionReconstruction::execute / BFMultiResolutionReconstruction::execute do
// (HAADF_MultiResolutionReconstruction.cpp:175-485): per level i of L, voxels of
// 2^(L-1-i) * final_resolution detector pixels, sigma_x * 2^((L-1-i)(1-3/p)), one inner iteration
// after the first level, the stop threshold doubled from level 2, the previous level's volume
// replicated 2x2x2 and its gains, offsets and variances handed on.  Each level writes its files
// (ReconstructedObject.bin, Final*Parameters.bin, FinalVariances.bin, ReconstructedSinogram.bin)
// to <output dir>/<factor>x/; the last one also writes the MRC output file and, beside it, the
// .vtk and .am volumes.  Parameters that the reference's pipeline keeps in float members are
// rounded the same way (mbir_params.float_params).  The bright-field program always extends the
// object (the reference's pipeline default, which its command line never changes).
//
// Exit status: 0 on success, 1 on a parse or reconstruction error (the reference returns
// EXIT_FAILURE for both).
#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/mbir_gb300.h"

#ifndef MBIR_CLI_BF
#define MBIR_CLI_BF 0
#endif

namespace {

const char* kProgram = MBIR_CLI_BF ? "BFReconstruction" : "HAADFReconstruction";

struct Flag {
  const char* name;   // long name (without --)
  const char* alias;  // one-letter short name or ""
  bool has_value;
  bool required;
  const char* def;    // default value ("" for none)
  const char* help;
};

// the reference flag sets, in its order
const Flag kHaadfFlags[] = {
    {"sinofile", "s", true, true, "", "The Sinogram File"},
    {"brightfield", "", true, false, "", "Acquired Bright Field tilt series"},
    {"outputfile", "", true, true, "", "The Output File"},
    {"subvolume", "", true, false, "", "SubVolume to Reconstruct in the form xmin,ymin,zmin,xmax,ymax,zmax"},
    {"thickness", "", true, true, "0", "Thickness of sample in nm"},
    {"tilt_selection", "", true, false, "0", "Which Tilt Values to use from file (0: a, 1: b)"},
    {"diffuseness", "", true, false, "0.2", "Diffuseness Parameter (Markov Random Field Parameter)"},
    {"final_resolution", "", true, false, "1", "The final resolution multiple for the reconstruction"},
    {"sigma_x", "", true, true, "1.0", "Sigma X Value"},
    {"stop_threshold", "", true, false, "0.005", "Stopping Threshold for inner loop"},
    {"num_resolutions", "", true, false, "3", "The number of resolutions to use"},
    {"target_gain", "", true, true, "1", "Normalizing value for unscattered electrons"},
    {"interpolate_initial_recon", "", false, false, "", "Interpolate Initial Reconstruction Value"},
    {"outer_iterations", "", true, false, "30", "Outer Iterations to use"},
    {"inner_iterations", "", true, false, "10", "Number of Inner Iterations"},
    {"default_offset", "", true, false, "0", "Default offset for all Tilts"},
    {"use_default_offset", "", false, false, "", "Use the Default Offset Value"},
    {"default_variance", "", true, false, "1", "Default variance for all Tilts"},
    {"default_recon_value", "", true, false, "0", "Default initial value of reconstruction"},
    {"extend_object", "", false, false, "", "To extend the object or not"},
    {"delete_tmp_files", "", false, false, "", "Delete all the Temp files that are created"},
    {"initial_recon_file", "i", true, false, "", "Initial Reconstruction to initialize algorithm"},
    {"exclude_views", "", true, false, "", "Comma separated list of tilts to exclude by index"},
};
const Flag kBfFlags[] = {
    {"sinofile", "s", true, true, "", "The Sinogram File"},
    {"outputfile", "", true, true, "", "The Output File"},
    {"subvolume", "", true, true, "", "SubVolume to Reconstruct in the form xmin,ymin,zmin,xmax,ymax,zmax"},
    {"thickness", "", true, true, "0", "Thickness of sample in nm"},
    {"tilt_selection", "", true, false, "0", "Which Tilt Values to use from file (0: a, 1: b)"},
    {"diffuseness", "", true, false, "0.2", "Diffuseness Parameter (Markov Random Field Parameter)"},
    {"final_resolution", "", true, false, "1", "The final resolution multiple for the reconstruction"},
    {"sigma_x", "", true, true, "1.0", "Sigma X Value"},
    {"stop_threshold", "", true, false, ".001", "Stopping Threshold for inner loop"},
    {"num_resolutions", "", true, false, "3", "The number of resolutions to use"},
    {"target_gain", "", true, false, "1", "Target Gain for unscattered electrons"},
    {"bragg_T", "", true, false, "3", "Value of Bragg threshold T"},
    {"bragg_delta", "", true, false, "0.5", "value of delta in the bragg rejector"},
    {"bf_offset", "", true, false, "0", "value of offset in the BF data"},
    {"interpolate_initial_recon", "", false, false, "", "Interpolate Initial Reconstruction Value"},
    {"outer_iterations", "", true, false, "600", "Outer Iterations to use"},
    {"inner_iterations", "", true, false, "100", "Number of Inner Iterations"},
    {"default_dosage", "", true, true, "0", "Default dosage for all Tilts"},
    {"use_default_dosage", "", false, false, "", "Use the Default dosage Value"},
    {"default_variance", "", true, false, "1", "Default variance for all Tilts"},
    {"default_recon_value", "", true, false, "0", "Default initial value of reconstruction"},
    {"extend_object", "", false, false, "", "To extend the object or not (the pipeline always does)"},
    {"delete_tmp_files", "", false, false, "", "Delete all the Temp files that are created"},
    {"initial_recon_file", "i", true, false, "", "Initial Reconstruction to initialize algorithm"},
    {"exclude_views", "", true, false, "", "Comma separated list of tilts to exclude by index"},
};

template <size_t N>
constexpr size_t count_of(const Flag (&)[N]) { return N; }

const Flag* flags() { return MBIR_CLI_BF ? kBfFlags : kHaadfFlags; }
size_t n_flags() { return MBIR_CLI_BF ? count_of(kBfFlags) : count_of(kHaadfFlags); }

void usage() {
  std::printf("USAGE: %s [options]\n", kProgram);
  for (size_t i = 0; i < n_flags(); ++i) {
    const Flag& f = flags()[i];
    std::printf("   %s%s%s--%s%s\n        %s%s%s\n", f.required ? "" : "[", f.alias[0] ? "-" : "",
                f.alias[0] ? (std::string(f.alias) + ", ").c_str() : "", f.name,
                f.has_value ? " <value>" : "", f.help, f.def[0] ? " (default " : "",
                f.def[0] ? (std::string(f.def) + ")" + (f.required ? "" : "]")).c_str()
                         : (f.required ? "" : "]"));
  }
}

const Flag* find_flag(const std::string& arg) {
  for (size_t i = 0; i < n_flags(); ++i) {
    const Flag& f = flags()[i];
    if (arg == std::string("--") + f.name || (f.alias[0] && arg == std::string("-") + f.alias))
      return &f;
  }
  return nullptr;
}

// TCLAP-style parsing: "--name value", "-a value", "--switch"; returns false on an error
bool parse(int argc, char** argv, std::map<std::string, std::string>& out, std::string& err) {
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "-h" || a == "--help") {
      out["help"] = "1";
      return true;
    }
    const Flag* f = find_flag(a);
    if (!f) {
      err = "Argument: " + a + "\n             Couldn't find match for argument";
      return false;
    }
    if (f->has_value) {
      if (i + 1 >= argc) {
        err = "Argument: " + a + "\n             Missing a value for this argument!";
        return false;
      }
      out[f->name] = argv[++i];
    } else {
      out[f->name] = "1";
    }
  }
  for (size_t i = 0; i < n_flags(); ++i) {
    const Flag& f = flags()[i];
    if (f.required && !out.count(f.name)) {
      err = std::string("Required argument missing: ") + f.name;
      return false;
    }
    if (!out.count(f.name) && f.has_value && f.def[0]) out[f.name] = f.def;
  }
  return true;
}

bool parse_ints(const std::string& s, std::vector<int>& v) {
  v.clear();
  size_t p = 0;
  while (p < s.size()) {
    char* end = nullptr;
    const long x = std::strtol(s.c_str() + p, &end, 10);
    if (end == s.c_str() + p) return false;
    v.push_back(static_cast<int>(x));
    p = static_cast<size_t>(end - s.c_str());
    if (p < s.size()) {
      if (s[p] != ',') return false;
      ++p;
    }
  }
  return true;
}

std::string parent_path(const std::string& f) {
  const size_t k = f.find_last_of('/');
  return k == std::string::npos ? "." : (k == 0 ? "/" : f.substr(0, k));
}
std::string stem(const std::string& f) {
  const size_t k = f.find_last_of('/');
  std::string b = k == std::string::npos ? f : f.substr(k + 1);
  const size_t d = b.find_last_of('.');
  return d == std::string::npos ? b : b.substr(0, d);
}
bool make_dirs(const std::string& d) {
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

// --initial_recon_file: doubles in y-x-z order (InitialReconstructionBinReader.cpp:101-155),
// returned as [z][x][y] floats of the given size
bool read_object_bin(const std::string& path, int n_z, int n_x, int n_y, std::vector<double>& out) {
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

double num(const std::map<std::string, std::string>& a, const char* k) {
  return std::strtod(a.at(k).c_str(), nullptr);
}
int inum(const std::map<std::string, std::string>& a, const char* k) {
  return static_cast<int>(std::strtol(a.at(k).c_str(), nullptr, 10));
}

}  // namespace

int main(int argc, char** argv) {
  std::printf("Starting MBIR Reconstruction Version %s\n", mbir_version());
  std::map<std::string, std::string> a;
  std::string err;
  if (argc < 2 || !parse(argc, argv, a, err)) {
    if (!err.empty()) std::printf("PARSE ERROR: %s\n\n", err.c_str());
    usage();
    std::printf("Error Parsing the arguments.\n");
    return EXIT_FAILURE;
  }
  if (a.count("help")) {
    usage();
    return EXIT_SUCCESS;
  }
  // HAADF with a bright-field tilt series (--brightfield): read at every level with that
  // level's sinogram subvolume (HAADF_MultiResolutionReconstruction.cpp:189-203, :370-422)
  const std::string bright_field =
      (!MBIR_CLI_BF && a.count("brightfield")) ? a["brightfield"] : std::string();

  mbir_params p;
  mbir_params_default(&p, MBIR_CLI_BF ? MBIR_MODALITY_BF : MBIR_MODALITY_HAADF);
  p.float_params = 1;
  p.sample_thickness = num(a, "thickness");
  p.tilt_selection = inum(a, "tilt_selection");
  p.diffuseness = num(a, "diffuseness");
  p.final_resolution = inum(a, "final_resolution");
  p.sigma_x = num(a, "sigma_x");
  p.stop_threshold = num(a, "stop_threshold");
  p.num_resolutions = inum(a, "num_resolutions");
  p.target_gain = num(a, "target_gain");
  p.outer_iterations = inum(a, "outer_iterations");
  p.inner_iterations = inum(a, "inner_iterations");
  p.default_variance = num(a, "default_variance");
  p.default_recon_value = num(a, "default_recon_value");
  if (MBIR_CLI_BF) {
    p.bragg_threshold = num(a, "bragg_T");
    p.bragg_delta = num(a, "bragg_delta");
    p.bf_offset = num(a, "bf_offset");
    p.default_dosage = num(a, "default_dosage");
    p.use_default_offset = a.count("use_default_dosage") ? 1 : 0;
    p.extend_object = 1;
  } else {
    p.default_offset = num(a, "default_offset");
    p.use_default_offset = a.count("use_default_offset") ? 1 : 0;
    p.extend_object = a.count("extend_object") ? 1 : 0;
  }
  // the reference always hands the engine a subvolume (six zeros when the flag is absent)
  p.use_subvolume = 1;
  if (a.count("subvolume")) {
    std::vector<int> sv;
    if (!parse_ints(a["subvolume"], sv) || sv.size() != 6) {
      std::printf("Error Parsing the Subvolume Dimensions. They should be entered as --subvolume "
                  "64,128,256,80,150,280\nError Parsing the arguments.\n");
      return EXIT_FAILURE;
    }
    for (int i = 0; i < 6; ++i) p.subvolume[i] = sv[i];
  }
  if (a.count("exclude_views")) {
    std::vector<int> ev;
    if (!parse_ints(a["exclude_views"], ev) || ev.size() > 256) {
      std::printf("Error Parsing the Tilt Mask Values. They should be entered as 4,7,12,34,67\n"
                  "Error Parsing the arguments.\n");
      return EXIT_FAILURE;
    }
    p.n_excluded_views = static_cast<int32_t>(ev.size());
    for (size_t i = 0; i < ev.size(); ++i) p.excluded_views[i] = ev[i];
  }
  const std::string sino = a["sinofile"], output = a["outputfile"];
  const std::string out_dir = parent_path(output);
  if (!make_dirs(out_dir)) {
    std::printf("Error creating the output directory '%s'\n   Exiting Now.\n", out_dir.c_str());
    return EXIT_FAILURE;
  }
  const int levels = p.num_resolutions > 0 ? p.num_resolutions : 1;
  const int interp = (1 << (levels - 1)) * std::max(1, p.final_resolution);
  // p = diffuseness + 1 in float, as the pipeline computes it
  const double pq = static_cast<double>(static_cast<float>(p.diffuseness) + 1.0f);
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<double> prev;
  int prev_dims[3] = {0, 0, 0};
  std::vector<double> g, o, v;
  std::vector<std::string> temp_files;
  for (int i = 0; i < levels; ++i) {
    mbir_params q = p;
    q.level = i;
    q.qggmrf_q = pq;
    q.sigma_x = std::pow(2.0, (levels - 1 - i) * (1 - 3 / pq)) *
                static_cast<double>(static_cast<float>(p.sigma_x));
    if (i > 0) {
      q.inner_iterations = 1;
      // later levels take the nuisance and the volume from the level before
      q.default_recon_value = 0.0;
      q.default_variance = 1.0;
      q.use_default_offset = 0;
      q.default_offset = 0.0;
    }
    if (i >= 2) q.stop_threshold = static_cast<float>(p.stop_threshold) * 2.0f;
    q.interpolate_initial_recon = i == 0 ? (a.count("interpolate_initial_recon") ? 1 : 0) : 1;
    const std::string level_dir = out_dir + "/" + std::to_string(interp >> i) + "x";
    if (!make_dirs(level_dir)) {
      std::printf("Could not create path: %s\n", level_dir.c_str());
      return EXIT_FAILURE;
    }
    mbir_engine* e = mbir_create(&q);
    if (!e) {
      std::printf("Error Reconstructing the Data\n");
      return EXIT_FAILURE;
    }
    int rc = mbir_load_sinogram_mrc(e, sino.c_str());
    if (rc == MBIR_OK && !bright_field.empty()) rc = mbir_load_bright_field_mrc(e, bright_field.c_str());
    int32_t d[6] = {0, 0, 0, 0, 0, 0};
    if (rc == MBIR_OK) rc = mbir_get_dims(e, d);
    if (rc == MBIR_OK && i == 0 && a.count("initial_recon_file") &&
        !a["initial_recon_file"].empty()) {
      const int f = q.interpolate_initial_recon ? 2 : 1;
      std::vector<double> init;
      if (!read_object_bin(a["initial_recon_file"], d[0] / f, d[1] / f, d[2] / f, init)) {
        std::printf("Error opening Input file '%s'\n", a["initial_recon_file"].c_str());
        mbir_destroy(e);
        return EXIT_FAILURE;
      }
      rc = mbir_set_initial_volume_f64(e, init.data(), static_cast<int64_t>(init.size()));
    }
    if (rc == MBIR_OK && i > 0) {
      rc = mbir_set_initial_volume_f64(e, prev.data(), static_cast<int64_t>(prev.size()));
      if (rc == MBIR_OK) rc = mbir_set_initial_nuisance(e, g.data(), o.data(), v.data());
    }
    std::printf("%dx: reconstructing %d x %d x %d voxels (z, x, y) from %d views\n", interp >> i,
                d[0], d[1], d[2], d[3]);
    // the HAADF program's intermediate images, <outer>_<inner>_ReconstructedVolume.rec
    if (rc == MBIR_OK && !MBIR_CLI_BF) rc = mbir_set_intermediate_dir(e, level_dir.c_str());
    if (rc == MBIR_OK) rc = mbir_run(e);
    if (rc == MBIR_OK) {
      const bool last = i == levels - 1;
      const std::string vtk = out_dir + "/" + stem(output) + ".vtk";
      const std::string am = out_dir + "/" + stem(output) + ".am";
      rc = last ? mbir_write_outputs_ex(e, level_dir.c_str(), output.c_str(), vtk.c_str(),
                                        am.c_str())
                : mbir_write_outputs(e, level_dir.c_str(), nullptr);
      for (const char* n : {"ReconstructedObject.bin", "FinalGainParameters.bin",
                            "FinalOffsetParameters.bin", "FinalVariances.bin",
                            "ReconstructedSinogram.bin"})
        temp_files.push_back(level_dir + "/" + n);
      for (int o = 0; o < q.outer_iterations; ++o)
        for (int k = 0; k < std::max(1, q.inner_iterations); ++k) {
          const std::string rec = level_dir + "/" + std::to_string(o) + "_" + std::to_string(k) +
                                  "_ReconstructedVolume.rec";
          if (FILE* f = std::fopen(rec.c_str(), "rb")) {
            std::fclose(f);
            temp_files.push_back(rec);
          }
        }
    }
    if (rc == MBIR_OK) {
      prev.assign(static_cast<size_t>(d[0]) * d[1] * d[2], 0.0);
      g.assign(d[3], 0.0);
      o.assign(d[3], 0.0);
      v.assign(d[3], 0.0);
      rc = mbir_get_volume_f64(e, prev.data(), static_cast<int64_t>(prev.size()));
      if (rc == MBIR_OK) rc = mbir_get_nuisance(e, g.data(), o.data(), v.data());
      prev_dims[0] = d[0];
      prev_dims[1] = d[1];
      prev_dims[2] = d[2];
    }
    if (rc != MBIR_OK) {
      std::printf("%s\nError Reconstructing the Data\n", mbir_last_error(e));
      mbir_destroy(e);
      return EXIT_FAILURE;
    }
    mbir_status st;
    mbir_status_get(e, &st);
    std::printf("%dx: %d ICD calls, %lld voxel updates, ICD device time %.1f ms\n", interp >> i,
                st.sweeps_done, static_cast<long long>(st.voxels_updated), st.icd_ms_total);
    mbir_destroy(e);
  }
  if (a.count("delete_tmp_files"))
    for (const std::string& f : temp_files) std::remove(f.c_str());
  const double s =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("Final Dimensions of Object:\n  Nx = %d\n  Ny = %d\n  Nz = %d\n", prev_dims[1],
              prev_dims[2], prev_dims[0]);
  std::printf("Total Running Time: %.3f s\nCompleted MBIR Reconstruction Run\n", s);
  return EXIT_SUCCESS;
}
