// mbir_reconstruct.cpp -- the reference's two reconstruction programs, HAADFReconstruction and
// BFReconstruction, over this library's C ABI.
//
// Built twice (MBIR_CLI_BF = 0 / 1) into openmbir-tem_gb300/bin/.  Each program accepts the flag
// set of the reference program of the same name (Code/Applications/HAADFReconstruction/
// HAADFReconstructionArgsParser.cpp:143-211, Code/Applications/BFReconstruction/
// BFReconstructionArgsParser.cpp:145-226) and runs the multi-resolution pipeline through
// mbir_gb300::HAADF_MultiResolutionReconstruction / BFMultiResolutionReconstruction
// (include/mbir_gb300.hpp), the classes that replace the reference's pipeline classes: per level
// the voxel size, sigma_x, iteration and stop-threshold rules of
// HAADF_MultiResolutionReconstruction.cpp:175-485, the previous level's volume replicated 2x2x2
// and its nuisance handed on, each level's files in <output dir>/<factor>x/ and the MRC, .vtk
// and .am volumes from the last level.  The pipeline's messages are printed one per line.  The
// bright-field program always extends the object (the reference's pipeline default, which its
// command line never changes).
//
// Exit status: 0 on success, 1 on a parse or reconstruction error (the reference returns
// EXIT_FAILURE for both).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/mbir_gb300.hpp"

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

#if MBIR_CLI_BF
  mbir_gb300::BFMultiResolutionReconstruction m;
#else
  mbir_gb300::HAADF_MultiResolutionReconstruction m;
#endif
  m.setInputFile(a["sinofile"]);
  m.setOutputFile(a["outputfile"]);
  if (!bright_field.empty()) m.setBrightFieldFile(bright_field);
  if (a.count("initial_recon_file")) m.setInitialReconstructionFile(a["initial_recon_file"]);
  m.setDeleteTempFiles(a.count("delete_tmp_files") > 0);
  m.setSampleThickness(num(a, "thickness"));
  m.setTiltSelection(inum(a, "tilt_selection"));
  m.setMRFShapeParameter(num(a, "diffuseness"));
  m.setFinalResolution(inum(a, "final_resolution"));
  m.setSigmaX(num(a, "sigma_x"));
  m.setStopThreshold(num(a, "stop_threshold"));
  m.setNumberResolutions(inum(a, "num_resolutions"));
  m.setTargetGain(num(a, "target_gain"));
  m.setInterpolateInitialReconstruction(a.count("interpolate_initial_recon") > 0);
  m.setOuterIterations(inum(a, "outer_iterations"));
  m.setInnerIterations(inum(a, "inner_iterations"));
  m.setDefaultVariance(num(a, "default_variance"));
  m.setInitialReconstructionValue(num(a, "default_recon_value"));
#if MBIR_CLI_BF
  m.setBraggThreshold(num(a, "bragg_T"));
  m.setBraggDelta(num(a, "bragg_delta"));
  m.setBfOffset(num(a, "bf_offset"));
  m.setDefaultDosage(num(a, "default_dosage"));
  m.setUseDefaultDosage(a.count("use_default_dosage") > 0);
#else
  m.setDefaultOffsetValue(num(a, "default_offset"));
  m.setUseDefaultOffset(a.count("use_default_offset") > 0);
  m.setExtendObject(a.count("extend_object") > 0);
#endif
  if (a.count("subvolume")) {
    std::vector<int> sv;
    if (!parse_ints(a["subvolume"], sv) || sv.size() != 6) {
      std::printf("Error Parsing the Subvolume Dimensions. They should be entered as --subvolume "
                  "64,128,256,80,150,280\nError Parsing the arguments.\n");
      return EXIT_FAILURE;
    }
    m.setSubvolume(sv);
  }
  if (a.count("exclude_views")) {
    std::vector<int> ev;
    if (!parse_ints(a["exclude_views"], ev) || !m.setViewMasks(ev)) {
      std::printf("Error Parsing the Tilt Mask Values. They should be entered as 4,7,12,34,67\n"
                  "Error Parsing the arguments.\n");
      return EXIT_FAILURE;
    }
  }
  m.setMessageHandler([](const std::string& msg) { std::printf("%s\n", msg.c_str()); });
  const auto t0 = std::chrono::steady_clock::now();
  if (m.execute() != MBIR_OK) return EXIT_FAILURE;
  const double s =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  const int32_t* d = m.getDims();
  std::printf("Final Dimensions of Object:\n  Nx = %d\n  Ny = %d\n  Nz = %d\n", d[1], d[2], d[0]);
  std::printf("Total Running Time: %.3f s\nCompleted MBIR Reconstruction Run\n", s);
  return EXIT_SUCCESS;
}
