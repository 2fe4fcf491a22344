// ref_sigmax_main.cpp -- runs the reference's SigmaXEstimation filter (GenericFilters/
// SigmaXEstimation.cpp) from the command line, the way its GUIs drive it
// (Applications/HAADFGui/HAADFGui.cpp:1784-1803).  TEST INFRASTRUCTURE ONLY: linked by
// oracle/build_ref.py against the reference built from its own sources, to pin the library's
// mbir_estimate_sigma_x.
//
// usage: SigmaXEstimate file.mrc thickness target_gain use_bf(0/1) bf_offset x0 x1 y0 y1 tilt...
// prints the estimate with 17 significant digits.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "MBIRLib/GenericFilters/SigmaXEstimation.h"

int main(int argc, char** argv) {
  if (argc < 10) {
    std::fprintf(stderr, "usage: %s file.mrc thickness gain use_bf bf_offset x0 x1 y0 y1 tilt...\n",
                 argv[0]);
    return 2;
  }
  SigmaXEstimation::Pointer e = SigmaXEstimation::New();
  e->setInputFile(argv[1]);
  e->setSampleThickness(std::strtod(argv[2], nullptr));
  e->setTargetGain(std::strtod(argv[3], nullptr));
  e->setUseBFOffset(std::atoi(argv[4]) != 0);
  e->setBfOffset(std::strtod(argv[5], nullptr));
  e->setDefaultOffset(0.0);
  e->setXDims(std::atoi(argv[6]), std::atoi(argv[7]));
  e->setYDims(std::atoi(argv[8]), std::atoi(argv[9]));
  std::vector<float> tilts;
  for (int i = 10; i < argc; ++i) tilts.push_back(static_cast<float>(std::strtod(argv[i], nullptr)));
  e->setTiltAngles(tilts);
  e->execute();
  if (e->getErrorCondition() < 0) return 1;
  std::printf("%.17g\n", e->getSigmaXEstimate());
  return 0;
}
