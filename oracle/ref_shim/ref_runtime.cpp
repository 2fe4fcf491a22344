/*
 * ref_runtime.cpp -- run-time stand-ins linked into the reference built from its own sources.
 *
 * TEST INFRASTRUCTURE ONLY: this file is part of the recipe that compiles OpenMBIR-TEM's
 * reconstruction path (Code/MBIRLib, the POSIX part of Code/MXA and the two command-line
 * programs) into oracle/_ref, where it serves as the parity pin of the CPU restatement.  The
 * product never links it.
 *
 * 1. Clock seed.  The reference seeds every visit-order generator from the wall clock
 *    (HAADF_ReconstructionEngine_UpdateVoxels.cpp:161-162, VoxelUpdateList.cpp:171-172,
 *    BFReconstructionEngine_Extra.cpp:1082,1189), so two runs never agree.  EIMTime.c is
 *    compiled with its clock function renamed to ref_clock_ms; EIMTOMO_getMilliSeconds here
 *    returns MBIR_REF_FIXED_MS when that variable is set (every generator then starts from the
 *    same 32-bit seed, and the phase timers print zero) and the real clock otherwise.
 * 2. Zeroed heap.  The engines leave some AdvancedParameters fields unset
 *    (HAADF_ReconstructionEngine.cpp:244-259 never sets NOISE_ESTIMATION, which
 *    HAADF_ForwardModel.cpp:62,81 reads).  Every operator new here returns zeroed memory, so
 *    such fields read 0 on every run.
 */
#include <cstdlib>
#include <cstring>
#include <new>

extern "C" unsigned long long int ref_clock_ms(void);

extern "C" unsigned long long int EIMTOMO_getMilliSeconds(void) {
  static const char* fixed = std::getenv("MBIR_REF_FIXED_MS");
  if (fixed && *fixed) return std::strtoull(fixed, nullptr, 10);
  return ref_clock_ms();
}

static void* zeroed_alloc(std::size_t n) {
  void* p = std::calloc(n ? n : 1, 1);
  if (!p) throw std::bad_alloc();
  return p;
}

void* operator new(std::size_t n) { return zeroed_alloc(n); }
void* operator new[](std::size_t n) { return zeroed_alloc(n); }
void* operator new(std::size_t n, const std::nothrow_t&) noexcept { return std::calloc(n ? n : 1, 1); }
void* operator new[](std::size_t n, const std::nothrow_t&) noexcept { return std::calloc(n ? n : 1, 1); }
void operator delete(void* p) noexcept { std::free(p); }
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete(void* p, std::size_t) noexcept { std::free(p); }
void operator delete[](void* p, std::size_t) noexcept { std::free(p); }
