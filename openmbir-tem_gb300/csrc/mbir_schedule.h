// mbir_schedule.h -- level schedule of a sparse ICD call (see mbir_schedule.cpp).
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

#if defined(__CUDACC__)
#define MBIR_HD __host__ __device__
#else
#define MBIR_HD
#endif

namespace mbir {

struct LevelScheduleIn {
  int n_z, n_x, n_theta, n_r;
  int nb;                  // footprint bins per view
  int stride;              // conflict-free class stride of the row walk
  const int32_t* rows;     // [n_z] row order of the sweep
  const uint8_t* lineok;   // [n_z*n_x] non-empty A-column
  const uint8_t* active;   // [n_z*n_x] lines of the call (nullptr: all)
  const int16_t* lo;       // [n_z*n_x][n_theta] first footprint bin
  const uint16_t* mask;    // [n_z*n_x][n_theta] bit b: bin lo+b has a nonzero A entry
};

struct LevelScheduleWork {
  std::vector<int32_t> bin_level, line_level, order, level, pos;
  std::vector<uint64_t> bin_used, line_used;  // colour sets (colour_schedule)
  std::vector<int32_t> class_size;
};

// Fills lines (the call's lines level by level) and lofs (level offsets, size levels+1);
// returns the number of levels, or -1 on invalid input.
int level_schedule(const LevelScheduleIn& in, LevelScheduleWork& w, std::vector<int32_t>& lines,
                   std::vector<int32_t>& lofs);

// Greedy colouring of the call's conflict graph (two lines conflict when they share a touched
// bin at some view or are 3x3 (z, x) neighbours): lines visited z-major (z, then x ascending),
// each takes the smallest colour that no conflicting earlier line holds and that has fewer than
// class_cap lines (0: no cap; the kernel runs class_cap voxels at once).  Fills lines (colour by
// colour, z-major within a colour) and lofs (colour offsets); returns the number of colours, -1
// on invalid input, -2 when more than max_colours would be needed.
int colour_schedule(const LevelScheduleIn& in, int max_colours, int class_cap,
                    LevelScheduleWork& w, std::vector<int32_t>& lines,
                    std::vector<int32_t>& lofs);

// First bin and nonzero mask per (line, view) from the FP32 A-column table.
void acol_bins(const float* table, int n_lines, int n_theta, int nb, int16_t* lo, uint16_t* mask);

// One A-column table entry (e[0]: the first bin's int32 bits, e[1..nb]: the values): bit b of
// the mask when value b is positive, and the first bin (0 when no value is).  The host bins
// above and the device colouring's packed bins (packed_footprint) both come from these.
inline MBIR_HD unsigned footprint_mask(const float* e, int nb) {
  unsigned bits = 0;
  for (int b = 0; b < nb; ++b)
    if (e[1 + b] > 0.f) bits |= 1u << b;
  return bits;
}
inline MBIR_HD int16_t footprint_lo(const float* e, unsigned bits) {
  int32_t j;
  memcpy(&j, e, sizeof(j));
  return static_cast<int16_t>(bits ? j : 0);
}
// (first bin << 16) | mask, the first bin as its 16-bit pattern
inline MBIR_HD int32_t packed_footprint(const float* e, int nb) {
  const unsigned bits = footprint_mask(e, nb);
  return static_cast<int32_t>(
      (static_cast<uint32_t>(static_cast<uint16_t>(footprint_lo(e, bits))) << 16) | bits);
}

}  // namespace mbir
