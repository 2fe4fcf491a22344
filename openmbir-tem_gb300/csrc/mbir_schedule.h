// mbir_schedule.h -- level schedule of a sparse ICD call (see mbir_schedule.cpp).
#pragma once
#include <cstdint>
#include <vector>

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
};

// Fills lines (the call's lines level by level) and lofs (level offsets, size levels+1);
// returns the number of levels, or -1 on invalid input.
int level_schedule(const LevelScheduleIn& in, LevelScheduleWork& w, std::vector<int32_t>& lines,
                   std::vector<int32_t>& lofs);

// First bin and nonzero mask per (line, view) from the FP32 A-column table.
void acol_bins(const float* table, int n_lines, int n_theta, int nb, int16_t* lo, uint16_t* mask);

}  // namespace mbir
