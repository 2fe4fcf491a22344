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

}  // namespace mbir
