// mbir_schedule.cpp -- level schedule of a sparse ICD call (host, C++17).
//
// A bright-field NHICD call updates 1/20 of the voxel lines (BFReconstructionEngine.cpp:610-646,
// BFReconstructionEngine_Extra.cpp:576-628).  Walked row by row, a row of a slice holds ~25 of
// the call's voxels, spread over the row's conflict-free classes, so most barrier steps of the
// row walk carry only a handful of voxels.  Across rows, most pairs of listed voxels touch no
// common detector bin, so many of them can run together.  This file groups the call's lines
// into levels:
//
//   level(line) = 1 + max( level of every earlier line of the visit order that shares a
//                          detector bin with it at some view,
//                          level of every earlier line in its 3x3 (z, x) neighbourhood )
//
// Two lines in one level are then independent: they touch disjoint error-sinogram entries
// (and, for bright field, selector bytes), neither reads the other's voxel (prior neighbours
// and the zero-skipping test read the 3x3x3 neighbourhood, whose in-slice part is the 3x3
// (z, x) window), and they are not reordered against any line they depend on.  Independent
// updates commute exactly, so running the levels in turn gives the bits of the visit order.
// The voxel lines' footprints do not depend on y, so one schedule serves every voxel slice.
//
// The visit order is the row walk's: rows in the sweep's row order, within a row the classes
// x = k (mod stride) for k = 0..stride-1, x ascending in a class.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mbir_schedule.h"

namespace mbir {

int level_schedule(const LevelScheduleIn& in, LevelScheduleWork& w, std::vector<int32_t>& lines,
                   std::vector<int32_t>& lofs) {
  const int nz = in.n_z, nx = in.n_x, nt = in.n_theta, nr = in.n_r, nb = in.nb, S = in.stride;
  if (nz <= 0 || nx <= 0 || nt <= 0 || nr <= 0 || nb <= 0 || nb > 16 || S <= 0) return -1;
  w.bin_level.assign(static_cast<size_t>(nt) * nr, 0);
  w.line_level.assign(static_cast<size_t>(nz) * nx, 0);
  w.order.clear();
  w.level.clear();
  int max_level = 0;
  for (int rr = 0; rr < nz; ++rr) {
    const int z = in.rows[rr];
    if (z < 0 || z >= nz) return -1;
    for (int k = 0; k < S && k < nx; ++k) {
      for (int x = k; x < nx; x += S) {
        const size_t l = static_cast<size_t>(z) * nx + x;
        if (!in.lineok[l] || (in.active != nullptr && !in.active[l])) continue;
        const int16_t* lo = in.lo + l * nt;
        const uint16_t* mk = in.mask + l * nt;
        int m = 0;
        for (int v = 0; v < nt; ++v) {
          const unsigned bits = mk[v];
          if (!bits) continue;
          const int32_t* row = w.bin_level.data() + static_cast<size_t>(v) * nr + lo[v];
          for (int b = 0; b < nb; ++b)
            if ((bits >> b) & 1u) m = std::max(m, row[b]);
        }
        for (int dz = -1; dz <= 1; ++dz) {
          const int zz = z + dz;
          if (zz < 0 || zz >= nz) continue;
          for (int dx = -1; dx <= 1; ++dx) {
            const int xx = x + dx;
            if (xx < 0 || xx >= nx) continue;
            m = std::max(m, w.line_level[static_cast<size_t>(zz) * nx + xx]);
          }
        }
        const int L = m + 1;
        for (int v = 0; v < nt; ++v) {
          const unsigned bits = mk[v];
          if (!bits) continue;
          int32_t* row = w.bin_level.data() + static_cast<size_t>(v) * nr + lo[v];
          for (int b = 0; b < nb; ++b)
            if ((bits >> b) & 1u) row[b] = L;
        }
        w.line_level[l] = L;
        w.order.push_back(static_cast<int32_t>(l));
        w.level.push_back(L);
        max_level = std::max(max_level, L);
      }
    }
  }
  // counting sort by level (stable: visit order within a level)
  lofs.assign(static_cast<size_t>(max_level) + 1, 0);
  for (int L : w.level) lofs[L]++;
  for (int L = 1; L <= max_level; ++L) lofs[L] += lofs[L - 1];
  lines.assign(w.order.size(), 0);
  std::vector<int32_t>& pos = w.pos;
  pos.assign(lofs.begin(), lofs.end() - 1);
  for (size_t i = 0; i < w.order.size(); ++i) lines[pos[w.level[i] - 1]++] = w.order[i];
  return max_level;
}

// Colouring: the same independence argument as the levels above, with the visit order chosen
// for few barrier steps instead of given.  Colour classes are independent sets of the conflict
// graph; running them in colour order is the sequential ICD of the order "all lines of colour
// 0, then colour 1, ...", whose result does not depend on the order inside a class.  A 1/20 NHICD
// call of a 128 x 512 plane with 61 views needs about 0.45 times as many colours as the row
// walk needs levels.
// Colour sets are bit planes: word k of bin (v, j) at bin_used[k][v][j] and of line l at
// line_used[k][l], so the few words in use (colours < 64 * used words) stay cache-resident.
// zero the colour-set words (planes 0..words-1, the planes in use) of every line coloured so
// far (w.order) and of its bins
static void colour_clear(const LevelScheduleIn& in, int words, LevelScheduleWork& w) {
  const int nt = in.n_theta, nr = in.n_r, nb = in.nb;
  const size_t bplane = static_cast<size_t>(nt) * nr;
  const size_t lplane = static_cast<size_t>(in.n_z) * in.n_x;
  for (int32_t l : w.order) {
    const int16_t* lo = in.lo + static_cast<size_t>(l) * nt;
    const uint16_t* mk = in.mask + static_cast<size_t>(l) * nt;
    for (int v = 0; v < nt; ++v) {
      const unsigned bits = mk[v];
      if (!bits) continue;
      const size_t j0 = static_cast<size_t>(v) * nr + lo[v];
      for (int k = 0; k < words; ++k)
        for (int b = 0; b < nb; ++b)
          if ((bits >> b) & 1u) w.bin_used[k * bplane + j0 + b] = 0;
    }
    for (int k = 0; k < words; ++k) w.line_used[k * lplane + l] = 0;
  }
}

// Colouring: the same independence argument as the levels above, with the visit order chosen
// for few barrier steps instead of given.  Colour classes are independent sets of the conflict
// graph; running them in colour order is the sequential ICD of the order "all lines of colour
// 0, then colour 1, ...", whose result does not depend on the order inside a class.  A 1/20 NHICD
// call of a 128 x 512 plane with 61 views needs about 0.45 times as many colours as the row
// walk needs levels.
int colour_schedule(const LevelScheduleIn& in, int max_colours, int class_cap,
                    LevelScheduleWork& w, std::vector<int32_t>& lines,
                    std::vector<int32_t>& lofs) {
  const int nz = in.n_z, nx = in.n_x, nt = in.n_theta, nr = in.n_r, nb = in.nb;
  if (nz <= 0 || nx <= 0 || nt <= 0 || nr <= 0 || nb <= 0 || nb > 16 || max_colours <= 0)
    return -1;
  const int words = (max_colours + 63) / 64;
  const size_t bplane = static_cast<size_t>(nt) * nr, lplane = static_cast<size_t>(nz) * nx;
  // the colour-set planes stay allocated between calls; a call clears what it set
  if (w.bin_used.size() != bplane * words) w.bin_used.assign(bplane * words, 0);
  if (w.line_used.size() != lplane * words) w.line_used.assign(lplane * words, 0);
  w.order.clear();
  w.level.clear();
  int n_colours = 0;
  std::vector<uint64_t> forbid(words), full(words, 0);
  w.class_size.assign(static_cast<size_t>(words) * 64, 0);
  for (int z = 0; z < nz; ++z) {
    for (int x = 0; x < nx; ++x) {
      const size_t l = static_cast<size_t>(z) * nx + x;
      if (!in.lineok[l] || (in.active != nullptr && !in.active[l])) continue;
      const int16_t* lo = in.lo + l * nt;
      const uint16_t* mk = in.mask + l * nt;
      const int used_words = std::min(n_colours / 64 + 1, words);
      std::copy(full.begin(), full.end(), forbid.begin());
      for (int k = 0; k < used_words; ++k) {
        const uint64_t* plane = w.bin_used.data() + k * bplane;
        uint64_t f = forbid[k];
        for (int v = 0; v < nt; ++v) {
          const unsigned bits = mk[v];
          if (!bits) continue;
          const uint64_t* row = plane + static_cast<size_t>(v) * nr + lo[v];
          for (int b = 0; b < nb; ++b)
            if ((bits >> b) & 1u) f |= row[b];
        }
        const uint64_t* lp = w.line_used.data() + k * lplane;
        for (int dz = -1; dz <= 1; ++dz) {
          const int zz = z + dz;
          if (zz < 0 || zz >= nz) continue;
          for (int dx = -1; dx <= 1; ++dx) {
            const int xx = x + dx;
            if (xx >= 0 && xx < nx) f |= lp[static_cast<size_t>(zz) * nx + xx];
          }
        }
        forbid[k] = f;
      }
      int col = -1;
      for (int k = 0; k < words && col < 0; ++k)
        if (~forbid[k]) {
          const uint64_t free_bits = ~forbid[k];
          int b = 0;
          while (!((free_bits >> b) & 1ull)) ++b;
          col = 64 * k + b;
        }
      if (col < 0 || col >= max_colours) {
        colour_clear(in, std::min(n_colours / 64 + 1, words), w);
        return -2;
      }
      const uint64_t bit = 1ull << (col & 63);
      const int wk = col >> 6;
      uint64_t* plane = w.bin_used.data() + wk * bplane;
      for (int v = 0; v < nt; ++v) {
        const unsigned bits = mk[v];
        if (!bits) continue;
        uint64_t* row = plane + static_cast<size_t>(v) * nr + lo[v];
        for (int b = 0; b < nb; ++b)
          if ((bits >> b) & 1u) row[b] |= bit;
      }
      w.line_used[wk * lplane + l] |= bit;
      if (class_cap > 0 && ++w.class_size[col] >= class_cap) full[wk] |= bit;
      w.order.push_back(static_cast<int32_t>(l));
      w.level.push_back(col + 1);
      if (col + 1 > n_colours) n_colours = col + 1;
    }
  }
  colour_clear(in, std::min((n_colours + 63) / 64, words), w);
  lofs.assign(static_cast<size_t>(n_colours) + 1, 0);
  for (int L : w.level) lofs[L]++;
  for (int L = 1; L <= n_colours; ++L) lofs[L] += lofs[L - 1];
  lines.assign(w.order.size(), 0);
  std::vector<int32_t>& pos = w.pos;
  pos.assign(lofs.begin(), lofs.end() - 1);
  for (size_t i = 0; i < w.order.size(); ++i) lines[pos[w.level[i] - 1]++] = w.order[i];
  return n_colours;
}

// Per-view first bin and nonzero-bin mask of every voxel line from the A-column table
// ([line][view][acol_width(nb) float4]: first bin as int bits, then nb values).
void acol_bins(const float* table, int n_lines, int n_theta, int nb, int16_t* lo,
               uint16_t* mask) {
  const int wf = ((nb + 1 + 3) / 4) * 4;
  static_assert(sizeof(int32_t) == sizeof(float), "int32 and float differ in size");
  for (size_t i = 0; i < static_cast<size_t>(n_lines) * n_theta; ++i) {
    const float* e = table + i * wf;
    const unsigned bits = footprint_mask(e, nb);
    lo[i] = footprint_lo(e, bits);
    mask[i] = static_cast<uint16_t>(bits);
  }
}

}  // namespace mbir
