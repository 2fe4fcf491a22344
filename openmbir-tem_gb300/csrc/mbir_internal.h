// mbir_internal.h -- structures shared by the host engine and the sm_103a kernels.
//
// HBM layout (FP32 by default; FP64 when the engine runs in double precision):
//   sinogram-shaped arrays (measured y, error e, projection yest): [t][theta][r_pad]
//     -- one detector row t (a y-slice of the tilt series) is one contiguous block of
//        n_theta * n_rp values, so a voxel slice's footprint rows are a single TMA bulk copy;
//   volume x: [y][z][x] -- one voxel slice is contiguous;
//   per-view tables: detector response H [theta][bins+1], (gain, weight) pairs, projection
//     coefficients; per-slice t-response (first row, count, values).
#pragma once
#include <cuda_runtime.h>
#include <vector_types.h>

#include <cstdint>

namespace mbir {

constexpr int kMaxViewsPerLane = 8;   // n_theta <= 256 (parallel sweeps)
// Above this many views the parallel sweeps work on the slices in HBM with 32 lanes x 8 views;
// the reference-order kernels, the reference-exact mode and the batch take at most this many
constexpr int kMaxViewsShaped = 160;

// Voxel-group shape of the FP32 sweep kernels for n_theta views: 0 = 16 lanes x 4 views per
// lane (two voxels per warp), 1 = 32 lanes x 3 views, 2 = 32 lanes x 5 views, 3 = 32 lanes x 8
// views.
inline int lane_shape(int n_theta) {
  return n_theta <= 64 ? 0 : (n_theta <= 96 ? 1 : (n_theta <= kMaxViewsShaped ? 2 : 3));
}
// Explicit shapes of the public parameter: 1 = 16x4, 2 = 32x2, 3 = 32x3, 4 = 32x5, 5 = 32x8
// (slices in HBM); the largest view count each covers
inline int shape_max_views(int shape) {
  return shape == 1 ? 64 : shape == 2 ? 64 : shape == 3 ? 96 : shape == 4 ? 160
                                                                          : shape == 5 ? 256 : 0;
}
// The shape an FP32 sweep launch uses: the explicit one when it covers the views, else the
// default for the view count
inline int resolved_shape(int shape, int n_theta) {
  if (shape < 1 || shape > 5 || n_theta > shape_max_views(shape))
    shape = 1 + (lane_shape(n_theta) == 0 ? 0 : lane_shape(n_theta) + 1);
  return shape;
}
constexpr int kWarps = 16;            // warps per ICD block
constexpr int kMaxTRows = 4;          // t rows a voxel slice may touch
constexpr int kStatSlots = 4;         // sum|dx| (ROI), sum|x| (ROI), zero-skipped, updated

struct DevGeom {
  int n_theta, n_r, n_rp, n_t;
  int n_x, n_y, n_z;
  int bins;            // detector response bins (64)
  double kr;           // delta_r / OffsetR: detector-bin distance -> response-table index
  double half_width;   // delta_xz / delta_r: footprint half width in detector bins
  int roi_x0, roi_x1, roi_z0, roi_z1;  // ROI mask as index ranges [x0,x1] x [z0,z1]
};

// Type-erased table pointers: Real = float or double according to the engine precision.
struct DevTables {
  const void* H;         // Real [n_theta][bins+1], last entry repeats bins-1
  const float2* bx;      // [n_theta] (hi, lo) of delta_xz*cos/delta_r   (FP32 path)
  const double* bxd;     // [n_theta] delta_xz*cos/delta_r               (FP64 path)
  const double* u0;      // [n_theta] detector coordinate (bins) of voxel (0,0)
  const double* bz;      // [n_theta] delta_xz*sin/delta_r
  const void* gw;        // Real2 [n_theta] (gain I_theta, weight 1/alpha_theta)
  const int* t_first;    // [n_y]
  const int* t_count;    // [n_y]
  const void* hval;      // Real [n_y][kMaxTRows]
  const uint8_t* lineok; // [n_z][n_x] 1 when the voxel line's A-column is not empty
};

struct DevFilter {
  double f[27];          // prior weights [dy+1][dz+1][dx+1]
  double mrf_p, mrf_q, mrf_c, mrf_alpha;
  double sig_p, sig_pq;  // sigma^P, sigma^(P-Q)
  double inv_sig_pq;     // 1 / sigma^(P-Q)
};

enum SweepMode : int { kModeICD = 0, kModeProject = 1 };

// Fixed-point scale of the per-line update magnitudes and the ROI sums accumulated with
// integer atomics (integer addition is associative, so the sums do not depend on the order in
// which voxels finish): value = count * 2^-32.
constexpr double kFixScale = 4294967296.0;

// Bright-field extras of a sweep (BFForwardModel / BFUpdateYSlice).  Per-entry arrays share the
// sinogram layout [t][theta][row]; the selector rows are padded to n_sp bytes (a multiple of 16)
// so a slice's selector rows are bulk-copied like its error rows.
struct DevBF {
  const void* w;                // Real [n_t][n_theta][n_rp] measurement weights
  uint8_t* sel;                 // [n_t][n_theta][n_sp] Bragg selector (1 = selected)
  int n_sp;                     // selector row stride (bytes)
  const uint8_t* active;        // [n_z][n_x] lines of this call (nullptr: all lines)
  unsigned long long* mag_fx;   // [n_z][n_x] fixed-point sum |dx| per line (nullptr: off)
  double bragg_t;               // current Bragg threshold T
  double bragg_dt;              // delta * T
};

struct SweepArgs {
  DevGeom g;
  DevTables tab;
  DevFilter flt;
  void* x;               // Real [n_y][n_z][n_x]
  void* e;               // Real [n_t][n_theta][n_rp]  (ICD: error; project: accumulated yest)
  const int* row_order;  // [n_z]
  int stride;            // x stride of a conflict-free class
  int colour;            // y parity of the slices in this launch
  int n_slices;          // slices in this launch
  int mode;              // SweepMode
  int iter_nonzero;      // zero skipping active (not the first sweep)
  int zero_skipping;
  int smem_rows;         // 1: stage the slice in shared memory
  int n_rs;              // shared-memory row stride (values)
  int fp64;              // 1: Real = double
  int bf;                // 1: bright-field data term (DevBF below)
  DevBF bfa;
  int shape;             // FP32 voxel-group shape (1..4), 0: lane_shape(n_theta)
  int y_first;           // slab launch: first slice (its parity is the colour)
  int y_end;             // slab launch: slices y < y_end; 0 = whole-volume launch from `colour`
  double* stats;         // [gridDim.x][kStatSlots]
  int* err;              // device error word
  // Level schedule (FP32; nullptr: walk the rows).  The voxel lines of the call in levels:
  // lines of one level are pairwise independent (no shared detector bin at any view, not prior
  // neighbours) and every line's level is above that of each earlier line of the visit order it
  // conflicts with, so running the levels in turn gives the visit order's result.  Footprints
  // do not depend on y, so one schedule serves every slice.
  const int* sched_lines;  // [lofs[n_levels]] z*n_x + x, level by level
  const int* sched_lofs;   // [n_levels + 1]
  int n_levels;
  const int* sched_count;  // device [2] (lines, levels) written by the colour kernel, or nullptr
                           // (then n_levels holds the level count)
  const float4* acol;      // [n_z*n_x][n_theta][acol_width(NB)] A-column table (FP32)
};

// A-column table entry of one voxel line at one view: the first bin (int bits) and the NB
// footprint values, padded to whole float4s.
constexpr int acol_width(int nb) { return (nb + 1 + 3) / 4; }

// The per-block shared-memory limit (opt-in) of the current device.  Launchers set a kernel's
// dynamic limit attribute to this minus the kernel's static shared memory (dyn_smem_limit)
// rather than to their own size: the attribute belongs to the function, not the launch, and
// host threads launching the same kernel with different sizes would otherwise race (a launch
// above the value another thread just set fails).
inline int smem_optin_limit() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 48 * 1024;
  if (cached[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cached[dev] = v > 0 ? v : 48 * 1024;
  }
  return cached[dev];
}

template <typename F>
inline int dyn_smem_limit(F* func) {
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(func)) != cudaSuccess) return 0;
  return smem_optin_limit() - static_cast<int>(fa.sharedSizeBytes);
}

// Colour schedule of a sparse ICD call on the device (mbir_colour.cu); the same result as the
// host colour_schedule.
struct ColourArgs {
  int n_z, n_x, n_theta, n_r, nb;
  int words;                      // colour-set words per bin and line (2, 4 or 8)
  int max_colours;                // <= 64 * words
  int class_cap;                  // 1..32 lines per colour
  const int32_t* packed;          // [n_z*n_x][n_theta] (first bin << 16) | nonzero-bin mask
  const uint8_t* lineok;          // [n_z*n_x]
  const uint8_t* active;          // [n_z*n_x] lines of the call (nullptr: all)
  const int32_t* vis;             // [n] the call's lines (lineok and active), ascending
  int n;
  unsigned* conf;                 // [n] scratch: conflict words of each block of 32 lines
  unsigned* conf_p1;              // [n] scratch: conflict words against the block before
  unsigned* conf_p2;              // [n] scratch: against the block before that
  unsigned* conf_p3;              // [n] scratch: against the block before that one
  unsigned* conf_p4;              // [n] scratch: against the fourth block back
  int16_t* colour;                // [n_z*n_x] scratch: colour of each of the call's lines
  unsigned long long* bin_used;   // [n_theta][n_r][words] scratch, cleared by the launcher
  unsigned long long* line_used;  // [n_z*n_x][words] scratch, cleared by the launcher
  int32_t* lines;                 // [n_z*n_x] out: lines colour by colour
  int32_t* lofs;                  // [max_colours + 1] out: colour offsets
  int32_t* count;                 // [2] out: lines, colours
  int* err;                       // value 4 is ORed in when max_colours do not suffice, 2 when
                                  // a wait of the multi-CTA form ran out of time
  // multi-CTA form (used when fsets and flags are set and the device launches cooperatively)
  unsigned long long* fsets;      // [ceil(n/31)*31][words] scratch: taken-colour sets per line
  int* flags;                     // [3*ceil(n/31)] scratch: ready, coloured, written per block
  int* abort_flag;                // [1] scratch
  unsigned long long wait_ns;     // limit of each wait on a flag
  int helpers;                    // helper CTAs (0: the one-CTA form)
  int sequential;                 // 1: every block line by line (the parallel form's check)
};
int launch_colour_schedule(const ColourArgs& a, void* stream);
size_t colour_smem_bytes(int n_theta, int words);
bool colour_schedule_fits(int n_theta, int words);  // shared memory of both kernels
// packed[i] = (first bin << 16) | nonzero mask of A-column table entry i (packed_footprint), for
// the n = lines x views entries of the table
int launch_pack_footprints(const float4* table, size_t n, int nb, int32_t* packed, void* stream);

// Batched sweep: per-series sweep arguments and a queue of (series, slice y) items.
struct BatchArgs {
  const SweepArgs* series;   // [n_series] in device memory (colour field unused)
  const int2* items;         // [n_items] (series, y): colour-0 items first, then colour-1
  int n_items;
  int* queue;                // item counter (zeroed before the launch)
  int* done;                 // [n_series] finished colour-0 slices (zeroed before the launch)
  const int* need;           // [n_series] number of colour-0 slices
  unsigned long long wait_ns;  // limit of a colour-1 slice's wait for its colour-0 slices
};

struct RefOrderArgs {
  DevGeom g;
  DevTables tab;
  DevFilter flt;
  void* x;
  void* e;
  const int* lines;      // visit order: z*n_x + x
  int n_lines;
  int iter_nonzero;
  int zero_skipping;
  int fp64;
  int bf;
  DevBF bfa;
  double* stats;         // [kStatSlots]
};

// Reference-exact FP64 mode (mbir_exact.cu): every operation in the reference's order.
struct ExactArgs {
  DevGeom g;
  DevFilter flt;
  double x0, z0, delta_xz, delta_r, R0, RMax, offset_r;
  const double* cosv;    // [n_theta]
  const double* sinv;
  const double* H;       // [n_theta][bins] as the reference builds it
  const double* gain;    // [n_theta]
  const double* weight;  // [n_theta]
  const int* t_first;
  const int* t_count;
  const double* hval;    // [n_y][kMaxTRows]
  const uint8_t* lineok;
  double* x;             // [n_y][n_z][n_x]
  double* e;             // [n_t][n_theta][n_rp]
  const int* lines;
  int n_lines;
  int iter_nonzero, zero_skipping;
  double* stats;         // [kStatSlots]
  // bright field (BFUpdateYSlice / BFForwardModel::computeTheta, updateErrorSinogram)
  int bf;
  const double* bw;      // [n_t][n_theta][n_rp] weights
  uint8_t* bsel;         // [n_t][n_theta][n_sp] selector
  int n_sp;
  double bragg_t, bragg_delta;
  double* mag;           // [n_z][n_x] per-line sum |dx| (reset for each line of the call)
  // HAADF with bright-field data: bright-field count + BF_OFFSET per entry, [n_t][n_theta][n_rp]
  // (nullptr without)
  const double* bfm;
};

// HAADF with bright-field data (mbir_bfassist.cu; the reference-exact forms in mbir_exact.cu).
// Arrays share the [t][theta][r_pad] layout; m = bright-field count + BF_OFFSET.
int launch_bfa_error(const void* y, const void* yest, const void* m, void* e, const double* mu,
                     int n_theta, int n_rp, int n_r, int n_t, int fp64, void* stream);
int launch_bfa_weights(const void* m, const double* wv, void* w, int n_theta, int n_rp, int n_r,
                       int n_t, int fp64, void* stream);
int launch_bfa_sums(int kind, const void* m, const void* e, double* partial, double* out,
                    int n_theta, int n_rp, int n_r, int n_t, int n_chunk, int fp64, void* stream);
int launch_bfa_offset_apply(const void* m, void* e, const double* step, int n_theta, int n_rp,
                            int n_r, int n_t, int fp64, void* stream);
int launch_exact_bfa_error(const ExactArgs& a, const double* y, const double* yest,
                           const double* mu, void* stream);
int launch_exact_bfa_offsets(const ExactArgs& a, double* mu, void* stream);

// Bright-field sinogram-wide passes (mbir_bf.cu).  Arrays share the [t][theta][row] layout.
struct BfSino {
  void* e;               // Real error sinogram
  void* w;               // Real weights
  uint8_t* sel;          // selector, rows of n_sp bytes
  int n_theta, n_r, n_rp, n_sp, n_t;
  int fp64;
};
int launch_layout_from_double(const double* host_layout, void* dev_layout, int n_theta, int n_r,
                              int n_rp, int n_t, int fp64, void* stream);
int launch_bf_offset_sums(const BfSino& b, int exact, double T, double dl, double* partial,
                          int n_chunk, double* out, void* stream);
int launch_bf_offset_apply(const BfSino& b, const double* step, void* stream);
int launch_bf_selector(const BfSino& b, double T, void* stream);
int launch_bf_variance_sums(const BfSino& b, int exact, const double* alpha, double* partial,
                            double* out, void* stream);
int launch_bf_scale_weights(const BfSino& b, double alpha, void* stream);
int launch_bf_cost_sums(const BfSino& b, int exact, double T, double dl, double* partial,
                        double* out, void* stream);
int launch_bf_mag_reset(unsigned long long* fx, const uint8_t* active, int n, void* stream);
int launch_bf_mag_update(const unsigned long long* fx, const uint8_t* active, double* mag, int n,
                         void* stream);
int launch_bf_vsc(const double* mag, double* filt, int n_z, int n_x, void* stream);
int launch_bf_nh_mask(const double* filt, double thr, uint8_t* active, int n, void* stream);
int launch_roi_sum(const DevGeom& g, int exact, int kind, const double* mag, const void* x,
                   int fp64, double* partial, double* out, void* stream);

int launch_exact_icd(const ExactArgs& a, void* stream);
int launch_exact_project(const ExactArgs& a, double* yest, void* stream);
int launch_exact_view_sums(const ExactArgs& a, int kind, const double* y, const double* mu,
                           double* out, void* stream);

// launchers (mbir_kernels.cu); fp64 selects Real = double for the void* arrays
int launch_sweep(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
int launch_ref_order(const RefOrderArgs& a, int nb, void* stream);
// sched: the layout of a scheduled bright-field call (smaller: no response table or row lists)
size_t sweep_smem_bytes(int n_theta, int n_x, int n_rs, int t_rows, int bins, int fp64,
                        int n_sp, bool sched = false);
int launch_sweep_f32_smem(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
int launch_sweep_f32_smem_haadf(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
int launch_sweep_f32_smem_bf(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
int launch_sweep_f32_hbm(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
int launch_sweep_f32_hbm_bf(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
// A-column table [n_z*n_x][n_theta][acol_width(nb)] of the FP32 sweep (level-scheduled calls)
int launch_acol_f32(const DevGeom& g, const DevTables& tab, int nb, float4* out, void* stream);
int launch_sweep_f64(const SweepArgs& a, int nb, size_t smem_bytes, void* stream);
int launch_ref_order_f32(const RefOrderArgs& a, int nb, void* stream);
// persistent batched sweep (FP32, slices staged or in HBM per series); shape = lane_shape of
// the largest n_theta in the batch
// one launch per group = 2 * (voxel-group shape - 1) + bright field; threads: 512 (one CTA per
// SM) or 256 (two CTAs per SM when the shared memory allows)
int launch_batch_sweep(const BatchArgs& b, int nb, int group, int threads, size_t smem_bytes,
                       int grid,
                       void* stream);
int launch_batch_sweep_nb3(const BatchArgs& b, int group, int threads, size_t smem_bytes, int grid,
                           void* stream);
int launch_batch_sweep_nb5(const BatchArgs& b, int group, int threads, size_t smem_bytes, int grid,
                           void* stream);
int launch_ref_order_f64(const RefOrderArgs& a, int nb, void* stream);
int launch_sino_to_dev(const float* host_layout, void* dev_layout, int n_theta, int n_r, int n_rp,
                       int n_t, int fp64, void* stream);
int launch_sino_to_host(const void* dev_layout, float* host_layout, int n_theta, int n_r,
                        int n_rp, int n_t, int fp64, void* stream);
int launch_vol_to_dev(const float* zxy, void* yzx, int n_z, int n_x, int n_y, int fp64,
                      void* stream);
// the same from an FP64 volume in device memory ([z][x][y] doubles)
int launch_vol64_to_dev(const double* zxy, void* yzx, int n_z, int n_x, int n_y, int fp64,
                        void* stream);
int launch_vol_to_host(const void* yzx, float* zxy, int n_z, int n_x, int n_y, int fp64,
                       void* stream);
int launch_error_from_projection(const void* y, const void* yest, void* e, const double* mu,
                                 int n_theta, int n_rp, int n_r, int n_t, int fp64, void* stream);
// per-view FP64 sums; kind 0: joint-estimation sums (6), kind 1: sum e^2 (1)
// per-view sums over detector rows [t_begin, t_end)
int launch_view_sums_rows(int kind, const void* y, const void* e, const double* mu,
                          const double* gain, const double* wv, double* partial, double* out,
                          int n_theta, int n_rp, int n_r, int t_begin, int t_end, int n_chunk,
                          int fp64, void* stream);
int launch_view_sums(int kind, const void* y, const void* e, const double* mu,
                     const double* gain, const double* wv, double* partial, double* out,
                     int n_theta, int n_rp, int n_r, int n_t, int n_chunk, int fp64,
                     void* stream);
int launch_rebuild_error(const void* y, void* e, const double* mu_old, const double* gain_old,
                         const double* mu_new, const double* gain_new, int n_theta, int n_rp,
                         int n_r, int n_t, int fp64, void* stream);
int launch_prior_cost(const void* x, const DevFilter& f, int n_z, int n_x, int n_y,
                      double* partial, int n_blocks, int fp64, void* stream);
int launch_reduce_stats(const double* in, int n_rows, int n_cols, double* out, void* stream);

}  // namespace mbir
