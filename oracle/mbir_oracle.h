/*
 * mbir_oracle.h -- CPU restatement (FP64) of OpenMBIR-TEM's HAADF reconstruction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300 engine: only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The
 * product (libmbir_gb300.so) never links, loads or calls it.
 *
 * Every function restates one piece of the reference (Code/MBIRLib/...) in plain C with
 * the reference's own FP64 arithmetic and loop order; each cites the file:line it follows.
 *
 * PINNED TO THE REFERENCE: the reference's own HAADFReconstruction and BFReconstruction programs,
 * compiled from their sources by oracle/build_ref.py (stand-in Boost/TBB headers, a frozen clock
 * seed), produce outputs that this restatement reproduces bit for bit when it is given the
 * parameters the reference's pipeline hands its engine (oracle/refrun.py) and the C library's
 * pow (pinned_pow = 0): the forward projection, 20 HAADF outer iterations with gain/offset and
 * variance estimation, and 42 bright-field NHICD calls with the Bragg schedule
 * (tests/test_oracle_vs_ref.py against the fixtures of tests/golden/, and live runs).
 */
#ifndef MBIR_ORACLE_H_
#define MBIR_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One resolution level of the engine; field meanings follow TomoInputs and
 * AdvancedParameters (Code/MBIRLib/Reconstruction/ReconstructionStructures.h:113-187). */
typedef struct orc_params {
  double delta_xz_factor;     /* inputs->delta_xz before it is scaled by delta_r (2^(levels-1-i)*final_res) */
  double interpolate_factor;  /* inputs->interpolateFactor (2^(levels-1)*final_res) */
  double length_z;            /* sample thickness in nm (inputs->LengthZ before stretching) */
  int32_t extend_object;
  double x_shrink_factor;     /* 0.6 */
  int32_t z_stretch;          /* 2 */
  int32_t response_bins;      /* 64 */
  int32_t profile_resolution; /* 1536 */
  int32_t beam_resolution;    /* 512 */
  int32_t compat_double_angle;/* 1: voxel profile built from deg*(pi/180)^2 as the HAADF engine does */
  double sigma_x;
  double mrf_p, mrf_q, mrf_c, mrf_alpha;
  double target_gain, default_offset, default_variance, default_recon_value;
  int32_t use_default_offset;
  int32_t joint_estimation, noise_model, zero_skipping;
  double stop_threshold;
  int32_t outer_iterations, inner_iterations;
  double threshold_reduction_factor;
  int32_t pinned_pow;         /* 1: QGGMRF powers by orc_pinned_pow instead of the C library */
  /* bright field (BrightField/BFConstants.h, BFForwardModel) */
  int32_t modality;           /* 0 HAADF, 1 BF */
  int32_t noise_estimation;   /* BF NOISE_ESTIMATION (1): one global variance */
  double bragg_threshold;     /* desired T of the Bragg selector */
  double bragg_delta;         /* delta of the Bragg rejector */
  double bf_offset;           /* added to the raw counts before -log */
  int32_t nhicd;              /* BF NHICD line lists (BFConstants.h); 0: every line per call */
} orc_params;

typedef struct orc_ctx orc_ctx;

/* x^y (x >= 0) by double-double arithmetic from IEEE add/mul/div only; see mbir_oracle.c */
double orc_pinned_pow(double x, double y);

/* geometry + tables; counts is [n_theta][n_r][n_t] (t fastest), tilts in degrees */
orc_ctx* orc_create(const orc_params* p, const double* counts, const double* tilts_deg,
                    int n_theta, int n_r, int n_t, double delta_r, double delta_t);
void orc_destroy(orc_ctx* c);

/* dims[0..2] = n_z, n_x, n_y; geo[0..7] = delta_xz, delta_xy, x0, y0, z0, length_x, length_y, length_z */
void orc_dims(const orc_ctx* c, int32_t* dims, double* geo);
/* offsets[0..1] = OffsetR, OffsetT */
void orc_offsets(const orc_ctx* c, double* offsets);

/* raw state access (FP64, reference layouts): volume [z][x][y]; sinogram arrays [theta][r][t] */
double* orc_volume(orc_ctx* c);
double* orc_error(orc_ctx* c);
double* orc_weight(orc_ctx* c);
double* orc_yest(orc_ctx* c);
/* the measurements the engine works on: the input counts (BF: -log(counts + bf_offset) once
 * prepared) */
double* orc_counts(orc_ctx* c);
double* orc_gain(orc_ctx* c);
double* orc_offset(orc_ctx* c);
double* orc_variance(orc_ctx* c);
const double* orc_detector_response(const orc_ctx* c); /* [n_theta][bins] */
const double* orc_ht(const orc_ctx* c);                /* [bins] */
const double* orc_voxel_profile(const orc_ctx* c);     /* [n_theta][profile_resolution] */
const double* orc_mag_map(const orc_ctx* c);           /* [z][x] */

/* A-matrix column for voxel line (z,x): returns count, fills index (theta*n_r + r) and value */
int orc_amatrix_column(const orc_ctx* c, int z, int x, int32_t* index, double* value, int cap);
/* voxel-line response for slice y: returns count, first t in *t_first, values */
int orc_voxel_line_response(const orc_ctx* c, int y, int32_t* t_first, double* value, int cap);

void orc_init_volume(orc_ctx* c, const double* vol /* NULL: default_recon_value */);
int orc_init_nuisance(orc_ctx* c);        /* initial gains/offsets/variances + renormalisation */
void orc_forward_project(orc_ctx* c);     /* fills yest */
void orc_measurement_weight(orc_ctx* c);  /* e = y - yest - mu, w = 1/alpha */

/* stats[0] = sum|dx| over ROI, stats[1] = sum|x_old| over ROI, stats[2] = zero-skipped count,
 * stats[3] = updated voxel count */
void orc_icd_sweep_reference(orc_ctx* c, uint32_t seed, int outer, int inner, double* stats);
/* the reference's multi-threaded sweep: contiguous y ranges, one per worker thread */
void orc_icd_sweep_reference_mt(orc_ctx* c, uint32_t seed, int outer, int inner, int n_threads,
                                double* stats);
/* the GPU parallel order: colour c in {0,1}: slices y = c, c+2, ...; rows in row_order; within
 * a row, classes k = 0..stride-1 of x = k, k+stride, ... */
void orc_icd_sweep_slices(orc_ctx* c, const int32_t* row_order, int stride, int outer, int inner,
                          double* stats);
/* explicit list of voxel lines (z*n_x+x); every line sweeps all y in order */
void orc_icd_sweep_lines(orc_ctx* c, const int32_t* lines, int n_lines, int outer, int inner,
                         double* stats);

int orc_joint_estimation(orc_ctx* c);
/* HAADF with bright-field data (initializeBrightFieldData): counts [n_theta][n_r][n_t], NULL to
 * clear; call before orc_init_nuisance / orc_measurement_weight */
void orc_set_bf_assist(orc_ctx* c, const double* bf_counts);
void orc_update_weights(orc_ctx* c);
/* parts[0] = data term, parts[1] = prior term, parts[2] = noise term; returns the sum */
double orc_cost(const orc_ctx* c, double* parts);

/* visit order of UpdateYSlice (mt19937 seeded with `seed`, swap-remove) -> n_z*n_x line ids */
void orc_visit_order(uint32_t seed, int n_z, int n_x, int32_t* out);

/* Full single-level execute(): volume init, nuisance init, projection, weights, outer/inner
 * loops with a fixed reference-order seed per sweep.  cost_log (optional, capacity n_cost)
 * receives the cost after every sweep; returns the number of sweeps run. */
int orc_run(orc_ctx* c, uint32_t seed, double* cost_log, int n_cost);
/* the same with sweep k visiting in the order drawn from seed + k * seed_step */
int orc_run_seeded(orc_ctx* c, uint32_t seed, uint32_t seed_step, double* cost_log, int n_cost);

/* ---- bright field -------------------------------------------------------------------- */
/* selector [n_theta][n_r][n_t] (1: entry selected, quadratic data term) */
unsigned char* orc_selector(orc_ctx* c);
double* orc_filt_map(orc_ctx* c);    /* [n_z][n_x] 5x5 Hamming-filtered mag map */
void orc_set_bragg(orc_ctx* c, double t);
double orc_get_bragg(const orc_ctx* c);
/* GenRandList permutation (boost uniform_int on mt19937): out_index[i] = new position of
 * element i */
void orc_rand_list_perm(uint32_t seed, int n, int32_t* out_index);
/* one BFUpdateYSlice call over voxel lines (z*n_x+x) in the given order, y ascending */
void orc_bf_sweep_lines(orc_ctx* c, const int32_t* lines, int n_lines, int outer, int inner,
                        double* stats);
/* the same call in the GPU's slice order over the lines with active[z*n_x+x] != 0 */
void orc_bf_sweep_slices(orc_ctx* c, const unsigned char* active, const int32_t* row_order,
                         int stride, int outer, int inner, double* stats);
/* the same call with each slice visiting the given lines (z*n_x+x) in the given order */
void orc_bf_sweep_slices_order(orc_ctx* c, const int32_t* lines, int n_lines, int outer,
                               int inner, double* stats);
void orc_bf_vsc(orc_ctx* c);
double orc_bf_nh_threshold(const orc_ctx* c);
int orc_bf_nh_lines(const orc_ctx* c, double threshold, int32_t* lines);
double orc_roi_volume_sum(const orc_ctx* c);
double orc_roi_mag_sum(const orc_ctx* c);
void orc_bf_joint_estimation(orc_ctx* c);
void orc_bf_update_weights(orc_ctx* c);
void orc_bf_update_selector(orc_ctx* c);
double orc_bf_cost(const orc_ctx* c, double* parts);
/* BFReconstructionEngine::execute loops in reference (list) order with lists drawn from
 * `seed`; runs at most max_calls updateVoxels calls (<= 0: no limit); returns the calls run */
int orc_bf_run(orc_ctx* c, uint32_t seed, int max_calls);
/* the same with every list drawn from `seed` (the reference with its clock seed frozen) */
int orc_bf_run_fixed_seed(orc_ctx* c, uint32_t seed, int max_calls);
/* y-slab sharding: one colour of the slice-order sweep over slices [y0, y1); per-view sums over
 * detector rows [t0, t1) (kind 0: [theta][6] jointEstimation sums, kind 1: [theta] sum e^2);
 * nuisance update with the jointEstimation error rebuild (variance may be null) */
void orc_icd_sweep_colour(orc_ctx* c, const int32_t* row_order, int stride, int colour, int y0,
                          int y1, int outer, int inner, double* stats);
void orc_view_sums(const orc_ctx* c, int kind, int t0, int t1, double* out);
/* bright-field slabs (rows [t0, t1), slices [y0, y1)) */
void orc_bf_reset_mag(orc_ctx* c, const unsigned char* active);
void orc_bf_sweep_colour(orc_ctx* c, const unsigned char* active, const int32_t* row_order,
                         int stride, int colour, int y0, int y1, int outer, int inner,
                         double* stats);
void orc_bf_offset_sums(const orc_ctx* c, int t0, int t1, double* out);
void orc_bf_apply_offsets(orc_ctx* c, const double* sums, int t0, int t1);
void orc_bf_variance_sums(orc_ctx* c, int t0, int t1, double* out3);
void orc_bf_apply_variance(orc_ctx* c, const double* sums, int t0, int t1);
double orc_roi_volume_sum_range(const orc_ctx* c, int y0, int y1);
void orc_apply_nuisance(orc_ctx* c, const double* gain, const double* offset,
                        const double* variance);
/* one call with the reference's worker split over y (timing of the reference CPU path) */
void orc_bf_sweep_lines_mt(orc_ctx* c, const int32_t* lines, int n_lines, int outer, int inner,
                           int n_threads, double* stats);

#ifdef __cplusplus
}
#endif
#endif
