/*
 * mbir_gb300.h -- C ABI of the GB300-native MBIR reconstruction engine (HAADF/BF electron
 * tomography).  Plain pointers and sizes only; no C++ or CUDA types cross this boundary.
 *
 * Reference interface each entry point replaces (paths relative to the OpenMBIR-TEM root):
 *   HAADF_ReconstructionEngine::New / set{TomoInputs,Sinogram,Geometry,AdvParams,ForwardModel}
 *     -> mbir_params_default + mbir_create + mbir_set_sinogram / mbir_load_sinogram_mrc
 *        (Code/MBIRLib/HAADF/HAADF_ReconstructionEngine.h:67-99; wiring in
 *         Code/MBIRLib/HAADF/HAADF_MultiResolutionReconstruction.cpp:392-437)
 *   HAADF_ReconstructionEngine::execute -> mbir_run  (HAADF_ReconstructionEngine.cpp:327-913)
 *   AbstractFilter::setCancel / getErrorCondition -> mbir_cancel / return codes + mbir_last_error
 *     (Code/MBIRLib/Common/AbstractFilter.h:46-82, Observable.h:65-101)
 *   Geometry->Object read-out, HAADF_ForwardModel::getI_0/getMu/getAlpha
 *     -> mbir_get_volume / mbir_get_nuisance (HAADF_ForwardModel.h:70-90)
 *   HAADF_ForwardModel::writeMRCFile / writeReconstructionFile / writeNuisanceParameters
 *     -> mbir_write_outputs (HAADF_ForwardModel.cpp:34-245)
 * The step-wise entry points (mbir_prepare, mbir_sweep, mbir_joint_estimation,
 * mbir_update_weights, mbir_compute_cost, mbir_forward_project) expose the phases execute()
 * runs internally (forward projection :655-691, updateVoxels :739-740, jointEstimation :774,
 * updateWeights :784, computeCost :1147) so callers can drive or check them one at a time.
 *
 * Threading: mbir_run blocks; mbir_cancel and mbir_status may be called from another thread.
 * Engines are independent.  Every function returns MBIR_OK (0) or a negative MBIR_E* code;
 * no C++ exception crosses this boundary.
 */
#ifndef MBIR_GB300_H_
#define MBIR_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MBIR_OK 0
#define MBIR_EINVAL (-1)     /* bad argument or parameter */
#define MBIR_ENOMEM (-2)     /* device or host allocation failed */
#define MBIR_EDEVICE (-3)    /* CUDA error / no usable device */
#define MBIR_EIO (-4)        /* file could not be read or written */
#define MBIR_ESTATE (-5)     /* call made in the wrong order */
#define MBIR_ETIMEOUT (-6)   /* a bounded device wait gave up */
#define MBIR_ENOTSUP (-7)    /* configuration this build does not run */
#define MBIR_ECANCELLED (-999) /* the reference's cancel code (HAADF_ReconstructionEngine.cpp:401) */

#define MBIR_MODALITY_HAADF 0
#define MBIR_MODALITY_BF 1

#define MBIR_ORDER_PARALLEL 0  /* red/black y-slices x conflict-free voxel sets (GPU order) */
#define MBIR_ORDER_REFERENCE 1 /* the reference's single-task random line order, y sequential */

#define MBIR_SEED_PER_CALL 0   /* reference order: HAADF sweep k visits in the order drawn from
                                  seed + k, BF NHICD call k's list from seed + 1 + k (the reference
                                  reseeds from its millisecond clock each time) */
#define MBIR_SEED_FIXED 1      /* reference order: every order and list drawn from `seed`, as the
                                  reference draws them when its clock seed does not change */

#define MBIR_PRECISION_FP32 0  /* volume, error sinogram and footprints in FP32 (reductions FP64) */
#define MBIR_PRECISION_FP64 1  /* everything in FP64, the reference's Real_t */

/* Parameter set: the reference CLI/pipeline inputs (HAADFReconstructionArgsParser.cpp:143-211,
 * BFReconstructionArgsParser.cpp:145-226), the AdvancedParameters
 * (ReconstructionStructures.h:164-187, defaults HAADF_ReconstructionEngine.cpp:244-259), the
 * QGGMRF constants (HAADF_QGGMRFPriorModel.cpp:10-21) and the engine's own switches.
 * mbir_params_default fills every field; unset fields are zero. */
typedef struct mbir_params {
  int32_t struct_size;        /* sizeof(mbir_params), checked by mbir_create */
  int32_t modality;           /* MBIR_MODALITY_HAADF / MBIR_MODALITY_BF */
  /* pipeline / TomoInputs */
  double sample_thickness;    /* --thickness (nm) */
  double diffuseness;         /* --diffuseness; prior q = diffuseness + 1 */
  double sigma_x;             /* --sigma_x */
  double stop_threshold;      /* --stop_threshold */
  int32_t num_resolutions;    /* --num_resolutions */
  int32_t final_resolution;   /* --final_resolution */
  int32_t level;              /* resolution level this engine runs (0 = coarsest); -1 = finest */
  double target_gain;         /* --target_gain */
  int32_t outer_iterations;   /* --outer_iterations */
  int32_t inner_iterations;   /* --inner_iterations */
  double default_offset;      /* --default_offset */
  int32_t use_default_offset; /* --use_default_offset */
  double default_variance;    /* --default_variance */
  double default_recon_value; /* --default_recon_value */
  int32_t extend_object;      /* --extend_object */
  int32_t interpolate_initial_recon; /* --interpolate_initial_recon: mbir_set_initial_volume takes
                                 a half-size volume and replicates each voxel 2x2x2 */
  int32_t tilt_selection;     /* --tilt_selection: 0 = a-tilt, 1 = b-tilt */
  int32_t use_subvolume;      /* --subvolume given */
  int32_t subvolume[6];       /* xmin,ymin,zmin,xmax,ymax,zmax */
  double default_pixel_size;  /* nm; used when the MRC has no FEI extended header */
  int32_t n_excluded_views;   /* --exclude_views */
  int32_t excluded_views[256];
  /* AdvancedParameters */
  double x_shrink_factor;     /* 0.6 */
  int32_t z_stretch;          /* 2 */
  int32_t detector_response_bins; /* 64 */
  int32_t profile_resolution; /* 1536 */
  int32_t beam_resolution;    /* 512 */
  int32_t joint_estimation;   /* 1 */
  int32_t zero_skipping;      /* 1 */
  int32_t noise_model;        /* 1 */
  int32_t noise_estimation;   /* 0 (never set by the reference; zero-initialised here) */
  int32_t estimate_prior;     /* 0 (1 is not supported: mbir_create fails, MBIR_ENOTSUP elsewhere) */
  double threshold_reduction_factor; /* 1 */
  /* QGGMRF prior rho(d) = (|d|^P/s^P) / (c + |d|^(P-Q)/s^(P-Q)) */
  double qggmrf_p;            /* 2 */
  double qggmrf_q;            /* 0 -> diffuseness + 1 */
  double qggmrf_c;            /* 0.001 HAADF, 0.01 BF */
  double qggmrf_alpha;        /* 1.5 over-relaxation */
  /* bright field */
  double bragg_threshold, bragg_delta, bf_offset, default_dosage;
  /* engine switches */
  int32_t order_mode;         /* MBIR_ORDER_PARALLEL / MBIR_ORDER_REFERENCE */
  int32_t precision;          /* MBIR_PRECISION_FP32 / MBIR_PRECISION_FP64 */
  uint32_t seed;              /* visit-order seed (reference mode: mt19937 seed per sweep) */
  int32_t compat_double_angle;/* 1: HAADF voxel profile from deg*(pi/180)^2, as the reference */
  int32_t cost_every_sweep;   /* 1: evaluate the FP64 MAP cost after every sweep */
  int32_t device;             /* CUDA device ordinal */
  int32_t verbose;
  int32_t slice_staging;      /* 0: a slice's detector rows sit in shared memory when they fit,
                                 1: always work on them in HBM (same results, for tuning) */
  int32_t nhicd;              /* BF: 1 = non-homogeneous ICD line lists (the reference's NHICD
                                 build, BFConstants.h), 0 = every voxel line in each call */
  int32_t lane_shape;         /* FP32 voxel-group shape: 0 = autotuned at prepare; 1 = 16 lanes x
                                 4 views (<= 64 views), 2 = 32 x 2 (<= 64), 3 = 32 x 3 (<= 96),
                                 4 = 32 x 5 (<= 160), 5 = 32 x 8 (161-256 views; slices in HBM,
                                 taken by default there).  Results depend on the shape in the last
                                 bits (summation order); fix it for bit-reproducible runs.  Above
                                 160 views: parallel order only, no batch. */
  int32_t call_schedule;      /* BF NHICD calls (FP32, parallel order): 0 = colour the call's
                                 conflict graph and run the colour classes in turn (one barrier
                                 per class; the visit order is colour by colour), 1 = walk the
                                 rows class by class, 2 = the row walk's visit order run in
                                 dependency levels (one barrier per level, the row walk's
                                 bits).  mbir_get_call_lines returns the visit order of 0 and 2.
                                 The colouring runs on the device; the schedules of the 20
                                 homogeneous sub-lists are built once and reused. */
  int32_t seed_mode;          /* MBIR_SEED_PER_CALL / MBIR_SEED_FIXED (reference order) */
  int32_t float_params;       /* 1: round the parameters the reference's pipeline keeps in float
                                 members (thickness, target gain, stop threshold, sigma_x,
                                 diffuseness with q = diffuseness + 1 in float, default offset,
                                 variance and initial value, Bragg T / delta / offset, the BF
                                 offset -log(dosage + bf_offset)), so results equal the
                                 reference's command-line runs; 0: use the values as given */
} mbir_params;

typedef struct mbir_status {
  int32_t state;          /* 0 created, 1 sinogram set, 2 prepared, 3 running, 4 done, <0 error */
  int32_t outer_iter, inner_iter;
  int32_t sweeps_done;
  double last_cost;       /* NaN when not computed */
  double last_rel_update; /* sum|dx| / sum|x| over the ROI from the last sweep */
  double icd_ms_total;    /* device time in the ICD kernels */
  double total_ms;        /* wall time of mbir_run */
  int64_t voxels_visited; /* voxel visits in ICD sweeps (updated + zero-skipped) */
  int64_t voxels_updated; /* voxel updates (not zero-skipped) */
  int64_t footprint_entries; /* sum over voxel lines (z,x) of the A-column nonzeros */
  int32_t t_rows;         /* detector rows touched by one voxel slice (voxel-line response) */
  int32_t stride;         /* x stride of the conflict-free voxel sets */
  int32_t staged;         /* 1: voxel slices staged in shared memory, 0: slices read from HBM */
  int32_t lane_shape;     /* voxel-group shape in use (see mbir_params.lane_shape) */
  int32_t sched_levels;   /* dependency levels of the last level-scheduled BF call (0: none) */
  double sched_ms_total;  /* host time spent building level schedules */
  double kernel_ms_total; /* device time of the parallel-order sweep kernels alone (colour
                             launches; icd_ms_total also holds list, schedule and statistics) */
  double colour_ms_total; /* device time of the colour-schedule launches (call_schedule 0) */
} mbir_status;

typedef struct mbir_engine mbir_engine;

/* defaults of InitializeAdvancedParams + the CLI defaults for the modality */
void mbir_params_default(mbir_params* p, int32_t modality);

mbir_engine* mbir_create(const mbir_params* p);
void mbir_destroy(mbir_engine* e);
const char* mbir_last_error(const mbir_engine* e);

/* Sinogram already cut to the region of interest: counts[theta][r][t] (t fastest), tilts in
 * degrees (one per view), pixel pitch in nm.  Replaces MRCSinogramInitializer's result. */
int32_t mbir_set_sinogram(mbir_engine* e, const float* counts, const float* tilts_deg,
                          int32_t n_theta, int32_t n_r, int32_t n_t, double delta_r,
                          double delta_t);
/* MRC modes 0/1/2/6 with FEI extended header; honours use_subvolume/subvolume,
 * excluded_views and tilt_selection exactly as the reference reader. */
int32_t mbir_load_sinogram_mrc(mbir_engine* e, const char* path);

/* HAADF with bright-field data: a bright-field tilt series of the sinogram's size,
 * counts[theta][r][t]; each count plus BF_OFFSET (32768) multiplies its measurement's model,
 * and the joint estimation estimates the offsets only.  After the sinogram, before prepare.
 * Replaces HAADF_ReconstructionEngine::setBFTomoInputs/setBFSinogram and
 * initializeBrightFieldData (HAADF_MultiResolutionReconstruction.cpp:421-422,
 * HAADF_ReconstructionEngine_Extra.cpp:84-176, :429, :643-668, _UpdateVoxels.cpp:354-364,
 * :438-446).  Engines with it run alone: not in a batch, not in slabs.  MBIR_EINVAL when the
 * sizes differ ("The two file sizes are not matched"). */
int32_t mbir_set_bright_field(mbir_engine* e, const float* counts, int32_t n_theta, int32_t n_r,
                              int32_t n_t);
/* The same from an MRC file, read with the sinogram's subvolume (and, when that read fails,
 * over the sinogram's own extent), as the reference reads its --brightfield file. */
int32_t mbir_load_bright_field_mrc(mbir_engine* e, const char* path);

/* Optional initial volume [z][x][y] (y fastest), sized as mbir_get_dims reports; with
 * interpolate_initial_recon set, (N_z/2) x (N_x/2) x (N_y/2) values, each filling its 2x2x2 block
 * (InitialReconstructionBinReader.cpp:101-131; needs the sinogram set first). */
int32_t mbir_set_initial_volume(mbir_engine* e, const float* vol, int64_t n);
/* The same as doubles: the reference hands resolution levels the doubles of
 * ReconstructedObject.bin, and an FP64 engine starts from them exactly. */
int32_t mbir_set_initial_volume_f64(mbir_engine* e, const double* vol, int64_t n);
/* Optional initial nuisance vectors (length n_theta each; NULL keeps the default). */
int32_t mbir_set_initial_nuisance(mbir_engine* e, const double* gains, const double* offsets,
                                  const double* variances);

/* dims[0..2] = N_z, N_x, N_y of the volume; dims[3..5] = N_theta, N_r, N_t */
int32_t mbir_get_dims(mbir_engine* e, int32_t* dims);

/* execute(): prepare + outer/inner loop + nuisance updates; blocking. */
int32_t mbir_run(mbir_engine* e);

/* Step-wise phases of execute() */
int32_t mbir_prepare(mbir_engine* e);
int32_t mbir_sweep(mbir_engine* e, int32_t outer, int32_t inner, double* stats4);
int32_t mbir_joint_estimation(mbir_engine* e);
int32_t mbir_update_weights(mbir_engine* e);
int32_t mbir_compute_cost(mbir_engine* e, double* parts3, double* total);
int32_t mbir_forward_project(mbir_engine* e);

/* Read-outs (host buffers owned by the caller) */
int32_t mbir_get_volume(mbir_engine* e, float* out, int64_t n);
/* The volume as doubles, [z][x][y] (an FP64 engine's values exactly; the values written to
 * ReconstructedObject.bin). */
int32_t mbir_get_volume_f64(mbir_engine* e, double* out, int64_t n);          /* [z][x][y] */
int32_t mbir_get_error_sinogram(mbir_engine* e, float* out, int64_t n);  /* [theta][r][t] */
int32_t mbir_get_projection(mbir_engine* e, float* out, int64_t n);      /* last forward projection [theta][r][t] */
int32_t mbir_get_nuisance(mbir_engine* e, double* gains, double* offsets, double* variances);
/* detector response H [n_theta][bins] and t-response H_t [bins] (FP64 as built) */
int32_t mbir_get_tables(mbir_engine* e, double* H, double* Ht);
/* parallel-mode schedule: row order of sweep `sweep` (N_z entries) and the x stride */
int32_t mbir_get_schedule(mbir_engine* e, int32_t sweep, int32_t* row_order, int32_t* stride);
/* voxel lines (z*N_x + x) of the last sweep or bright-field call: the visit order in reference
 * order, ascending in parallel order (a bright-field NHICD call updates a subset of lines).
 * *n receives the count; lines may be null to query it. */
int32_t mbir_get_call_lines(mbir_engine* e, int32_t* lines, int32_t cap, int32_t* n);
/* bright field: Bragg selector [theta][r][t] (1 = selected), weights [theta][r][t], per-line
 * update magnitudes and their VSC-filtered map [z][x], current Bragg threshold T.  Outputs may
 * be null.  Replaces BFForwardModel's selector/weight state and the magUpdateMap of
 * BFReconstructionEngine::execute (BFReconstructionEngine.cpp:670-690). */
int32_t mbir_get_bf_state(mbir_engine* e, uint8_t* selector, float* weights, double* mag,
                          double* filtered_mag, double* bragg_t);
/* BFForwardModel::setBraggThreshold (BFForwardModel.h): T used by the next calls */
int32_t mbir_set_bragg_threshold(mbir_engine* e, double t);

/* y-slab sharding of one reconstruction over several engines (one per GPU), driven by a host
 * that exchanges boundary planes and sums per-view statistics between them.  Replaces the
 * y-range task split of updateVoxels (HAADF_ReconstructionEngine_UpdateVoxels.cpp:666-723)
 * across devices instead of threads.  Parallel order (bright field below).
 *   mbir_set_slab: later colour sweeps and view sums cover slices [y0, y1) only (0, 0 = all)
 *   mbir_sweep_colour: one colour (0 even, 1 odd slices) of the parallel sweep; the row order of
 *     sweep k serves both colours and the sweep counts after colour 1
 *   mbir_get_planes / mbir_set_planes: voxel planes y .. y+n-1 as [n][z][x] floats (FP32 engines)
 *   mbir_view_sums: kind 0 = the six jointEstimation sums per view [theta][6] (y w, w, yh w,
 *     yh w y, y^2 w, yh^2 w; _Extra.cpp:474-517), kind 1 = sum e^2 per view (:825-833), over the
 *     detector rows of the slab
 *   mbir_apply_nuisance: new gain/offset (null to keep) with the jointEstimation error rebuild
 *     (:600-612) and/or new variance (null to keep) */
int32_t mbir_set_slab(mbir_engine* e, int32_t y0, int32_t y1);
int32_t mbir_sweep_colour(mbir_engine* e, int32_t colour, int32_t outer, int32_t inner,
                          double* stats4);
int32_t mbir_get_planes(mbir_engine* e, int32_t y, int32_t n, float* out);
int32_t mbir_set_planes(mbir_engine* e, int32_t y, int32_t n, const float* in);
int32_t mbir_view_sums(mbir_engine* e, int32_t kind, double* out);
int32_t mbir_apply_nuisance(mbir_engine* e, const double* gain, const double* offset,
                            const double* variance);
/* Bright-field slabs (BFReconstructionEngine_Extra.cpp:624-752, the y-range task split of a
 * call, with the tasks' magnitude maps reduced afterwards, :719-752): one NHICD call is
 *   mbir_bf_call_begin: the call's lines (next homogeneous sub-list, or the non-homogeneous
 *     list from the magnitude map), schedule and row order; then mbir_sweep_colour (0, 1) with
 *     the halo exchange after each colour
 *   mbir_bf_call_magnitudes: the call's update magnitude per line [z][x] over the slab's slices
 *     (sum |dx| in fixed point, 2^-32 units), for the host to add over slabs
 *   mbir_bf_call_end: the magnitude map takes the summed magnitudes (null: the slab's own) and
 *     the call is counted
 * and after an outer iteration
 *   mbir_bf_slab_sums: kind 2 = the offset step's numerator and denominator per view [theta][2]
 *     (jointEstimation, BFForwardModel.cpp:390-441); kind 3 = the variance sums over selected
 *     and rejected entries and the number of entries [3] (updateWeights, :447-511; scales the
 *     slab's weights by the current variance first, so once per update), over the slab's
 *     detector rows
 *   mbir_bf_slab_apply: the same kind's sums added over slabs: offset steps or the common
 *     variance, then the Bragg selector (updateSelector, :517-531)
 *   mbir_roi_sums: the stop rule's ROI sums (_Extra.cpp:1200-1248): [0] of the magnitude map,
 *     [1] of the slab's volume (to add over slabs) */
int32_t mbir_bf_call_begin(mbir_engine* e, int32_t outer, int32_t inner);
int32_t mbir_bf_call_magnitudes(mbir_engine* e, uint64_t* out);
int32_t mbir_bf_call_end(mbir_engine* e, const uint64_t* magnitudes);
int32_t mbir_bf_slab_sums(mbir_engine* e, int32_t kind, double* out);
int32_t mbir_bf_slab_apply(mbir_engine* e, int32_t kind, const double* sums);
int32_t mbir_roi_sums(mbir_engine* e, double* out2);
int32_t mbir_status_get(mbir_engine* e, mbir_status* st);
void mbir_cancel(mbir_engine* e);

/* ReconstructedVolume MRC (float32, z reversed, x cropped as the reference), ReconstructedObject.bin
 * (double, y-x-z), Final{Gain,Offset}Parameters.bin and FinalVariances.bin (double[N_theta]),
 * ReconstructedSinogram.bin ((y - e) * I + mu, double [theta][r][t]) in `dir`.  Replaces
 * HAADF_ForwardModel::writeMRCFile / writeReconstructionFile / writeNuisanceParameters /
 * writeSinogramFile (HAADF_ForwardModel.cpp:34-137). */
int32_t mbir_write_outputs(mbir_engine* e, const char* dir, const char* mrc_path);
/* The same plus the VTK legacy volume (binary structured points, big-endian float32, scalar
 * "TomoVoxel") and the Avizo AmiraMesh volume (binary little-endian float lattice) when their
 * paths are not NULL or empty; replaces writeVtkFile / writeAvizoFile
 * (HAADF_ForwardModel.cpp:139-242, VTKFileWriters.hpp, AvizoUniformCoordinateWriter.cpp). */
int32_t mbir_write_outputs_ex(mbir_engine* e, const char* dir, const char* mrc_path,
                              const char* vtk_path, const char* avizo_path);
/* HAADF: during mbir_run, after every inner iteration, the volume as the MRC file
 * <dir>/<outer>_<inner>_ReconstructedVolume.rec, the intermediate image the reference writes to
 * its temporary directory (HAADF_ReconstructionEngine.cpp:757-763); NULL or "" turns it off. */
int32_t mbir_set_intermediate_dir(mbir_engine* e, const char* dir);

/* Checkpoint and exact resume of a HAADF run (without bright-field data).  mbir_write_checkpoint
 * (after mbir_run or between step-wise phases) writes to `dir` (an existing directory) the
 * reference's level hand-off files ReconstructedObject.bin, Final{Gain,Offset}Parameters.bin and
 * FinalVariances.bin (HAADF_MultiResolutionReconstruction.cpp:212-222 reads them back;
 * InitialReconstructionBinReader.cpp:73-168) plus ReconstructedSinogram.bin and Checkpoint.bin
 * (the outer iterations mbir_run has completed, the sweeps done, the stop threshold after its
 * reductions and the error sinogram).
 * mbir_read_checkpoint, on an engine created with the same parameters and given the same series
 * (after mbir_set_sinogram / mbir_load_sinogram_mrc), makes every later prepare start from that
 * state, and mbir_run continues at the checkpoint's outer iteration up to outer_iterations: a
 * run of N outer iterations and a run of K, checkpointed and resumed to N, give the same bits.
 * MBIR_EINVAL when the checkpoint comes from another configuration or series, MBIR_EIO when a
 * file is missing or short, MBIR_ENOTSUP for bright field.  The reference resumes only from a
 * volume (--initial_recon_file, HAADFReconstructionArgsParser.cpp:189-190). */
int32_t mbir_write_checkpoint(mbir_engine* e, const char* dir);
int32_t mbir_read_checkpoint(mbir_engine* e, const char* dir);

/* Observer of an engine's messages, in place of the reference's Observable::notify(msg,
 * progress, aspect) (Code/MBIRLib/Common/Observable.h:65-101); the aspect numbers follow its
 * ObserverAspect order.  The engine sends "Calculating A Matrix...." (0, progress message) and
 * "Starting Forward Projection" (10, progress value and message) from prepare, the path of each
 * intermediate image (0, intermediate image), "Reconstruction Complete" (100, progress value
 * and message) at the end of mbir_run, and the text of every error it returns (100, error
 * message; the same text as mbir_last_error).  mbir_run also sends after every outer iteration
 * one line of metrics as a JSON object (progress = the share of outer_iterations done, progress
 * message): {"outer", "sweeps" (ICD calls so far), "rel_update" (the last sweep's
 * sum|dx| / sum|x| over the ROI), "cost" (the last FP64 cost, null when none was computed),
 * "voxels_updated", "icd_ms" (both so far)}.  fn runs on the thread that does the engine's
 * work: the caller's, or for an engine in a batch or a server, one of their threads.  It must not
 * throw, and must not call the same engine except mbir_cancel, mbir_status_get and
 * mbir_last_error.  fn = NULL removes the observer. */
#define MBIR_UPDATE_PROGRESS_VALUE 0
#define MBIR_UPDATE_PROGRESS_MESSAGE 1
#define MBIR_UPDATE_WARNING_MESSAGE 2
#define MBIR_UPDATE_ERROR_MESSAGE 3
#define MBIR_UPDATE_PROGRESS_VALUE_AND_MESSAGE 4
#define MBIR_UPDATE_INTERMEDIATE_IMAGE 5
typedef void (*mbir_observer_fn)(const char* msg, int32_t progress, int32_t aspect, void* user);
int32_t mbir_set_observer(mbir_engine* e, mbir_observer_fn fn, void* user);

/* Multi-resolution pipeline (HAADF_MultiResolutionReconstruction::execute,
 * HAADF_MultiResolutionReconstruction.cpp:175-485): coarse-to-fine levels with sigma_x scaling
 * and 2x voxel replication hand-off; writes the final volume to out ([z][x][y], n floats). */
int32_t mbir_run_multires(const mbir_params* p, const float* counts, const float* tilts_deg,
                          int32_t n_theta, int32_t n_r, int32_t n_t, double delta_r,
                          double delta_t, float* out, int64_t n, int32_t* dims_out);

/* Batched execution (config "many uneven reconstructions"): prepared FP32 parallel-order
 * engines on one device advance together, one persistent cooperative launch per ICD sweep
 * covering every voxel slice of every engine; gain/offset, variance and cost stay per engine.
 * The reference has no counterpart: it runs one reconstruction per process
 * (HAADF_MultiResolutionReconstruction.cpp:175-485). */
typedef struct mbir_batch mbir_batch;
mbir_batch* mbir_batch_create(int32_t device);
void mbir_batch_destroy(mbir_batch* b);
int32_t mbir_batch_add(mbir_batch* b, mbir_engine* e);
int32_t mbir_batch_remove(mbir_batch* b, mbir_engine* e);
int32_t mbir_batch_size(const mbir_batch* b);
/* threads per CTA of the persistent batched sweep (the slice-group shape): 512 (one slice per
 * SM), 256 (two slices per SM; a slice's detector rows are staged in shared memory only when
 * two CTAs' worth fits, otherwise they are used in place in HBM) or 0 (default: tuned online,
 * the second to fifth sweeps running 512, 256, 256, 512 and the one with the lower device time
 * per updated voxel kept).  Same results either way.  get: the value in use (0 while tuning). */
int32_t mbir_batch_set_threads(mbir_batch* b, int32_t threads);
int32_t mbir_batch_get_threads(mbir_batch* b);
/* Limit (seconds, default 10) of the device-side wait in a batched sweep: a colour-1 slice waits
 * for its series' colour-0 slices, and a wait that runs out skips that slice; the sweep then
 * returns MBIR_ETIMEOUT and the engines stay usable.  No counterpart in the reference (its
 * threads join with no limit, HAADF_ReconstructionEngine_UpdateVoxels.cpp:715). */
int32_t mbir_batch_set_wait_limit(mbir_batch* b, double seconds);
/* one sweep of every engine (outer index drives zero skipping); stats: 4 doubles per engine */
int32_t mbir_batch_sweep(mbir_batch* b, int32_t outer, double* stats);
/* outer iterations (batched sweep + per-engine gain/offset, variance, cost) until each engine's
 * relative cost change <= cost_rel_tol or max_outer; per-engine iteration counts and costs */
int32_t mbir_batch_run(mbir_batch* b, int32_t max_outer, double cost_rel_tol,
                       int32_t* outer_done, double* final_cost);
/* device time (ms) of the last batched sweep and of all batched sweeps */
double mbir_batch_last_ms(const mbir_batch* b);
double mbir_batch_total_ms(const mbir_batch* b);
const char* mbir_batch_last_error(const mbir_batch* b);

/* Serving (config "served stream"): a request loop on one device that admits tilt series of
 * any size by device memory, keeps each admitted request resident, advances all active
 * requests together (one batched sweep per outer iteration, continuous batching: arrivals join
 * between sweeps) and retires each one when its relative cost change <= cost_rel_tol or after
 * max_outer iterations.  Thread-safe.  No reference counterpart. */
typedef struct mbir_server mbir_server;
typedef struct mbir_server_stats {
  int64_t submitted, completed, failed;
  int32_t active, queued;
  double p50_ms, p99_ms, mean_ms;  /* request latency: completion - submission */
  double voxel_updates;            /* voxel visits of retired requests */
  double busy_s;                   /* worker time with requests on the device */
  double batched_sweep_ms;         /* device time of all batched sweeps */
  int64_t batched_sweeps;
  int64_t budget_bytes;            /* device-memory budget for admitted requests */
  int64_t peak_bytes;              /* largest estimated footprint resident at one time */
  int32_t peak_active;             /* most requests on the device at one time */
  int32_t reserved;
  int64_t admitted;                /* requests admitted so far */
  int64_t admitted_out_of_order;   /* admissions that overtook an earlier request (0: FIFO) */
} mbir_server_stats;
/* mem_budget_bytes <= 0: 80% of the free device memory; max_active <= 0: 64 */
mbir_server* mbir_server_create(int32_t device, int64_t mem_budget_bytes, int32_t max_active);
void mbir_server_destroy(mbir_server* s);
/* returns a request id > 0, or a negative MBIR_E* code; inputs are copied */
int64_t mbir_server_submit(mbir_server* s, const mbir_params* p, const float* counts,
                           const float* tilts_deg, int32_t n_theta, int32_t n_r, int32_t n_t,
                           double delta_r, double delta_t, int32_t max_outer,
                           double cost_rel_tol);
/* state: 0 queued, 1 active, 2 done, < 0 failed with that code */
int32_t mbir_server_poll(mbir_server* s, int64_t id, int32_t* state, double* latency_ms,
                         int32_t* outer_done, double* cost);
int32_t mbir_server_wait(mbir_server* s, int64_t id, double timeout_s);
int32_t mbir_server_result(mbir_server* s, int64_t id, float* out, int64_t n, int32_t* dims);
int32_t mbir_server_release(mbir_server* s, int64_t id);
int32_t mbir_server_get_stats(mbir_server* s, mbir_server_stats* st);
const char* mbir_server_last_error(const mbir_server* s);

/* Estimate of sigma_x from an MRC tilt series (host only), as SigmaXEstimation::execute
 * (GenericFilters/SigmaXEstimation.cpp:137-234) computes it for the reference's GUIs: per view the
 * mean absolute deviation of the counts in the region x_range x y_range (bright field, with
 * use_bf_offset: of log(counts + bf_offset)), divided by target_gain, times cos(tilt) /
 * sample_thickness, summed over the tilts and divided by the view count.  The region follows the
 * reference's reader (columns x_range[0]..x_range[1] and rows y_range[0]..y_range[1] read
 * inclusively, the first (x1-x0)(y1-y0) values used); a NULL range or negative bounds mean
 * 0..nx (0..ny).  tilts_deg: n_tilts angles, or n_tilts = 0 for the FEI header's a-tilts. */
int32_t mbir_estimate_sigma_x(const char* mrc_path, double sample_thickness, double target_gain,
                              int32_t use_bf_offset, double bf_offset, const float* tilts_deg,
                              int32_t n_tilts, const int32_t* x_range, const int32_t* y_range,
                              double* sigma_x);

/* Library version string */
const char* mbir_version(void);

/* Per-view sums of squared errors, sums_dev[v] = sum over r, t of error_dev[v][r][t]^2 (the sums a
 * per-view noise-variance estimate divides by N_r N_t), computed on caller-owned device buffers
 * (FP32 error sinogram in the reference's [theta][r][t] layout, FP64 output of n_theta values)
 * with no allocation: for callers whose device memory is owned by their own pool, or whose path
 * must not allocate.  No counterpart in the reference (it is this
 * library's addition).  Limits: n_theta <= 1024 (MBIR_EINVAL beyond); the scratch (128 KiB of
 * per-view partial sums, fully rewritten by every call) lives in one static device array per
 * device, so calls that overlap in time race and must be serialised by the caller.  The first call
 * on a device looks the scratch up (with that device current): make it before any stream capture.
 * Launches on `stream` (a cudaStream_t, 0 = legacy default stream) and does not synchronise. */
int32_t mbir_error_view_sums_noalloc(const float* error_dev, int32_t n_theta, int32_t n_r,
                                     int32_t n_t, double* sums_dev, void* stream);

/* Dependency levels of one sparse ICD call (host only; the schedule a level-scheduled BF NHICD
 * call runs with mbir_params.call_schedule = 2).  The visit order is the row walk's: rows in rows[n_z],
 * within a row the classes x = k (mod stride), k = 0..stride-1, x ascending.  A line (z*n_x + x)
 * is in the call when lineok[l] and (active == NULL or active[l]).  lo[l*n_theta + v] is the
 * first detector bin of line l at view v and bit b of mask[l*n_theta + v] marks bin lo+b as
 * touched (b < nb <= 16, lo+b in [0, n_r)).  level(l) = 1 + the largest level of an earlier line
 * that shares a touched bin at some view or lies in l's 3x3 (z, x) neighbourhood.  Writes the
 * lines level by level (visit order within a level) to lines[lines_cap] and the level offsets to
 * lofs[lofs_cap] (n_levels + 1 values); *n_lines, *n_levels receive the counts.  Replaces no
 * reference interface (the reference updates a call's lines one after another,
 * BFReconstructionEngine_Extra.cpp:476-628).  MBIR_EINVAL on bad input or short buffers. */
int32_t mbir_level_schedule(int32_t n_z, int32_t n_x, int32_t n_theta, int32_t n_r, int32_t nb,
                            int32_t stride, const int32_t* rows, const uint8_t* lineok,
                            const uint8_t* active, const int16_t* lo, const uint16_t* mask,
                            int32_t* lines, int32_t lines_cap, int32_t* lofs, int32_t lofs_cap,
                            int32_t* n_lines, int32_t* n_levels);

/* The last scheduled BF call's schedule (call_schedule 0 or 2): its lines level by level
 * (lines[cap]) and the level offsets (lofs[lofs_cap], n_levels + 1 values); *n_lines and
 * *n_levels receive the counts (0 after a row-walk call).  Any pointer may be NULL.  No
 * counterpart in the reference (its calls run one line after another). */
int32_t mbir_get_call_schedule(mbir_engine* e, int32_t* lines, int32_t cap, int32_t* lofs,
                               int32_t lofs_cap, int32_t* n_lines, int32_t* n_levels);
/* The footprint support the schedules use, for a prepared FP32 BF engine with NHICD: per line
 * l = z*n_x + x and view v, lo[l*n_theta + v] = first detector bin and bit b of
 * mask[l*n_theta + v] = bin lo+b has a nonzero FP32 A-matrix entry; lineok[l] = the line's
 * A-column is not empty.  MBIR_ENOTSUP when the engine builds no schedules.  Mirrors the A-column
 * support of AMatrixCol (Code/MBIRLib/Common/AMatrixCol.cpp:148-232). */
int32_t mbir_get_footprint_bins(mbir_engine* e, int16_t* lo, uint16_t* mask,
                                uint8_t* lineok);

/* Colour schedule of one sparse ICD call (host only; what a BF NHICD call runs with
 * call_schedule = 0).  Same inputs as mbir_level_schedule without the row walk: the call's
 * lines are visited z-major (z, then x ascending) and each takes the smallest colour that no
 * earlier line sharing a touched bin at some view, or lying in its 3x3 (z, x) neighbourhood,
 * holds and that has fewer than class_cap lines (0: no cap; the engine caps classes at the
 * sweep kernel's voxel groups).  Writes the lines colour by colour (z-major within a colour)
 * and the colour offsets;
 * MBIR_EINVAL on bad input, short buffers or more than max_colours (<= 4096) colours.  Replaces
 * no reference interface (the reference draws a random visit order per call,
 * BFReconstructionEngine_Extra.cpp:576-628). */
int32_t mbir_colour_schedule(int32_t n_z, int32_t n_x, int32_t n_theta, int32_t n_r, int32_t nb,
                             int32_t max_colours, int32_t class_cap, const uint8_t* lineok,
                             const uint8_t* active,
                             const int16_t* lo, const uint16_t* mask, int32_t* lines,
                             int32_t lines_cap, int32_t* lofs, int32_t lofs_cap, int32_t* n_lines,
                             int32_t* n_colours);

#ifdef __cplusplus
}
#endif
#endif
