// mbir_engine.h -- host side of the GB300 MBIR engine (C++17).  One Engine = one
// reconstruction resident on one GPU: sinogram, error sinogram, volume and nuisance state
// stay in HBM from prepare() to destruction.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <string>
#include <memory>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/mbir_gb300.h"
#include "mbir_internal.h"
#include "mbir_schedule.h"

namespace mbir {

// Allocator whose value-less construct leaves elements uninitialised: vector::resize without
// zeroing, for host buffers whose every element is written before it is read (the writing
// threads then take the first-touch page faults side by side).
template <typename T>
struct UninitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <typename U>
  UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <typename U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    ::new (static_cast<void*>(p)) U(std::forward<A>(a)...);
  }
};

// Geometry of one resolution level, FP64, as the reference derives it
// (InitialReconstructionInitializer.cpp:98-167, MRCSinogramInitializer.cpp:302-305).
struct Geometry {
  int n_theta = 0, n_r = 0, n_t = 0;
  double delta_r = 1, delta_t = 1, R0 = 0, RMax = 0, T0 = 0, TMax = 0;
  int n_x = 0, n_y = 0, n_z = 0;
  double delta_xz = 1, delta_xy = 1, x0 = 0, y0 = 0, z0 = 0;
  double length_x = 0, length_y = 0, length_z = 0;
  double offset_r = 0, offset_t = 0;
};

// Tables built once per level (FP64, mirrors of the reference's setup).
struct Tables {
  std::vector<double> cosv, sinv;        // [n_theta]
  std::vector<double> H;                 // [n_theta][bins]
  std::vector<double> Ht;                // [bins]
  std::vector<int> t_first, t_count;     // [n_y]
  std::vector<double> hval;              // [n_y][kMaxTRows]
  std::vector<uint8_t> line_nonempty;    // [n_z][n_x]
};

// mt19937 (Matsumoto & Nishimura 1998), the generator behind the reference's boost::mt19937.
class MT19937 {
 public:
  explicit MT19937(uint32_t seed) { this->seed(seed); }
  void seed(uint32_t s);
  uint32_t next();

 private:
  uint32_t mt_[624];
  int idx_ = 624;
};

// visit order of UpdateYSlice::execute (HAADF_ReconstructionEngine_UpdateVoxels.cpp:151-241)
void reference_visit_order(uint32_t seed, int n_z, int n_x, std::vector<int32_t>& out);

class Engine {
 public:
  explicit Engine(const mbir_params& p);
  ~Engine();

  int set_sinogram(const float* counts, const float* tilts_deg, int n_theta, int n_r, int n_t,
                   double delta_r, double delta_t);
  int load_mrc(const char* path);
  int set_initial_volume_f64(const double* vol, int64_t n);
  // HAADF: after every inner iteration the volume as <dir>/<outer>_<inner>_ReconstructedVolume.rec
  int set_intermediate_dir(const char* dir);
  int set_observer(mbir_observer_fn fn, void* user);
  // checkpoint of a HAADF run and its exact resume (the reference's .bin files + Checkpoint.bin)
  int write_checkpoint(const char* dir);
  int read_checkpoint(const char* dir);
  void notify(const std::string& msg, int progress, int aspect) const;
  void notify_iteration(int outer) const;  // one JSON line per completed outer iteration
  int write_volume_mrc(const std::string& path);
  template <typename T>
  int set_initial_volume_t(const T* vol, int64_t n);
  int get_volume_f64(double* out, int64_t n);
  int read_mrc_series(const char* path, std::vector<float>& counts, std::vector<float>& tilts,
                      int& n_theta, int& n_r, int& n_t, double& dr, bool need_tilts);
  // HAADF with bright-field data (initializeBrightFieldData): a bright-field tilt series of the
  // sinogram's size, [theta][r][t]; before prepare
  int set_bright_field(const float* counts, int n_theta, int n_r, int n_t);
  int load_bright_field_mrc(const char* path);
  bool bright_field_assisted() const { return !bfm_.empty(); }
  DevBF bfa_sweep_args() const;
  int bfa_offsets();
  int set_initial_volume(const float* vol, int64_t n);
  int set_initial_nuisance(const double* g, const double* o, const double* v);
  int dims(int32_t* d) const;

  int prepare();
  int sweep(int outer, int inner, double* stats4);
  int joint_estimation();
  int update_weights();
  int compute_cost(double* parts3, double* total);
  int forward_project();
  int run();

  int get_volume(float* out, int64_t n);
  int get_error(float* out, int64_t n);
  int get_projection(float* out, int64_t n);
  int get_nuisance(double* g, double* o, double* v);
  int get_tables(double* H, double* Ht);
  int get_schedule(int sweep, int32_t* row_order, int32_t* stride);
  // lines (z*n_x+x) of the last sweep/call in visit order (reference order) or ascending
  int get_call_lines(int32_t* lines, int32_t cap, int32_t* n) const;
  // the last scheduled call's lines level by level (colour classes or levels) and offsets
  int get_call_schedule(int32_t* lines, int32_t cap, int32_t* lofs, int32_t lofs_cap,
                        int32_t* n_lines, int32_t* n_levels) const;
  // first footprint bin and nonzero mask per (line, view) of the FP32 A-column, line flags
  int get_footprint_bins(int16_t* lo, uint16_t* mask, uint8_t* lineok) const;
  // bright field: selector [theta][r][t], weights [theta][r][t], magnitude map [z][x],
  // filtered map [z][x], current Bragg threshold (each output optional)
  int get_bf_state(uint8_t* sel, float* w, double* mag, double* filt, double* bragg_t);
  int set_bragg_threshold(double t);
  // y-slab sharding (mbir_shard.cu): sweeps and per-view sums restricted to slices [y0, y1)
  int set_slab(int y0, int y1);
  int slab_rows_owned();

  int sweep_colour(int colour, int outer, int inner, double* stats4);
  int get_planes(int y, int n, float* out);
  int set_planes(int y, int n, const float* in);
  int view_sums(int kind, double* out);
  int apply_nuisance(const double* gain, const double* offset, const double* variance);
  // bright-field slabs: an NHICD call as bf_slab_begin, sweep_colour (0, 1), bf_slab_end, the
  // call's per-line update magnitudes and the offset and variance sums summed over slabs by
  // the host
  int bf_slab_begin(int outer, int inner);
  int bf_slab_magnitudes(unsigned long long* out);  // the call's, fixed point, this slab's part
  int bf_slab_end(const unsigned long long* mag);   // summed over slabs (null: this slab's)
  int bf_slab_sums(int kind, double* out);   // 2: offset sums [theta][2]; 3: variance sums [2]
  int bf_slab_apply(int kind, const double* sums);
  int roi_sums(double* out2);  // ROI magnitude-map sum; ROI volume sum over the slab
  int status(mbir_status* st) const;
  void cancel() { cancel_.store(1); }
  int write_outputs(const char* dir, const char* mrc_path, const char* vtk_path = nullptr,
                    const char* avizo_path = nullptr);

  const char* last_error() const { return err_.c_str(); }
  int fail(int code, const std::string& msg);

  const Geometry& geometry() const { return g_; }

  // Hooks for the batched sweep (mbir_batch.cu).  batch_args fills the sweep arguments of this
  // engine's next parallel-order sweep (uploading its row order) and reports the shared memory
  // a staged slice needs; batch_finish records a sweep that ran inside a batch.
  int batch_args(int outer, int inner, SweepArgs* out, size_t* smem_needed);
  int batch_finish(int outer, int inner, const double* st4, double ms);
  double* slice_stats() const { return d_stats_; }
  double* sweep_stats() const { return d_stat4_; }
  int* error_word() const { return d_err_; }
  int nb() const { return nb_; }
  bool fp64() const { return fp64_ != 0; }
  const mbir_params& params() const { return p_; }
  int state() const { return state_; }
  int sweeps_done() const { return sweeps_done_; }
  int check_errors() { return check_device_error(); }

 private:
  // bright field (mbir_engine_bf.cu)
  int bf_prepare_host();                          // -log counts, master line list
  int bf_upload();                                // y, weights, selector, maps
  int bf_call_begin(int outer, int inner, DevBF* out);  // list, active mask, magnitude reset
  int bf_call_end();                              // magnitude map, counters
  int bf_call(int outer, int inner, double* stats4);
  int bf_joint_estimation();
  int bf_update_weights();
  int bf_compute_cost(double* parts3, double* total);
  int bf_run();
  int bf_roi_sum(int kind, double* out);
  int bf_prepare_schedule();                      // A-column table for level-scheduled calls
  int host_footprint_bins();                      // acol_lo_, acol_mask_ (once, on demand)
  int bf_schedule(const std::vector<int32_t>& rows, SweepArgs& a);  // the call's levels
  void bf_schedule_readback();                    // queue the device schedule's copy to host
  void bf_schedule_settle();                      // after the stream synchronised
  BfSino bf_sino() const;
  BfSino bf_sino_rows(int t0, int t1) const;      // detector rows [t0, t1) only
  void slab_rows(int* t0, int* t1) const;         // detector rows of the slab's slices
  int bf_parallel_args(int iter_nonzero, const DevBF& bfa, SweepArgs* a, size_t* smem);
  double bf_default_offset() const;

  int autotune_shape();  // pick the fastest voxel-group shape on a snapshot of the state
  int build_host();  // geometry, tables, stride, initial nuisance: no GPU needed
  int build_geometry();
  int build_tables();
  int compute_stride();
  int init_nuisance_host();
  int alloc_device();
  int upload_views();  // (gain, weight) pairs and mu/gain doubles
  int check_device_error();
  void row_order_for_sweep(int sweep, std::vector<int32_t>& order) const;
  ExactArgs exact_args();
  int cuda_check(int code, const char* what);
  void release();
  void add_kernel_time();

  mbir_params p_;
  std::string err_;
  std::atomic<int> cancel_{0};
  int state_ = 0;
  bool host_ready_ = false;

  // host inputs
  std::vector<float> counts_;     // [theta][r][t]
  std::vector<double> bfm_;       // [theta][r][t] bright-field count + BF_OFFSET (assisted HAADF)
  std::string interm_dir_;        // per-iteration MRC volumes (empty: none)
  mbir_observer_fn observer_ = nullptr;  // progress and error messages (null: none)
  // checkpoints: where the run stands, and the state read_checkpoint hands to every prepare
  int outer_next_ = 0;    // outer iterations mbir_run has completed
  double stop_now_ = 0;   // the stop threshold after its reductions
  bool resume_ = false;
  int resume_outer_ = 0, resume_sweeps_ = 0;
  double resume_stop_ = 0;
  std::vector<unsigned char> resume_e_;  // the error sinogram in its device layout
  std::vector<double> resume_gain_, resume_offset_, resume_var_;
  void* observer_user_ = nullptr;
  std::vector<double> tilts_;     // degrees
  std::vector<double> init_vol_;  // optional [z][x][y]
  std::vector<double> user_gain_, user_offset_, user_var_;

  Geometry g_;
  Tables tab_;
  int bins_ = 64;
  int nb_ = 3;        // candidate bins per view (2*half_width + 1)
  int n_rp_ = 0;      // HBM row stride
  int n_rs_ = 0;      // shared-memory row stride
  int n_sp_ = 0;      // bright-field selector row stride (bytes, multiple of 16)
  int shape_ = 0;     // FP32 voxel-group shape in use (mbir_params.lane_shape)
  bool bf_ = false;   // bright-field modality
  int t_rows_ = 1;    // max t rows per voxel slice
  int stride_ = 2;    // conflict-free x stride
  bool stage_ = true; // slice fits in shared memory
  size_t smem_bytes_ = 0;
  size_t smem_sched_bytes_ = 0;  // scheduled bright-field calls
  DevFilter flt_{};
  DevGeom dg_{};

  // nuisance state (FP64, host copy is authoritative)
  std::vector<double> I_, mu_, alpha_, w_;
  std::vector<double> init_gain_, init_offset_, init_var_;

  // device buffers; "Real" arrays hold float (FP32 engine) or double (FP64 engine)
  int fp64_ = 0;
  size_t rb_ = 4;             // bytes per Real
  void* d_y_ = nullptr;       // Real [n_t][n_theta][n_rp]
  void* d_e_ = nullptr;
  void* d_yest_ = nullptr;
  void* d_x_ = nullptr;       // Real [n_y][n_z][n_x]
  float* d_stage_ = nullptr;  // host-layout staging buffer for transposes (float)
  void* d_H_ = nullptr;       // Real [n_theta][bins+1]
  float2* d_bx_ = nullptr;
  double* d_bxd_ = nullptr;
  double* d_u0_ = nullptr;
  double* d_bz_ = nullptr;
  void* d_gw_ = nullptr;      // Real2 [n_theta]
  int* d_tfirst_ = nullptr;
  int* d_tcount_ = nullptr;
  void* d_hval_ = nullptr;    // Real [n_y][kMaxTRows]
  int* d_rows_ = nullptr;
  uint8_t* d_lineok_ = nullptr;
  // reference-exact mode (FP64 + reference order)
  bool exact_ = false;
  double* d_cosv_ = nullptr;
  double* d_sinv_ = nullptr;
  double* d_Href_ = nullptr;
  int* d_lines_ = nullptr;
  double* d_stats_ = nullptr;   // [max slices][4]
  double* d_stat4_ = nullptr;   // [4]
  double* d_mu_ = nullptr;      // [n_theta]
  double* d_gain_ = nullptr;
  double* d_mu2_ = nullptr;
  double* d_gain2_ = nullptr;
  double* d_wv_ = nullptr;
  double* d_partial_ = nullptr; // view sums partials
  double* d_vsum_ = nullptr;    // [n_theta*6]
  int* d_err_ = nullptr;
  void* stream_ = nullptr;
  void* ev0_ = nullptr;
  void* ev1_ = nullptr;
  void* ev2_ = nullptr;   // around the colour launches of a sweep/call
  void* ev3_ = nullptr;
  bool kernel_timed_ = false;
  void* ev4_ = nullptr;   // around the colour-schedule launches of a BF call
  void* ev5_ = nullptr;
  bool colour_timed_ = false;
  double colour_ms_ = 0;
  double kernel_ms_ = 0.0;  // device time of the sweep kernels alone
  int n_chunk_ = 8;
  int prior_blocks_ = 152 * 4;

  // progress
  int sweeps_done_ = 0;
  int outer_ = 0, inner_ = 0;
  double last_cost_ = 0.0 / 0.0;
  double last_rel_ = 0.0;
  double icd_ms_ = 0.0;
  double total_ms_ = 0.0;
  int64_t visited_ = 0, updated_ = 0;
  int64_t footprint_entries_ = 0;

  // bright-field state
  void* d_w_ = nullptr;                     // Real [n_t][n_theta][n_rp] weights
  void* d_bfm_ = nullptr;                   // Real [n_t][n_theta][n_rp] bright-field factor m
  uint8_t* d_sel_ = nullptr;                // [n_t][n_theta][n_sp] Bragg selector
  unsigned long long* d_magfx_ = nullptr;   // [n_z][n_x] fixed-point magnitudes of a call
  double* d_mag_ = nullptr;                 // [n_z][n_x] update-magnitude map
  double* d_filt_ = nullptr;                // [n_z][n_x] VSC-filtered map
  uint8_t* d_active_ = nullptr;             // [n_z][n_x] lines of the current call
  double* d_bfpart_ = nullptr;              // reduction partials
  double* d_bfout_ = nullptr;               // reduction results
  double* d_alpha_ = nullptr;               // [n_theta] variance per view
  double* d_stage64_ = nullptr;             // FP64 host-layout staging
  std::vector<double, UninitAlloc<double>> ylog_;  // -log(counts + bf_offset), [theta][r][t]
  std::vector<int32_t> bf_master_;          // random permutation of all lines
  std::vector<int32_t> call_lines_;         // lines of the last sweep/call
  std::vector<uint8_t> active_host_;
  uint32_t bf_listsel_ = 0, bf_eff_ = 0;
  int slab_y0_ = 0, slab_y1_ = 0;           // 0, 0: the whole volume
  bool slab_call_open_ = false;             // a bright-field slab call between begin and end
  SweepArgs slab_args_{};
  size_t slab_smem_ = 0;
  int bf_calls_ = 0;
  double bragg_t_ = 0;

  // level-scheduled calls (FP32, parallel order, NHICD): A-column table on the device, its
  // bins on the host, the call's schedule
  float4* d_acol_ = nullptr;                // [n_z*n_x][n_theta][acol_width(nb)]
  std::vector<int16_t> acol_lo_;            // [n_z*n_x][n_theta]
  std::vector<uint16_t> acol_mask_;         // [n_z*n_x][n_theta]
  int* d_sched_ = nullptr;                  // [n_z*n_x] lines level by level
  int* d_lofs_ = nullptr;                   // [n_z*n_x + 1] level offsets
  int n_levels_ = 0;                        // levels of the last scheduled call
  double sched_ms_ = 0;                     // host time spent building schedules
  LevelScheduleWork sched_work_;
  std::vector<int32_t> sched_lines_, sched_lofs_;
  // device colour schedule (call_schedule 0)
  int32_t* d_packed_ = nullptr;             // [n_z*n_x][n_theta] (first bin << 16) | mask
  int32_t* d_vis_ = nullptr;                // [n_z*n_x] the call's lines, ascending
  unsigned* d_conf_ = nullptr;              // [n_z*n_x] conflict words
  std::vector<int32_t> vis_host_;
  int16_t* d_colour_ = nullptr;             // [n_z*n_x] scratch
  unsigned long long* d_bin_used_ = nullptr;   // [n_theta][n_r][cwords_]
  unsigned long long* d_line_used_ = nullptr;  // [n_z*n_x][cwords_]
  unsigned long long* d_cfsets_ = nullptr;  // [ceil(n_z*n_x/31)*31][cwords_] (multi-CTA)
  int* d_cflags_ = nullptr;                 // [3*ceil(n_z*n_x/31) + 1] (multi-CTA)
  int32_t* d_sched_count_ = nullptr;        // [2] lines, colours
  bool sched_on_device_ = false;            // the last call's schedule was built on the device
  bool readback_pending_ = false;
  int32_t sched_count_host_[2] = {0, 0};
  // colour words per bin / line of the device colouring (64 colours each): 8 while a call's
  // lines (1/20 of the lines) fit 4096, 16 (1024 colours) above that
  int cwords_ = 16;
  // colour schedules of the homogeneous sub-lists, which repeat every 20 calls: built once
  int cur_hslot_ = -1;                      // sub-list of the current call, -1: not homogeneous
  int32_t* d_hc_lines_ = nullptr;           // [n_z*n_x] slot k at its sub-list's offset
  int32_t* d_hc_lofs_ = nullptr;            // [20][lofs_cap()]
  int32_t* d_hc_count_ = nullptr;           // [20][2]
  std::vector<char> hc_valid_;
  std::vector<int> hc_start_;
  const int32_t* rb_lines_ = nullptr;       // the current call's schedule (for the read-back)
  const int32_t* rb_lofs_ = nullptr;
  const int32_t* rb_count_ = nullptr;
  size_t lofs_cap() const;
};

// GenRandList's permutation (Common/VoxelUpdateList.cpp:157-215) drawn from mt19937 through
// boost's uniform_int(0, n-1): element i of a list goes to position out[i].
void rand_list_perm(uint32_t seed, int n, std::vector<int32_t>& out);

// Host set-up loops: fn(begin, end) over [0, n) in contiguous chunks on up to 16 host threads
// (the caller's included).  One region runs threaded at a time per process; a region that starts
// while another runs (engines prepared side by side) runs on its caller's thread.  fn must
// write only its own range's outputs, so results do not depend on the split.
inline std::atomic<int>& host_parallel_busy() {
  static std::atomic<int> busy{0};
  return busy;
}
template <typename F>
void host_parallel(int n, F fn) {
  if (n <= 0) return;
  const int hw = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
  const int nt = std::min(n, std::min(hw, 16));
  int idle = 0;
  if (nt <= 1 || !host_parallel_busy().compare_exchange_strong(idle, 1)) {
    fn(0, n);
    return;
  }
  // the busy flag is released however this returns; threads that could not be created leave
  // their ranges to the calling thread, and the threads already started are always joined
  struct Release {
    ~Release() { host_parallel_busy().store(0); }
  } release;
  const int chunk = (n + nt - 1) / nt;
  std::vector<std::thread> pool;
  pool.reserve(nt - 1);
  int next = chunk;  // first index not handed to a thread
  for (int t = 1; t < nt; ++t) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    try {
      pool.emplace_back(fn, b, e);
    } catch (...) {
      break;  // thread limit reached: run the rest here
    }
    next = e;
  }
  struct Join {
    std::vector<std::thread>& p;
    ~Join() {
      for (auto& th : p)
        if (th.joinable()) th.join();
    }
  } join{pool};
  fn(0, std::min(n, chunk));
  if (next < n) fn(next, n);
}

// MRC I/O (mrc_io.cpp)
struct MrcVolume {
  int nx = 0, ny = 0, nz = 0, mode = 0;
  bool has_fei = false;
  std::vector<float> a_tilt, b_tilt, pixel_size;  // per section from the FEI extended header
  std::vector<float> data;                         // sub-volume as float, [z][y][x]
};
int mrc_read(const std::string& path, const int* vmin, const int* vmax, MrcVolume& out,
             bool header_only, std::string& err);
int mrc_write_volume(const std::string& path, const float* zxy, int n_z, int n_x, int n_y,
                     int x_start, int x_end, double length_x, std::string& err);
int estimate_sigma_x(const std::string& path, double thickness, double target_gain,
                     bool use_bf_offset, double bf_offset, const float* tilts, int n_tilts,
                     const int* xd, const int* yd, double* out, std::string& err);
int vtk_write_volume(const std::string& path, const float* zxy, int n_z, int n_x, int n_y,
                     int x_start, int x_end, std::string& err);
int avizo_write_volume(const std::string& path, const float* zxy, int n_z, int n_x, int n_y,
                       int x_start, int x_end, double delta_xy, double delta_xz,
                       std::string& err);

}  // namespace mbir
