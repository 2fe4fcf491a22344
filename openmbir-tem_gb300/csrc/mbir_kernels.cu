// mbir_kernels.cu -- sm_103a kernels of the MBIR hot path.
//
// The ICD sweep / projection kernels live in mbir_sweep.cuh (instantiated by
// mbir_sweep_f32.cu, mbir_sweep_f32_hbm.cu and mbir_sweep_f64.cu).  This file holds the rest:
//   view_sums_kernel  FP64 per-view reductions for gain/offset and variance estimation.
//   prior_cost_kernel FP64 accumulation of the QGGMRF prior term of the MAP cost.
// Every kernel is instantiated for Real = float (production) and Real = double (the
// reference's own precision, for order-exact parity and precision studies).
//
// Reference semantics follow Code/MBIRLib/HAADF/HAADF_ReconstructionEngine_UpdateVoxels.cpp
// (UpdateYSlice::execute :149-484), Code/MBIRLib/Common/AMatrixCol.cpp:82-239 (A-column),
// Code/MBIRLib/Reconstruction/QGGMRF_Functions.cpp:82-206 (prior), and
// HAADF_ReconstructionEngine_Extra.cpp:419-881 / HAADF_ReconstructionEngine.cpp:1147-1364.
#include <cuda_runtime.h>

#include <type_traits>

#include "mbir_internal.h"

namespace mbir {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier polls before giving up

template <typename Real>
struct V2;
template <>
struct V2<float> {
  using type = float2;
};
template <>
struct V2<double> {
  using type = double2;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- TMA bulk-copy helpers (cp.async.bulk + mbarrier) ------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
               "r"(smem_u32(src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// ---- warp reductions ------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(kFull, v, o);
    v = w < v ? w : v;
  }
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(kFull, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// ---- layout conversions ----------------------------------------------------------------
template <typename Real>
__global__ void sino_to_dev_kernel(const float* __restrict__ h, Real* __restrict__ d, int n_theta,
                                   int n_r, int n_rp, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const size_t rest = i / n_rp;
    const int v = static_cast<int>(rest % n_theta);
    const int t = static_cast<int>(rest / n_theta);
    d[i] = (r < n_r) ? static_cast<Real>(h[(static_cast<size_t>(v) * n_r + r) * n_t + t]) : Real(0);
  }
}
template <typename Real>
__global__ void sino_to_host_kernel(const Real* __restrict__ d, float* __restrict__ h, int n_theta,
                                    int n_r, int n_rp, int n_t) {
  const size_t total = static_cast<size_t>(n_theta) * n_r * n_t;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int t = static_cast<int>(i % n_t);
    const size_t rest = i / n_t;
    const int r = static_cast<int>(rest % n_r);
    const int v = static_cast<int>(rest / n_r);
    h[i] = static_cast<float>(d[(static_cast<size_t>(t) * n_theta + v) * n_rp + r]);
  }
}
template <typename Real>
__global__ void vol_to_dev_kernel(const float* __restrict__ zxy, Real* __restrict__ yzx, int n_z,
                                  int n_x, int n_y) {
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % n_x);
    const size_t rest = i / n_x;
    const int z = static_cast<int>(rest % n_z);
    const int y = static_cast<int>(rest / n_z);
    yzx[i] = static_cast<Real>(zxy[(static_cast<size_t>(z) * n_x + x) * n_y + y]);
  }
}
template <typename Real>
__global__ void vol64_to_dev_kernel(const double* __restrict__ zxy, Real* __restrict__ yzx,
                                    int n_z, int n_x, int n_y) {
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % n_x);
    const size_t rest = i / n_x;
    const int z = static_cast<int>(rest % n_z);
    const int y = static_cast<int>(rest / n_z);
    yzx[i] = static_cast<Real>(zxy[(static_cast<size_t>(z) * n_x + x) * n_y + y]);
  }
}
template <typename Real>
__global__ void vol_to_host_kernel(const Real* __restrict__ yzx, float* __restrict__ zxy, int n_z,
                                   int n_x, int n_y) {
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(i % n_y);
    const size_t rest = i / n_y;
    const int x = static_cast<int>(rest % n_x);
    const int z = static_cast<int>(rest / n_x);
    zxy[i] = static_cast<float>(yzx[(static_cast<size_t>(y) * n_z + z) * n_x + x]);
  }
}

// e = y - yest - mu_theta (calculateMeasurementWeight, HAADF_ReconstructionEngine_Extra.cpp:693-771)
template <typename Real>
__global__ void error_from_projection_kernel(const Real* __restrict__ y,
                                             const Real* __restrict__ yest, Real* __restrict__ e,
                                             const double* __restrict__ mu, int n_theta, int n_rp,
                                             int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const int v = static_cast<int>((i / n_rp) % n_theta);
    e[i] = (r < n_r) ? static_cast<Real>(static_cast<double>(y[i]) -
                                         static_cast<double>(yest[i]) - mu[v])
                     : Real(0);
  }
}

// Per-view FP64 sums.  kind 0 (jointEstimation, HAADF_ReconstructionEngine_Extra.cpp:474-517):
//   [0] sum y w, [1] sum w, [2] sum yh w, [3] sum yh w y, [4] sum y^2 w, [5] sum yh^2 w,
//   yh = (y - e - mu)/I.  kind 1 (updateWeights :825-833): [0] sum e^2.
template <typename Real, int K>
__global__ void view_sums_kernel(const Real* __restrict__ y, const Real* __restrict__ e,
                                 const double* __restrict__ mu, const double* __restrict__ gain,
                                 const double* __restrict__ wv, double* __restrict__ partial,
                                 int n_theta, int n_rp, int n_r, int t_begin, int t_end,
                                 int n_chunk) {
  const int v = blockIdx.x, ch = blockIdx.y;
  const int n_t = t_end - t_begin;
  const int t0 = t_begin + static_cast<int>(static_cast<long long>(ch) * n_t / n_chunk);
  const int t1 = t_begin + static_cast<int>(static_cast<long long>(ch + 1) * n_t / n_chunk);
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  const double m = mu[v], gi = gain[v], w = wv[v];
  for (int t = t0; t < t1; ++t) {
    const size_t base = (static_cast<size_t>(t) * n_theta + v) * n_rp;
    for (int r = threadIdx.x; r < n_r; r += blockDim.x) {
      const double ev = e[base + r];
      if (K == 1) {
        acc[0] += ev * ev;
      } else {
        const double yv = y[base + r];
        const double yh = (yv - ev - m) / gi;
        acc[0] += yv * w;
        acc[1] += w;
        acc[2] += yh * w;
        acc[K > 3 ? 3 : 0] += yh * w * yv;
        acc[K > 4 ? 4 : 0] += yv * yv * w;
        acc[K > 5 ? 5 : 0] += yh * yh * w;
      }
    }
  }
  __shared__ double red[32][K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double s = warp_sum(acc[k]);
    if (lane == 0) red[warp][k] = s;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int w2 = 0; w2 < static_cast<int>(blockDim.x >> 5); ++w2) s += red[w2][threadIdx.x];
    partial[(static_cast<size_t>(v) * n_chunk + ch) * K + threadIdx.x] = s;
  }
}

__global__ void view_sums_final_kernel(const double* __restrict__ partial, double* __restrict__ out,
                                       int n_theta, int n_chunk, int K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_theta * K) return;
  const int v = i / K, k = i % K;
  double s = 0.0;
  for (int c = 0; c < n_chunk; ++c) s += partial[(static_cast<size_t>(v) * n_chunk + c) * K + k];
  out[i] = s;
}

// e = y - mu_new - I_new * yh, yh = (y - e - mu_old)/I_old
// (jointEstimation, HAADF_ReconstructionEngine_Extra.cpp:464-472 and :600-612)
template <typename Real>
__global__ void rebuild_error_kernel(const Real* __restrict__ y, Real* __restrict__ e,
                                     const double* __restrict__ mu_old,
                                     const double* __restrict__ gain_old,
                                     const double* __restrict__ mu_new,
                                     const double* __restrict__ gain_new, int n_theta, int n_rp,
                                     int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    if (r >= n_r) continue;
    const int v = static_cast<int>((i / n_rp) % n_theta);
    const double yv = y[i];
    const double yh = (yv - static_cast<double>(e[i]) - mu_old[v]) / gain_old[v];
    // the product is rounded on its own (no fused multiply-subtract), as in the reference
    e[i] = static_cast<Real>(yv - mu_new[v] - __dmul_rn(gain_new[v], yh));
  }
}

// QGGMRF prior term of computeCost (HAADF_ReconstructionEngine.cpp:1285-1359): 13 forward
// neighbours per voxel, FP64 accumulation.  Offsets are (dz, dx, dy) with weight index
// [dy+1][dz+1][dx+1].
__constant__ int c_fwd[13][3] = {{0, 0, 1},  {0, 1, -1}, {0, 1, 0},   {0, 1, 1},   {1, -1, 0},
                                 {1, 0, 0},  {1, 1, 0},  {1, -1, -1}, {1, -1, 1},  {1, 0, -1},
                                 {1, 1, -1}, {1, 1, 1},  {1, 0, 1}};

template <typename Real>
__global__ void prior_cost_kernel(const Real* __restrict__ x, DevFilter q, int n_z, int n_x,
                                  int n_y, double* __restrict__ partial) {
  // one (y, z) row of n_x voxels at a time: 32-bit index arithmetic, coalesced row reads
  const int rows = n_y * n_z;
  constexpr bool kF32 = std::is_same<Real, float>::value;
  // FP32 engine: each voxel's 13 pair terms in FP32 (relative error ~1e-6 of the term),
  // summed per voxel and accumulated in FP64; FP64 engine: FP64 throughout
  const float P = static_cast<float>(q.mrf_p), PQ = static_cast<float>(q.mrf_p - q.mrf_q);
  const float isp = static_cast<float>(1.0 / q.sig_p), ispq = static_cast<float>(1.0 / q.sig_pq);
  const float cc = static_cast<float>(q.mrf_c);
  const bool p2 = q.mrf_p == 2.0;
  double acc = 0.0;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int yi = r / n_z, zi = r - yi * n_z;
    const Real* row = x + static_cast<size_t>(r) * n_x;
    for (int xi = threadIdx.x; xi < n_x; xi += blockDim.x) {
      const Real c = row[xi];
      float vsum = 0.f;
      for (int k = 0; k < 13; ++k) {
        const int zz = zi + c_fwd[k][0], xx = xi + c_fwd[k][1], yy = yi + c_fwd[k][2];
        if (zz < 0 || zz >= n_z || xx < 0 || xx >= n_x || yy < 0 || yy >= n_y) continue;
        const Real nv = x[(static_cast<size_t>(yy) * n_z + zz) * n_x + xx];
        const int fi = 9 * (c_fwd[k][2] + 1) + 3 * (c_fwd[k][0] + 1) + (c_fwd[k][1] + 1);
        if constexpr (kF32) {
          const float ad = fabsf(c - nv);
          const float num = p2 ? ad * ad : powf(ad, P);
          const float pq = powf(ad, PQ);
          vsum += static_cast<float>(q.f[fi]) * ((num * isp) / (cc + pq * ispq));
        } else {
          const double ad = fabs(static_cast<double>(c) - static_cast<double>(nv));
          const double num = pow(ad, q.mrf_p);
          const double pq = pow(ad, q.mrf_p - q.mrf_q);
          acc += q.f[fi] * ((num / q.sig_p) / (q.mrf_c + pq / q.sig_pq));
        }
      }
      if constexpr (kF32) acc += static_cast<double>(vsum);
    }
  }
  acc = warp_sum(acc);
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void reduce_rows_kernel(const double* __restrict__ in, int n_rows, int n_cols,
                                   double* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= n_cols) return;
  double s = 0.0;
  for (int r = 0; r < n_rows; ++r) s += in[static_cast<size_t>(r) * n_cols + c];
  out[c] = s;
}

inline int ok_or(cudaError_t e) { return e == cudaSuccess ? 0 : -3; }
inline int grid_for(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  if (g < 1) g = 1;
  return static_cast<int>(g);
}

}  // namespace

int launch_sweep_f32_smem(const SweepArgs& a, int nb, size_t smem, void* stream) {
  return a.bf ? launch_sweep_f32_smem_bf(a, nb, smem, stream)
              : launch_sweep_f32_smem_haadf(a, nb, smem, stream);
}

int launch_batch_sweep(const BatchArgs& b, int nb, int group, int threads, size_t smem, int grid,
                       void* stream) {
  if (nb == 3) return launch_batch_sweep_nb3(b, group, threads, smem, grid, stream);
  if (nb == 5) return launch_batch_sweep_nb5(b, group, threads, smem, grid, stream);
  return -7;
}

int launch_sweep(const SweepArgs& a, int nb, size_t smem, void* stream) {
  if (a.fp64) return launch_sweep_f64(a, nb, smem, stream);
  return a.smem_rows ? launch_sweep_f32_smem(a, nb, smem, stream)
                     : launch_sweep_f32_hbm(a, nb, smem, stream);
}

int launch_ref_order(const RefOrderArgs& a, int nb, void* stream) {
  return a.fp64 ? launch_ref_order_f64(a, nb, stream) : launch_ref_order_f32(a, nb, stream);
}

template <typename Real>
static inline Real* RP(void* p) {
  return static_cast<Real*>(p);
}
template <typename Real>
static inline const Real* RP(const void* p) {
  return static_cast<const Real*>(p);
}

int launch_sino_to_dev(const float* h, void* d, int n_theta, int n_r, int n_rp, int n_t, int fp64,
                       void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    sino_to_dev_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(h, RP<double>(d), n_theta, n_r,
                                                                 n_rp, n_t);
  else
    sino_to_dev_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(h, RP<float>(d), n_theta, n_r,
                                                                n_rp, n_t);
  return ok_or(cudaGetLastError());
}
int launch_sino_to_host(const void* d, float* h, int n_theta, int n_r, int n_rp, int n_t,
                        int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_theta) * n_r * n_t;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    sino_to_host_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(RP<double>(d), h, n_theta, n_r,
                                                                  n_rp, n_t);
  else
    sino_to_host_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(RP<float>(d), h, n_theta, n_r,
                                                                 n_rp, n_t);
  return ok_or(cudaGetLastError());
}
int launch_vol_to_dev(const float* zxy, void* yzx, int n_z, int n_x, int n_y, int fp64,
                      void* stream) {
  const size_t n = static_cast<size_t>(n_z) * n_x * n_y;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    vol_to_dev_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(zxy, RP<double>(yzx), n_z, n_x, n_y);
  else
    vol_to_dev_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(zxy, RP<float>(yzx), n_z, n_x, n_y);
  return ok_or(cudaGetLastError());
}
int launch_vol64_to_dev(const double* zxy, void* yzx, int n_z, int n_x, int n_y, int fp64,
                        void* stream) {
  const size_t n = static_cast<size_t>(n_z) * n_x * n_y;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    vol64_to_dev_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(zxy, RP<double>(yzx), n_z, n_x,
                                                                  n_y);
  else
    vol64_to_dev_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(zxy, RP<float>(yzx), n_z, n_x, n_y);
  return ok_or(cudaGetLastError());
}
int launch_vol_to_host(const void* yzx, float* zxy, int n_z, int n_x, int n_y, int fp64,
                       void* stream) {
  const size_t n = static_cast<size_t>(n_z) * n_x * n_y;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    vol_to_host_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(RP<double>(yzx), zxy, n_z, n_x, n_y);
  else
    vol_to_host_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(RP<float>(yzx), zxy, n_z, n_x, n_y);
  return ok_or(cudaGetLastError());
}
int launch_error_from_projection(const void* y, const void* yest, void* e, const double* mu,
                                 int n_theta, int n_rp, int n_r, int n_t, int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    error_from_projection_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(
        RP<double>(y), RP<double>(yest), RP<double>(e), mu, n_theta, n_rp, n_r, n_t);
  else
    error_from_projection_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(
        RP<float>(y), RP<float>(yest), RP<float>(e), mu, n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}
int launch_view_sums(int kind, const void* y, const void* e, const double* mu,
                     const double* gain, const double* wv, double* partial, double* out,
                     int n_theta, int n_rp, int n_r, int n_t, int n_chunk, int fp64,
                     void* stream) {
  return launch_view_sums_rows(kind, y, e, mu, gain, wv, partial, out, n_theta, n_rp, n_r, 0, n_t,
                               n_chunk, fp64, stream);
}

int launch_view_sums_rows(int kind, const void* y, const void* e, const double* mu,
                          const double* gain, const double* wv, double* partial, double* out,
                          int n_theta, int n_rp, int n_r, int t_begin, int t_end, int n_chunk,
                          int fp64, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid(n_theta, n_chunk);
  const int K = kind == 0 ? 6 : 1;
  if (fp64) {
    if (kind == 0)
      view_sums_kernel<double, 6><<<grid, 256, 0, s>>>(RP<double>(y), RP<double>(e), mu, gain, wv,
                                                        partial, n_theta, n_rp, n_r, t_begin, t_end, n_chunk);
    else
      view_sums_kernel<double, 1><<<grid, 256, 0, s>>>(RP<double>(y), RP<double>(e), mu, gain, wv,
                                                        partial, n_theta, n_rp, n_r, t_begin, t_end, n_chunk);
  } else {
    if (kind == 0)
      view_sums_kernel<float, 6><<<grid, 256, 0, s>>>(RP<float>(y), RP<float>(e), mu, gain, wv,
                                                       partial, n_theta, n_rp, n_r, t_begin, t_end, n_chunk);
    else
      view_sums_kernel<float, 1><<<grid, 256, 0, s>>>(RP<float>(y), RP<float>(e), mu, gain, wv,
                                                       partial, n_theta, n_rp, n_r, t_begin, t_end, n_chunk);
  }
  const int n = n_theta * K;
  view_sums_final_kernel<<<(n + 127) / 128, 128, 0, s>>>(partial, out, n_theta, n_chunk, K);
  return ok_or(cudaGetLastError());
}
int launch_rebuild_error(const void* y, void* e, const double* mu_old, const double* gain_old,
                         const double* mu_new, const double* gain_new, int n_theta, int n_rp,
                         int n_r, int n_t, int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    rebuild_error_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(
        RP<double>(y), RP<double>(e), mu_old, gain_old, mu_new, gain_new, n_theta, n_rp, n_r, n_t);
  else
    rebuild_error_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(
        RP<float>(y), RP<float>(e), mu_old, gain_old, mu_new, gain_new, n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}
int launch_prior_cost(const void* x, const DevFilter& f, int n_z, int n_x, int n_y,
                      double* partial, int n_blocks, int fp64, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    prior_cost_kernel<double><<<n_blocks, 256, 0, s>>>(RP<double>(x), f, n_z, n_x, n_y, partial);
  else
    prior_cost_kernel<float><<<n_blocks, 256, 0, s>>>(RP<float>(x), f, n_z, n_x, n_y, partial);
  return ok_or(cudaGetLastError());
}
int launch_reduce_stats(const double* in, int n_rows, int n_cols, double* out, void* stream) {
  reduce_rows_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(in, n_rows, n_cols, out);
  return ok_or(cudaGetLastError());
}

}  // namespace mbir
