// mbir_bfassist.cu -- HAADF reconstruction with bright-field data, the parallel engines' passes.
//
// With a bright-field tilt series of the same size (initializeBrightFieldData,
// HAADF_ReconstructionEngine_Extra.cpp:84-176) every HAADF measurement carries a factor
// m = bright-field count + BF_OFFSET: the error is y - m Y_Est - mu (:718-727), a footprint entry
// of the voxel update enters theta1/theta2 multiplied by m (_UpdateVoxels.cpp:354-364), the
// scatter subtracts m times the update (:438-446), and jointEstimation estimates the offsets
// only (:429, :643-668).  The parallel engines run this model through the bright-field sweep
// (per-entry weights, selector always on) on scaled variables: e' = e / m and w' = m^2 w.  Then
// theta2 = sum (pe m)^2 w = sum pe^2 w', theta1 = sum e (pe m) w = sum e' pe w', and the
// scatter e -= m k is e' -= k: the sweep's own arithmetic.  The passes here build e' and w',
// sum m e' and (m e')^2 per view (offsets, variance, cost) and apply an offset step to e'.
// The reference-exact mode keeps e itself (mbir_exact.cu).
#include <cuda_runtime.h>

#include "mbir_internal.h"

namespace mbir {
namespace {

inline int ok_or(cudaError_t e) { return e == cudaSuccess ? 0 : -3; }
inline int grid_for(size_t n, int block) {
  const size_t g = (n + block - 1) / block;
  return static_cast<int>(g < 152 * 32 ? g : 152 * 32);
}

template <typename Real>
__global__ void bfa_error_kernel(const Real* __restrict__ y, const Real* __restrict__ yest,
                                 const Real* __restrict__ m, Real* __restrict__ e,
                                 const double* __restrict__ mu, int n_theta, int n_rp, int n_r,
                                 int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const int v = static_cast<int>((i / n_rp) % n_theta);
    if (r < n_r) {
      const double mi = m[i];
      e[i] = static_cast<Real>((static_cast<double>(y[i]) - mi * static_cast<double>(yest[i]) -
                                mu[v]) / mi);
    } else {
      e[i] = Real(0);
    }
  }
}

template <typename Real>
__global__ void bfa_weight_kernel(const Real* __restrict__ m, const double* __restrict__ wv,
                                  Real* __restrict__ w, int n_theta, int n_rp, int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const int v = static_cast<int>((i / n_rp) % n_theta);
    const double mi = m[i];
    w[i] = (r < n_r) ? static_cast<Real>(mi * mi * wv[v]) : Real(0);
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// per view and t-chunk: sum of m e' (kind 0) or (m e')^2 (kind 1), FP64, fixed shape
template <typename Real>
__global__ void bfa_sums_kernel(const Real* __restrict__ m, const Real* __restrict__ e,
                                double* __restrict__ partial, int n_theta, int n_rp, int n_r,
                                int n_t, int n_chunk, int kind) {
  const int v = blockIdx.x, ch = blockIdx.y;
  const int t0 = static_cast<int>(static_cast<long long>(ch) * n_t / n_chunk);
  const int t1 = static_cast<int>(static_cast<long long>(ch + 1) * n_t / n_chunk);
  double acc = 0.0;
  for (int t = t0; t < t1; ++t) {
    const size_t base = (static_cast<size_t>(t) * n_theta + v) * n_rp;
    for (int r = threadIdx.x; r < n_r; r += blockDim.x) {
      const double d = static_cast<double>(m[base + r]) * static_cast<double>(e[base + r]);
      acc += kind == 0 ? d : d * d;
    }
  }
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  acc = warp_sum_d(acc);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w2 = 0; w2 < static_cast<int>(blockDim.x >> 5); ++w2) s += red[w2];
    partial[static_cast<size_t>(v) * n_chunk + ch] = s;
  }
}

__global__ void bfa_sums_final_kernel(const double* __restrict__ partial, double* __restrict__ out,
                                      int n_theta, int n_chunk) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_theta) return;
  double s = 0.0;
  for (int c = 0; c < n_chunk; ++c) s += partial[static_cast<size_t>(v) * n_chunk + c];
  out[v] = s;
}

template <typename Real>
__global__ void bfa_offset_apply_kernel(const Real* __restrict__ m, Real* __restrict__ e,
                                        const double* __restrict__ step, int n_theta, int n_rp,
                                        int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const int v = static_cast<int>((i / n_rp) % n_theta);
    if (r < n_r)
      e[i] = static_cast<Real>(static_cast<double>(e[i]) - step[v] / static_cast<double>(m[i]));
  }
}

template <typename Real>
const Real* CR(const void* p) {
  return static_cast<const Real*>(p);
}
template <typename Real>
Real* WR(void* p) {
  return static_cast<Real*>(p);
}

}  // namespace

int launch_bfa_error(const void* y, const void* yest, const void* m, void* e, const double* mu,
                     int n_theta, int n_rp, int n_r, int n_t, int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    bfa_error_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(
        CR<double>(y), CR<double>(yest), CR<double>(m), WR<double>(e), mu, n_theta, n_rp, n_r, n_t);
  else
    bfa_error_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(
        CR<float>(y), CR<float>(yest), CR<float>(m), WR<float>(e), mu, n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}

int launch_bfa_weights(const void* m, const double* wv, void* w, int n_theta, int n_rp, int n_r,
                       int n_t, int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    bfa_weight_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(CR<double>(m), wv, WR<double>(w),
                                                               n_theta, n_rp, n_r, n_t);
  else
    bfa_weight_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(CR<float>(m), wv, WR<float>(w),
                                                              n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}

int launch_bfa_sums(int kind, const void* m, const void* e, double* partial, double* out,
                    int n_theta, int n_rp, int n_r, int n_t, int n_chunk, int fp64, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid(n_theta, n_chunk);
  if (fp64)
    bfa_sums_kernel<double><<<grid, 256, 0, s>>>(CR<double>(m), CR<double>(e), partial, n_theta,
                                                 n_rp, n_r, n_t, n_chunk, kind);
  else
    bfa_sums_kernel<float><<<grid, 256, 0, s>>>(CR<float>(m), CR<float>(e), partial, n_theta,
                                                n_rp, n_r, n_t, n_chunk, kind);
  bfa_sums_final_kernel<<<(n_theta + 127) / 128, 128, 0, s>>>(partial, out, n_theta, n_chunk);
  return ok_or(cudaGetLastError());
}

int launch_bfa_offset_apply(const void* m, void* e, const double* step, int n_theta, int n_rp,
                            int n_r, int n_t, int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    bfa_offset_apply_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(
        CR<double>(m), WR<double>(e), step, n_theta, n_rp, n_r, n_t);
  else
    bfa_offset_apply_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(
        CR<float>(m), WR<float>(e), step, n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}

}  // namespace mbir
