// mbir_bf.cu -- bright-field sinogram-wide kernels (compiled with -fmad=false).
//
//   layout_from_double   host-layout FP64 staging [theta][r][t] -> device [t][theta][r_pad]
//   offset sums / apply  BFForwardModel::jointEstimation (BFForwardModel.cpp:390-441): per view
//                        the offset (log dosage) step num/den, e -= step
//   selector             BFForwardModel::updateSelector (:517-531): sel = e^2 w < T^2
//   variance sums        BFForwardModel::updateWeights (:447-511): w *= alpha_view, then the
//                        global sums over selected (e^2 w) and rejected (|e| sqrt(alpha w))
//                        entries; scale_weights then divides by the new common variance
//   cost sums            BFForwardModel::forwardCost (:812-846), data term
//   magnitude map        per-line sum |dx| of a call (fixed point -> FP64), the 5x5 Hamming
//                        VSC filter (BFReconstructionEngine_Extra.cpp:888-947), the NHICD
//                        list mask (GenNonHomList :1016-1047) and the stop-rule ROI sums
//                        (roiVolumeSum :1200-1215, stopCriteria :1239-1248)
//
// Each reduction has a parallel form (fixed-shape tree: deterministic, not the reference's
// order) and a reference-order form (one thread, the reference's loop order) used by the
// reference-exact mode; without fused multiply-adds the latter reproduce the reference's FP64
// arithmetic.  Elementwise passes are the same in both modes.
#include <cuda_runtime.h>

#include "mbir_internal.h"

namespace mbir {

namespace {

constexpr int kRedBlocks = 152 * 4;  // grid of the global parallel reductions

inline int ok_or(cudaError_t e) { return e == cudaSuccess ? 0 : -3; }
inline int grid_for(size_t n, int block) {
  size_t g = (n + block - 1) / block;
  if (g > 152 * 32) g = 152 * 32;
  if (g < 1) g = 1;
  return static_cast<int>(g);
}
template <typename Real>
inline Real* RP(void* p) {
  return static_cast<Real*>(p);
}
template <typename Real>
inline const Real* RP(const void* p) {
  return static_cast<const Real*>(p);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of K values (blockDim.x a multiple of 32, <= 1024); result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum(double (&acc)[K]) {
  __shared__ double red[32][K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const double s = warp_sum_d(acc[k]);
    if (lane == 0) red[warp][k] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0.0;
      for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w][k];
      acc[k] = s;
    }
  }
}

template <typename Real>
__global__ void layout_from_double_kernel(const double* __restrict__ h, Real* __restrict__ d,
                                          int n_theta, int n_r, int n_rp, int n_t) {
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

// one offset-sum term (BFForwardModel.cpp:405-420)
__device__ __forceinline__ void offset_term(double ev, double w, bool sel, double T, double dl,
                                            double& num, double& den) {
  if (sel) {
    num += (ev * w);
    den += w;
  } else {
    num += (T * dl * ev / fabs(ev)) * sqrt(w);
    den += ((T * dl * sqrt(w)) / fabs(ev));
  }
}

template <typename Real>
__global__ void offset_sums_kernel(const Real* __restrict__ e, const Real* __restrict__ w,
                                   const uint8_t* __restrict__ sel, double T, double dl,
                                   int n_theta, int n_rp, int n_sp, int n_r, int n_t, int n_chunk,
                                   double* __restrict__ partial) {
  const int v = blockIdx.x, ch = blockIdx.y;
  const int t0 = static_cast<int>(static_cast<long long>(ch) * n_t / n_chunk);
  const int t1 = static_cast<int>(static_cast<long long>(ch + 1) * n_t / n_chunk);
  double acc[2] = {0.0, 0.0};
  for (int t = t0; t < t1; ++t) {
    const size_t base = (static_cast<size_t>(t) * n_theta + v) * n_rp;
    const size_t sb = (static_cast<size_t>(t) * n_theta + v) * n_sp;
    for (int r = threadIdx.x; r < n_r; r += blockDim.x)
      offset_term(e[base + r], w[base + r], sel[sb + r] == 1, T, dl, acc[0], acc[1]);
  }
  block_sum<2>(acc);
  if (threadIdx.x == 0) {
    partial[(static_cast<size_t>(v) * n_chunk + ch) * 2 + 0] = acc[0];
    partial[(static_cast<size_t>(v) * n_chunk + ch) * 2 + 1] = acc[1];
  }
}

__global__ void chunk_final_kernel(const double* __restrict__ partial, double* __restrict__ out,
                                   int n_theta, int n_chunk, int K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_theta * K) return;
  const int v = i / K, k = i % K;
  double s = 0.0;
  for (int c = 0; c < n_chunk; ++c) s += partial[(static_cast<size_t>(v) * n_chunk + c) * K + k];
  out[i] = s;
}

// reference order: one thread per view, r then t
template <typename Real>
__global__ void offset_sums_ref_kernel(const Real* __restrict__ e, const Real* __restrict__ w,
                                       const uint8_t* __restrict__ sel, double T, double dl,
                                       int n_theta, int n_rp, int n_sp, int n_r, int n_t,
                                       double* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_theta) return;
  double num = 0, den = 0;
  for (int r = 0; r < n_r; r++)
    for (int t = 0; t < n_t; t++) {
      const size_t i = (static_cast<size_t>(t) * n_theta + v) * n_rp + r;
      const size_t si = (static_cast<size_t>(t) * n_theta + v) * n_sp + r;
      offset_term(e[i], w[i], sel[si] == 1, T, dl, num, den);
    }
  out[v * 2 + 0] = num;
  out[v * 2 + 1] = den;
}

template <typename Real>
__global__ void offset_apply_kernel(Real* __restrict__ e, const double* __restrict__ step,
                                    int n_theta, int n_rp, int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    if (r >= n_r) continue;
    const int v = static_cast<int>((i / n_rp) % n_theta);
    e[i] = static_cast<Real>(static_cast<double>(e[i]) - step[v]);
  }
}

template <typename Real>
__global__ void selector_kernel(const Real* __restrict__ e, const Real* __restrict__ w,
                                uint8_t* __restrict__ sel, double T, int n_theta, int n_rp,
                                int n_sp, int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_sp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_sp);
    if (r >= n_r) continue;
    const size_t row = i / n_sp;
    const size_t k = row * n_rp + r;
    const double ev = e[k];
    sel[i] = (ev * ev * static_cast<double>(w[k]) < T * T) ? 1 : 0;
  }
}

// one variance-sum term (BFForwardModel.cpp:470-480); w already multiplied by alpha_view
__device__ __forceinline__ void variance_term(double ev, double w, double a, bool sel,
                                              double& s1, double& s2) {
  if (sel)
    s1 += (ev * ev * w);
  else
    s2 += fabs(ev) * sqrt(a * w);
}

template <typename Real>
__global__ void variance_sums_kernel(const Real* __restrict__ e, Real* __restrict__ w,
                                     const uint8_t* __restrict__ sel,
                                     const double* __restrict__ alpha, int n_theta, int n_rp,
                                     int n_sp, int n_r, int n_t, double* __restrict__ partial) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  double acc[2] = {0.0, 0.0};
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    if (r >= n_r) continue;
    const size_t row = i / n_rp;
    const int v = static_cast<int>(row % n_theta);
    const double a = alpha[v];
    const Real wn = static_cast<Real>(static_cast<double>(w[i]) * a);
    w[i] = wn;
    variance_term(e[i], wn, a, sel[row * n_sp + r] == 1, acc[0], acc[1]);
  }
  block_sum<2>(acc);
  if (threadIdx.x == 0) {
    partial[blockIdx.x * 2 + 0] = acc[0];
    partial[blockIdx.x * 2 + 1] = acc[1];
  }
}

__global__ void blocks_final_kernel(const double* __restrict__ partial, double* __restrict__ out,
                                    int n_blocks, int K) {
  const int k = threadIdx.x;
  if (k >= K) return;
  double s = 0.0;
  for (int b = 0; b < n_blocks; ++b) s += partial[b * K + k];
  out[k] = s;
}

// reference order (one thread): first w *= alpha everywhere, then theta, r, t sums
template <typename Real>
__global__ void variance_sums_ref_kernel(const Real* __restrict__ e, Real* __restrict__ w,
                                         const uint8_t* __restrict__ sel,
                                         const double* __restrict__ alpha, int n_theta, int n_rp,
                                         int n_sp, int n_r, int n_t, double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int th = 0; th < n_theta; th++)
    for (int r = 0; r < n_r; r++)
      for (int t = 0; t < n_t; t++) {
        const size_t i = (static_cast<size_t>(t) * n_theta + th) * n_rp + r;
        w[i] = static_cast<Real>(static_cast<double>(w[i]) * alpha[th]);
      }
  double s1 = 0, s2 = 0;
  for (int th = 0; th < n_theta; th++)
    for (int r = 0; r < n_r; r++)
      for (int t = 0; t < n_t; t++) {
        const size_t i = (static_cast<size_t>(t) * n_theta + th) * n_rp + r;
        const size_t si = (static_cast<size_t>(t) * n_theta + th) * n_sp + r;
        variance_term(e[i], w[i], alpha[th], sel[si] == 1, s1, s2);
      }
  out[0] = s1;
  out[1] = s2;
}

template <typename Real>
__global__ void scale_weights_kernel(Real* __restrict__ w, double alpha, int n_theta, int n_rp,
                                     int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    if (r >= n_r) continue;
    w[i] = static_cast<Real>(static_cast<double>(w[i]) / alpha);
  }
}

// one data-term entry of forwardCost (BFForwardModel.cpp:822-830)
__device__ __forceinline__ double cost_term(double ev, double w, bool sel, double T, double dl) {
  if (sel) return (ev * ev * w);
  return (2 * T * dl * fabs(ev) * sqrt(w) + T * T * (1 - 2 * dl));
}

template <typename Real>
__global__ void cost_sums_kernel(const Real* __restrict__ e, const Real* __restrict__ w,
                                 const uint8_t* __restrict__ sel, double T, double dl, int n_theta,
                                 int n_rp, int n_sp, int n_r, int n_t,
                                 double* __restrict__ partial) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  double acc[1] = {0.0};
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    if (r >= n_r) continue;
    const size_t row = i / n_rp;
    acc[0] += cost_term(e[i], w[i], sel[row * n_sp + r] == 1, T, dl);
  }
  block_sum<1>(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
}

template <typename Real>
__global__ void cost_sums_ref_kernel(const Real* __restrict__ e, const Real* __restrict__ w,
                                     const uint8_t* __restrict__ sel, double T, double dl,
                                     int n_theta, int n_rp, int n_sp, int n_r, int n_t,
                                     double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double c = 0;
  for (int th = 0; th < n_theta; th++)
    for (int r = 0; r < n_r; r++)
      for (int t = 0; t < n_t; t++) {
        const size_t i = (static_cast<size_t>(t) * n_theta + th) * n_rp + r;
        const size_t si = (static_cast<size_t>(t) * n_theta + th) * n_sp + r;
        c += cost_term(e[i], w[i], sel[si] == 1, T, dl);
      }
  out[0] = c;
}

__global__ void mag_reset_kernel(unsigned long long* __restrict__ fx,
                                 const uint8_t* __restrict__ active, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && active[i]) fx[i] = 0ull;
}

__global__ void mag_update_kernel(const unsigned long long* __restrict__ fx,
                                  const uint8_t* __restrict__ active, double* __restrict__ mag,
                                  int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && active[i]) mag[i] = static_cast<double>(fx[i]) / kFixScale;
}

// 5x5 Hamming window of BFReconstructionEngine.cpp:157-185
__constant__ double c_hamming[5][5] = {{0.0013, 0.0086, 0.0159, 0.0086, 0.0013},
                                       {0.0086, 0.0581, 0.1076, 0.0581, 0.0086},
                                       {0.0159, 0.1076, 0.1993, 0.1076, 0.0159},
                                       {0.0086, 0.0581, 0.1076, 0.0581, 0.0086},
                                       {0.0013, 0.0086, 0.0159, 0.0086, 0.0013}};

__global__ void vsc_kernel(const double* __restrict__ mag, double* __restrict__ filt, int n_z,
                           int n_x) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_z * n_x) return;
  const int i = idx / n_x, j = idx % n_x;
  double f = 0;
  for (int p = -2; p <= 2; p++)
    for (int q = -2; q <= 2; q++)
      if (i + p >= 0 && i + p < n_z && j + q >= 0 && j + q < n_x)
        f += c_hamming[p + 2][q + 2] * mag[static_cast<size_t>(i + p) * n_x + (j + q)];
  filt[idx] = f;
}

__global__ void nh_mask_kernel(const double* __restrict__ filt, double thr,
                               uint8_t* __restrict__ active, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) active[i] = filt[i] > thr ? 1 : 0;
}

// ROI sums: kind 0 = sum of the magnitude map over ROI lines, kind 1 = sum of the volume over
// ROI lines and all y.  The ROI is the index box [x0,x1] x [z0,z1].
template <typename Real>
__global__ void roi_sums_kernel(const DevGeom g, int kind, const double* __restrict__ mag,
                                const Real* __restrict__ x, double* __restrict__ partial) {
  const size_t nl = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t total = kind == 0 ? nl : nl * g.n_y;
  double acc[1] = {0.0};
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t l = i % nl;
    const int z = static_cast<int>(l / g.n_x), xx = static_cast<int>(l % g.n_x);
    if (xx < g.roi_x0 || xx > g.roi_x1 || z < g.roi_z0 || z > g.roi_z1) continue;
    acc[0] += kind == 0 ? mag[l] : static_cast<double>(x[i]);  // x: [y][z][x]
  }
  block_sum<1>(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc[0];
}

template <typename Real>
__global__ void roi_sums_ref_kernel(const DevGeom g, int kind, const double* __restrict__ mag,
                                    const Real* __restrict__ x, double* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0;
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  for (int j = 0; j < g.n_z; j++)
    for (int k = 0; k < g.n_x; k++) {
      if (k < g.roi_x0 || k > g.roi_x1 || j < g.roi_z0 || j > g.roi_z1) continue;
      if (kind == 0) {
        s += mag[static_cast<size_t>(j) * g.n_x + k];
      } else {
        for (int i = 0; i < g.n_y; i++)
          s += static_cast<double>(x[static_cast<size_t>(i) * plane + static_cast<size_t>(j) * g.n_x + k]);
      }
    }
  out[0] = s;
}

}  // namespace

int launch_layout_from_double(const double* h, void* d, int n_theta, int n_r, int n_rp, int n_t,
                              int fp64, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (fp64)
    layout_from_double_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(h, RP<double>(d), n_theta,
                                                                        n_r, n_rp, n_t);
  else
    layout_from_double_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(h, RP<float>(d), n_theta,
                                                                       n_r, n_rp, n_t);
  return ok_or(cudaGetLastError());
}

int launch_bf_offset_sums(const BfSino& b, int exact, double T, double dl, double* partial,
                          int n_chunk, double* out, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (exact) {
    const int grid = (b.n_theta + 63) / 64;
    if (b.fp64)
      offset_sums_ref_kernel<double><<<grid, 64, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel, T,
                                                         dl, b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t,
                                                         out);
    else
      offset_sums_ref_kernel<float><<<grid, 64, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel, T, dl,
                                                        b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t, out);
    return ok_or(cudaGetLastError());
  }
  const dim3 grid(b.n_theta, n_chunk);
  if (b.fp64)
    offset_sums_kernel<double><<<grid, 256, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel, T, dl,
                                                    b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t, n_chunk,
                                                    partial);
  else
    offset_sums_kernel<float><<<grid, 256, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel, T, dl,
                                                   b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t, n_chunk,
                                                   partial);
  const int n = b.n_theta * 2;
  chunk_final_kernel<<<(n + 127) / 128, 128, 0, s>>>(partial, out, b.n_theta, n_chunk, 2);
  return ok_or(cudaGetLastError());
}

int launch_bf_offset_apply(const BfSino& b, const double* step, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = static_cast<size_t>(b.n_t) * b.n_theta * b.n_rp;
  if (b.fp64)
    offset_apply_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(RP<double>(b.e), step, b.n_theta,
                                                                 b.n_rp, b.n_r, b.n_t);
  else
    offset_apply_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(RP<float>(b.e), step, b.n_theta,
                                                                b.n_rp, b.n_r, b.n_t);
  return ok_or(cudaGetLastError());
}

int launch_bf_selector(const BfSino& b, double T, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = static_cast<size_t>(b.n_t) * b.n_theta * b.n_sp;
  if (b.fp64)
    selector_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel,
                                                             T, b.n_theta, b.n_rp, b.n_sp, b.n_r,
                                                             b.n_t);
  else
    selector_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel, T,
                                                            b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t);
  return ok_or(cudaGetLastError());
}

int launch_bf_variance_sums(const BfSino& b, int exact, const double* alpha, double* partial,
                            double* out, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (exact) {
    if (b.fp64)
      variance_sums_ref_kernel<double><<<1, 32, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel,
                                                        alpha, b.n_theta, b.n_rp, b.n_sp, b.n_r,
                                                        b.n_t, out);
    else
      variance_sums_ref_kernel<float><<<1, 32, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel, alpha,
                                                       b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t, out);
    return ok_or(cudaGetLastError());
  }
  if (b.fp64)
    variance_sums_kernel<double><<<kRedBlocks, 256, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel,
                                                            alpha, b.n_theta, b.n_rp, b.n_sp, b.n_r,
                                                            b.n_t, partial);
  else
    variance_sums_kernel<float><<<kRedBlocks, 256, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel,
                                                           alpha, b.n_theta, b.n_rp, b.n_sp, b.n_r,
                                                           b.n_t, partial);
  blocks_final_kernel<<<1, 32, 0, s>>>(partial, out, kRedBlocks, 2);
  return ok_or(cudaGetLastError());
}

int launch_bf_scale_weights(const BfSino& b, double alpha, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = static_cast<size_t>(b.n_t) * b.n_theta * b.n_rp;
  if (b.fp64)
    scale_weights_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(RP<double>(b.w), alpha, b.n_theta,
                                                                  b.n_rp, b.n_r, b.n_t);
  else
    scale_weights_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(RP<float>(b.w), alpha, b.n_theta,
                                                                 b.n_rp, b.n_r, b.n_t);
  return ok_or(cudaGetLastError());
}

int launch_bf_cost_sums(const BfSino& b, int exact, double T, double dl, double* partial,
                        double* out, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (exact) {
    if (b.fp64)
      cost_sums_ref_kernel<double><<<1, 32, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel, T, dl,
                                                    b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t, out);
    else
      cost_sums_ref_kernel<float><<<1, 32, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel, T, dl,
                                                   b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t, out);
    return ok_or(cudaGetLastError());
  }
  if (b.fp64)
    cost_sums_kernel<double><<<kRedBlocks, 256, 0, s>>>(RP<double>(b.e), RP<double>(b.w), b.sel, T,
                                                        dl, b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t,
                                                        partial);
  else
    cost_sums_kernel<float><<<kRedBlocks, 256, 0, s>>>(RP<float>(b.e), RP<float>(b.w), b.sel, T, dl,
                                                       b.n_theta, b.n_rp, b.n_sp, b.n_r, b.n_t,
                                                       partial);
  blocks_final_kernel<<<1, 32, 0, s>>>(partial, out, kRedBlocks, 1);
  return ok_or(cudaGetLastError());
}

int launch_bf_mag_reset(unsigned long long* fx, const uint8_t* active, int n, void* stream) {
  mag_reset_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(fx, active, n);
  return ok_or(cudaGetLastError());
}

int launch_bf_mag_update(const unsigned long long* fx, const uint8_t* active, double* mag, int n,
                         void* stream) {
  mag_update_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(fx, active,
                                                                                   mag, n);
  return ok_or(cudaGetLastError());
}

int launch_bf_vsc(const double* mag, double* filt, int n_z, int n_x, void* stream) {
  const int n = n_z * n_x;
  vsc_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(mag, filt, n_z, n_x);
  return ok_or(cudaGetLastError());
}

int launch_bf_nh_mask(const double* filt, double thr, uint8_t* active, int n, void* stream) {
  nh_mask_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(filt, thr, active,
                                                                                n);
  return ok_or(cudaGetLastError());
}

int launch_roi_sum(const DevGeom& g, int exact, int kind, const double* mag, const void* x,
                   int fp64, double* partial, double* out, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (exact) {
    if (fp64)
      roi_sums_ref_kernel<double><<<1, 32, 0, s>>>(g, kind, mag, RP<double>(x), out);
    else
      roi_sums_ref_kernel<float><<<1, 32, 0, s>>>(g, kind, mag, RP<float>(x), out);
    return ok_or(cudaGetLastError());
  }
  if (fp64)
    roi_sums_kernel<double><<<kRedBlocks, 256, 0, s>>>(g, kind, mag, RP<double>(x), partial);
  else
    roi_sums_kernel<float><<<kRedBlocks, 256, 0, s>>>(g, kind, mag, RP<float>(x), partial);
  blocks_final_kernel<<<1, 32, 0, s>>>(partial, out, kRedBlocks, 1);
  return ok_or(cudaGetLastError());
}

}  // namespace mbir
