// mbir_noalloc.cu -- per-view sums of squared errors on caller-owned device buffers, with no
// allocation of any kind.
//
// Callers that cannot allocate: a host framework that owns every byte of device memory through
// its own pool (and forbids cudaMalloc/cudaFree while it streams, since those synchronise the
// device and fragment its pool), or a latency-bound pipeline that must not pay an allocation on
// the path.  For them mbir_error_view_sums_noalloc computes, per view, the sum over r and t of
// e^2 (the sums a per-view noise-variance update divides by N_r N_t) from an error sinogram
// they already hold on the device, writing into an output buffer they own.
//
// The only scratch is the file-scope array below (kMaxViews x kChunks doubles, 128 KiB):
// per-(view, chunk) partial sums.  Every slot read in a call is written earlier in the same
// call, so nothing has to start at zero.  The scratch is shared by all calls on a device:
// calls that overlap in time (different streams, or different host threads without ordering)
// race on it and must be serialised by the caller.
//
// The first call on a device (with that device current) looks the scratch's address up with
// cudaGetSymbolAddress; that set-up can load the module, so make the first call before any
// stream capture.  Later calls only launch two kernels on the caller's stream.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mbir_gb300.h"

namespace {

constexpr int kMaxViews = 1024;  // largest n_theta accepted
constexpr int kChunks = 16;      // partial sums per view
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_view_partial[kMaxViews * kChunks];

std::mutex g_setup_mu;
double* g_partial_ptr[kMaxDevices] = {nullptr};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block (view v, chunk c): sum of e^2 over entries [c*len/kChunks, (c+1)*len/kChunks) of the
// view's contiguous n_r*n_t block ([theta][r][t] layout)
__global__ void view_sq_partial_kernel(const float* __restrict__ e, int n_rt,
                                       double* __restrict__ partial) {
  const int v = blockIdx.x, c = blockIdx.y;
  const long long b = static_cast<long long>(c) * n_rt / kChunks;
  const long long end = static_cast<long long>(c + 1) * n_rt / kChunks;
  const float* ev = e + static_cast<size_t>(v) * n_rt;
  double acc = 0.0;
  for (long long i = b + threadIdx.x; i < end; i += blockDim.x) {
    const double x = ev[i];
    acc += x * x;
  }
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  acc = warp_sum(acc);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) s += red[w];
    partial[v * kChunks + c] = s;
  }
}

__global__ void view_sq_final_kernel(const double* __restrict__ partial, int n_theta,
                                     double* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n_theta) return;
  double s = 0.0;
  for (int c = 0; c < kChunks; ++c) s += partial[v * kChunks + c];
  out[v] = s;
}

// once per device, with that device current
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MBIR_EDEVICE;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (g_partial_ptr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_view_partial) != cudaSuccess || p == nullptr)
      return MBIR_EDEVICE;
    g_partial_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_partial_ptr[dev];
  return MBIR_OK;
}

}  // namespace

extern "C" int32_t mbir_error_view_sums_noalloc(const float* error_dev, int32_t n_theta,
                                                int32_t n_r, int32_t n_t, double* sums_dev,
                                                void* stream) {
  if (error_dev == nullptr || sums_dev == nullptr || n_theta <= 0 || n_r <= 0 || n_t <= 0)
    return MBIR_EINVAL;
  if (n_theta > kMaxViews) return MBIR_EINVAL;  // scratch holds kMaxViews views
  if (static_cast<long long>(n_r) * n_t > 0x7fffffffLL) return MBIR_EINVAL;
  double* partial = nullptr;
  const int rc = scratch_for_current_device(&partial);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Each launch's own status is returned by cudaLaunchKernel; cudaGetLastError would also
  // return (and clear) an earlier, unrelated error of the caller's and report it as ours.
  int n_rt = n_r * n_t;
  void* a1[] = {const_cast<float**>(&error_dev), &n_rt, &partial};
  if (cudaLaunchKernel(reinterpret_cast<const void*>(view_sq_partial_kernel),
                       dim3(n_theta, kChunks), dim3(256), a1, 0, s) != cudaSuccess)
    return MBIR_EDEVICE;
  int nt = n_theta;
  void* a2[] = {&partial, &nt, &sums_dev};
  if (cudaLaunchKernel(reinterpret_cast<const void*>(view_sq_final_kernel),
                       dim3((n_theta + 127) / 128), dim3(128), a2, 0, s) != cudaSuccess)
    return MBIR_EDEVICE;
  return MBIR_OK;
}
