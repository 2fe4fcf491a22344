// mbir_kernels.cu -- sm_103a kernels of the MBIR hot path.
//
//   sweep_kernel      ICD sweep (and forward projection) over the voxel slices of one y-colour.
//                     One CTA owns one voxel slice y: the detector rows t of that slice (all
//                     views, all r) are staged into shared memory with TMA bulk copies and stay
//                     there for the whole sweep, so every theta1/theta2 gather and every
//                     error-sinogram scatter is an on-chip access.  Inside the slice, warps
//                     update voxels of one z-row whose A-columns do not overlap (x stride S),
//                     so the result is the sequential ICD of a fixed visit order.  Each warp
//                     builds its voxel's A-column on the fly (lanes over views), reduces
//                     theta1/theta2 with warp shuffles and solves the QGGMRF surrogate with one
//                     neighbour per lane.
//   ref_order_kernel  the reference's visit order (one voxel line after another, y in order)
//                     with the error sinogram in HBM; one warp, used for order-exact parity.
//   view_sums_kernel  FP64 per-view reductions for gain/offset and variance estimation.
//   prior_cost_kernel FP64 accumulation of the QGGMRF prior term of the MAP cost.
//
// Reference semantics follow Code/MBIRLib/HAADF/HAADF_ReconstructionEngine_UpdateVoxels.cpp
// (UpdateYSlice::execute :149-484), Code/MBIRLib/Common/AMatrixCol.cpp:82-239 (A-column),
// Code/MBIRLib/Reconstruction/QGGMRF_Functions.cpp:82-206 (prior), and
// HAADF_ReconstructionEngine_Extra.cpp:419-881 / HAADF_ReconstructionEngine.cpp:1147-1364.
#include <cuda_runtime.h>

#include "mbir_internal.h"

namespace mbir {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier polls before giving up

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
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Detector coordinate of a voxel row at one view, split as integer + fraction so that the
// per-voxel position keeps ~1e-7 bin accuracy in FP32.
struct RowBase {
  int ib;
  float fb;
};

// u = j0 + f (f in [0,1)) for voxel column x: u = base(z) + x * bx with bx given as hi+lo.
__device__ __forceinline__ void detector_pos(int x, RowBase rb, float2 bx, int& j0, float& f) {
  const float xf = static_cast<float>(x);
  const float p = xf * bx.x;
  const float pe = fmaf(xf, bx.x, -p);  // exact rounding error of x*bx.hi
  const float jp = floorf(p);
  float ff = (p - jp) + rb.fb + (pe + xf * bx.y);
  const float jf = floorf(ff);
  ff -= jf;
  j0 = rb.ib + static_cast<int>(jp) + static_cast<int>(jf);
  f = ff;
}

// A-matrix entries of one voxel at one view (AMatrixCol.cpp:148-232): bins j in
// [floor(u-d), floor(u+d)] on the detector, value = linear interpolation of the detector
// response at |u - (j+0.5)|, kept when > 0.
template <int NB>
__device__ __forceinline__ void view_footprint(const DevGeom& g, const float* __restrict__ hrow,
                                               int j0, float f, int& jlo, float (&a)[NB]) {
  const int lo = j0 + static_cast<int>(floorf(f - g.half_width));
  const int hi = j0 + static_cast<int>(floorf(f + g.half_width));
  jlo = lo;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int j = lo + b;
    float v = 0.f;
    if (j <= hi && j >= 0 && j < g.n_r) {
      const float delta = fabsf(static_cast<float>(j0 - j) + f - 0.5f);
      const float xr = delta * g.kr;
      const int idx = static_cast<int>(xr);
      if (idx < g.bins) {
        const float t = xr - static_cast<float>(idx);
        v = (1.f - t) * hrow[idx] + t * hrow[idx + 1];
      }
    }
    a[b] = v > 0.f ? v : 0.f;
  }
}

// rho'(d)/d of the QGGMRF prior (QGGMRF_Functions.cpp:90-104 divided by d), or rho''(0)
// (:109-112) when d == 0.
__device__ __forceinline__ float qggmrf_coef(const DevFilter& q, float d0) {
  if (d0 == 0.f) return q.mrf_p / (q.sig_p * q.mrf_c);
  const float ad = fabsf(d0);
  const float t1 = powf(ad, q.mrf_p - q.mrf_q) / q.sig_pq;
  const float t3 = q.mrf_c + t1;
  float r = (q.mrf_p - ((q.mrf_p - q.mrf_q) * t1) / t3) / (t3 * q.sig_p);
  if (q.mrf_p != 2.f) r *= powf(ad, q.mrf_p - 2.f);
  return r;
}

// One voxel (z, x, y) processed by one warp.  es points at the first detector row of slice y
// (row stride rs floats between views, plane stride ps between t rows).  Returns in wst
// (lane 0): ROI sum|dx|, ROI sum|x|, zero-skipped, updated.
template <int NB>
__device__ __forceinline__ void voxel_step(const DevGeom& g, const DevFilter& q,
                                           float* __restrict__ vol, float* es, int rs, int ps,
                                           const RowBase* rb, const float* sH,
                                           const float2* sbx, const float2* sgw, int z, int x,
                                           int y, int tcount, const float* hv, int mode,
                                           int iter_nonzero, int zero_skipping, int lane,
                                           double* wst) {
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t vidx = static_cast<size_t>(y) * plane + static_cast<size_t>(z) * g.n_x + x;
  const float V = vol[vidx];

  int jlo[kMaxViewsPerLane];
  float a[kMaxViewsPerLane][NB];
  bool any = false;
#pragma unroll
  for (int i = 0; i < kMaxViewsPerLane; ++i) {
    const int v = lane + 32 * i;
    jlo[i] = 0;
#pragma unroll
    for (int b = 0; b < NB; ++b) a[i][b] = 0.f;
    if (v < g.n_theta) {
      int j0;
      float f;
      detector_pos(x, rb[v], sbx[v], j0, f);
      const float u = static_cast<float>(j0) + f;
      if (!(u + g.half_width < 0.f || u - g.half_width > static_cast<float>(g.n_r))) {
        view_footprint<NB>(g, sH + v * (g.bins + 1), j0, f, jlo[i], a[i]);
#pragma unroll
        for (int b = 0; b < NB; ++b) any |= (a[i][b] > 0.f);
      }
    }
  }
  if (!__any_sync(kFull, any)) return;  // empty A-column: the line is never visited

  if (mode == kModeProject) {
    if (V != 0.f) {
#pragma unroll
      for (int i = 0; i < kMaxViewsPerLane; ++i) {
        const int v = lane + 32 * i;
        if (v >= g.n_theta) continue;
        const float gain = sgw[v].x;
        for (int tr = 0; tr < tcount; ++tr) {
          const float hh = hv[tr];
          float* row = es + tr * ps + v * rs + jlo[i];
#pragma unroll
          for (int b = 0; b < NB; ++b)
            if (a[i][b] > 0.f) row[b] += gain * (a[i][b] * hh * V);
        }
      }
    }
    return;
  }

  // 26-neighbourhood, one neighbour per lane (UpdateVoxels.cpp:283-306)
  float nb = 0.f;
  bool nvalid = false;
  if (lane < 27) {
    const int dy = lane / 9 - 1, dz = (lane / 3) % 3 - 1, dx = lane % 3 - 1;
    const int yy = y + dy, zz = z + dz, xx = x + dx;
    if (lane != 13 && yy >= 0 && yy < g.n_y && zz >= 0 && zz < g.n_z && xx >= 0 && xx < g.n_x) {
      nb = vol[static_cast<size_t>(yy) * plane + static_cast<size_t>(zz) * g.n_x + xx];
      nvalid = true;
    }
  }
  // zero skipping (UpdateVoxels.cpp:310-338)
  if (zero_skipping && iter_nonzero && V == 0.f) {
    if (!__any_sync(kFull, nb > 0.f)) {
      if (lane == 0) wst[2] += 1.0;
      return;
    }
  }
  // theta1 / theta2 (UpdateVoxels.cpp:343-369)
  float t1 = 0.f, t2 = 0.f;
#pragma unroll
  for (int i = 0; i < kMaxViewsPerLane; ++i) {
    const int v = lane + 32 * i;
    if (v >= g.n_theta) continue;
    const float2 gw = sgw[v];
    for (int tr = 0; tr < tcount; ++tr) {
      const float hh = hv[tr];
      const float* row = es + tr * ps + v * rs + jlo[i];
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (a[i][b] > 0.f) {
          const float pe = gw.x * a[i][b] * hh;
          t2 += pe * pe * gw.y;
          t1 += row[b] * pe * gw.y;
        }
      }
    }
  }
  const float theta1 = -warp_sum(t1);
  const float theta2 = warp_sum(t2);
  // bracket (find_min_max, UpdateVoxels.cpp:47-63): over all 27 entries, centre and
  // out-of-range entries count as 0
  float lo = warp_min(nb), hi = warp_max(nb);
  if (theta2 != 0.f) {
    const float cand = V - theta1 / theta2;
    lo = lo > cand ? cand : lo;
    hi = hi < cand ? cand : hi;
  }
  // QGGMRF surrogate, one iteration (QGGMRF_Functions.cpp:153-206)
  float s1 = 0.f, s2 = 0.f;
  if (nvalid) {
    const float tc = q.f[lane] * qggmrf_coef(q, V - nb);
    s1 = tc * nb;
    s2 = tc;
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  const float u = (s1 + theta2 * V - theta1) / (s2 + theta2);
  float nv = V + q.mrf_alpha * (u - V);
  nv = (nv < lo) ? lo : ((nv > hi) ? hi : nv);
  if (nv < 0.f) nv = 0.f;  // positivity (UpdateVoxels.cpp:394-400)
  const float dlt = nv - V;
  // error-sinogram scatter (UpdateVoxels.cpp:423-449)
  if (dlt != 0.f) {
#pragma unroll
    for (int i = 0; i < kMaxViewsPerLane; ++i) {
      const int v = lane + 32 * i;
      if (v >= g.n_theta) continue;
      const float gain = sgw[v].x;
      for (int tr = 0; tr < tcount; ++tr) {
        const float hh = hv[tr];
        float* row = es + tr * ps + v * rs + jlo[i];
#pragma unroll
        for (int b = 0; b < NB; ++b)
          if (a[i][b] > 0.f) row[b] -= gain * (a[i][b] * hh * dlt);
      }
    }
  }
  if (lane == 0) {
    vol[vidx] = nv;
    if (x >= g.roi_x0 && x <= g.roi_x1 && z >= g.roi_z0 && z <= g.roi_z1) {
      wst[0] += fabs(static_cast<double>(dlt));
      wst[1] += fabs(static_cast<double>(V));
    }
    wst[3] += 1.0;
  }
}

__device__ __forceinline__ void compute_row_base(const DevTables& tab, int n_theta, int z,
                                                 RowBase* rb, int tid, int nthreads) {
  for (int v = tid; v < n_theta; v += nthreads) {
    const double b = tab.u0[v] - static_cast<double>(z) * tab.bz[v];
    const double fl = floor(b);
    rb[v].ib = static_cast<int>(fl);
    rb[v].fb = static_cast<float>(b - fl);
  }
}

struct SmemLayout {
  size_t bar, stats, rb, bx, gw, H, hv, es, total;
};

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

__host__ __device__ inline SmemLayout smem_layout(int n_theta, int n_rs, int t_rows, int bins,
                                                  bool stage) {
  SmemLayout L;
  size_t o = 0;
  L.bar = o;
  o += 16;
  L.stats = o;
  o += sizeof(double) * kWarps * kStatSlots;
  L.rb = o;
  o = align_up(o + sizeof(RowBase) * n_theta, 16);
  L.bx = o;
  o = align_up(o + sizeof(float2) * n_theta, 16);
  L.gw = o;
  o = align_up(o + sizeof(float2) * n_theta, 16);
  L.H = o;
  o = align_up(o + sizeof(float) * n_theta * (bins + 1), 16);
  L.hv = o;
  o = align_up(o + sizeof(float) * kMaxTRows, 128);
  L.es = o;
  if (stage) o += sizeof(float) * static_cast<size_t>(t_rows) * n_theta * n_rs;
  L.total = align_up(o, 16);
  return L;
}

template <int NB, bool STAGE>
__global__ void __launch_bounds__(kWarps * 32, 1) sweep_kernel(SweepArgs A) {
  extern __shared__ __align__(128) unsigned char smem[];
  const DevGeom& g = A.g;
  const int y = A.colour + 2 * static_cast<int>(blockIdx.x);
  if (y >= g.n_y) return;
  const int tid = threadIdx.x, nthreads = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int tcount = A.tab.t_count[y], tfirst = A.tab.t_first[y];
  const SmemLayout L = smem_layout(g.n_theta, A.n_rs, tcount, g.bins, STAGE);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L.bar);
  double* sstat = reinterpret_cast<double*>(smem + L.stats);
  RowBase* rb = reinterpret_cast<RowBase*>(smem + L.rb);
  float2* sbx = reinterpret_cast<float2*>(smem + L.bx);
  float2* sgw = reinterpret_cast<float2*>(smem + L.gw);
  float* sH = reinterpret_cast<float*>(smem + L.H);
  float* shv = reinterpret_cast<float*>(smem + L.hv);

  for (int i = tid; i < g.n_theta * (g.bins + 1); i += nthreads) sH[i] = A.tab.H[i];
  for (int v = tid; v < g.n_theta; v += nthreads) {
    sbx[v] = A.tab.bx[v];
    sgw[v] = A.tab.gw[v];
  }
  if (tid < kMaxTRows) shv[tid] = A.tab.hval[y * kMaxTRows + tid];

  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  float* es;
  int rs, ps;
  const int rows = tcount * g.n_theta;
  const uint32_t row_bytes = static_cast<uint32_t>(g.n_rp * sizeof(float));
  if (STAGE) {
    es = reinterpret_cast<float*>(smem + L.es);
    rs = A.n_rs;
    ps = g.n_theta * A.n_rs;
    if (A.mode == kModeProject) {
      for (int i = tid; i < tcount * ps; i += nthreads) es[i] = 0.f;
      __syncthreads();
    } else {
      if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
      }
      __syncthreads();
      if (tid == 0) mbar_expect_tx(bar, static_cast<uint32_t>(rows) * row_bytes);
      __syncthreads();
      for (int r = tid; r < rows; r += nthreads) {
        const int tr = r / g.n_theta, v = r % g.n_theta;
        bulk_g2s(es + tr * ps + v * rs, A.e + (static_cast<size_t>(tfirst + tr)) * sino_plane +
                                            static_cast<size_t>(v) * g.n_rp,
                 row_bytes, bar);
      }
      const bool ok = mbar_wait(bar, 0);
      if (!__syncthreads_and(ok)) {
        if (tid == 0) atomicOr(A.err, 1);
        mbar_wait(bar, 0);  // give copies still in flight a second bounded chance to land
        return;
      }
    }
  } else {
    es = A.e + static_cast<size_t>(tfirst) * sino_plane;
    rs = g.n_rp;
    ps = static_cast<int>(sino_plane);
  }

  double wst[kStatSlots] = {0.0, 0.0, 0.0, 0.0};
  for (int rr = 0; rr < g.n_z; ++rr) {
    const int z = A.row_order[rr];
    __syncthreads();
    compute_row_base(A.tab, g.n_theta, z, rb, tid, nthreads);
    __syncthreads();
    for (int k = 0; k < A.stride; ++k) {
      for (int x = k + A.stride * warp; x < g.n_x; x += A.stride * kWarps)
        voxel_step<NB>(g, A.flt, A.x, es, rs, ps, rb, sH, sbx, sgw, z, x, y, tcount, shv, A.mode,
                       A.iter_nonzero, A.zero_skipping, lane, wst);
      __syncthreads();
    }
  }

  if (STAGE) {
    fence_proxy_async_smem();
    __syncthreads();
    for (int r = tid; r < rows; r += nthreads) {
      const int tr = r / g.n_theta, v = r % g.n_theta;
      bulk_s2g(A.e + (static_cast<size_t>(tfirst + tr)) * sino_plane +
                   static_cast<size_t>(v) * g.n_rp,
               es + tr * ps + v * rs, row_bytes);
    }
    bulk_commit();
    bulk_wait_all();
  }
  if (A.stats != nullptr) {
    if (lane == 0)
      for (int s = 0; s < kStatSlots; ++s) sstat[warp * kStatSlots + s] = wst[s];
    __syncthreads();
    if (tid < kStatSlots) {
      double acc = 0.0;
      for (int w = 0; w < nthreads / 32; ++w) acc += sstat[w * kStatSlots + tid];
      A.stats[static_cast<size_t>(blockIdx.x) * kStatSlots + tid] = acc;
    }
  }
}

template <int NB>
__global__ void __launch_bounds__(32, 1) ref_order_kernel(RefOrderArgs A) {
  extern __shared__ __align__(128) unsigned char smem[];
  const DevGeom& g = A.g;
  const int lane = threadIdx.x;
  const SmemLayout L = smem_layout(g.n_theta, 0, 0, g.bins, false);
  RowBase* rb = reinterpret_cast<RowBase*>(smem + L.rb);
  float2* sbx = reinterpret_cast<float2*>(smem + L.bx);
  float2* sgw = reinterpret_cast<float2*>(smem + L.gw);
  float* sH = reinterpret_cast<float*>(smem + L.H);
  for (int i = lane; i < g.n_theta * (g.bins + 1); i += 32) sH[i] = A.tab.H[i];
  for (int v = lane; v < g.n_theta; v += 32) {
    sbx[v] = A.tab.bx[v];
    sgw[v] = A.tab.gw[v];
  }
  __syncwarp();
  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  double wst[kStatSlots] = {0.0, 0.0, 0.0, 0.0};
  for (int n = 0; n < A.n_lines; ++n) {
    const int l = A.lines[n];
    const int z = l / g.n_x, x = l % g.n_x;
    __syncwarp();
    compute_row_base(A.tab, g.n_theta, z, rb, lane, 32);
    __syncwarp();
    for (int y = 0; y < g.n_y; ++y) {
      float* es = A.e + static_cast<size_t>(A.tab.t_first[y]) * sino_plane;
      voxel_step<NB>(g, A.flt, A.x, es, g.n_rp, static_cast<int>(sino_plane), rb, sH, sbx, sgw,
                     z, x, y, A.tab.t_count[y], A.tab.hval + y * kMaxTRows, kModeICD,
                     A.iter_nonzero, A.zero_skipping, lane, wst);
      __syncwarp();
    }
  }
  if (lane == 0)
    for (int s = 0; s < kStatSlots; ++s) A.stats[s] = wst[s];
}

// ---- layout conversions ----------------------------------------------------------------
__global__ void sino_to_dev_kernel(const float* __restrict__ h, float* __restrict__ d, int n_theta,
                                   int n_r, int n_rp, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const size_t rest = i / n_rp;
    const int v = static_cast<int>(rest % n_theta);
    const int t = static_cast<int>(rest / n_theta);
    d[i] = (r < n_r) ? h[(static_cast<size_t>(v) * n_r + r) * n_t + t] : 0.f;
  }
}
__global__ void sino_to_host_kernel(const float* __restrict__ d, float* __restrict__ h, int n_theta,
                                    int n_r, int n_rp, int n_t) {
  const size_t total = static_cast<size_t>(n_theta) * n_r * n_t;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int t = static_cast<int>(i % n_t);
    const size_t rest = i / n_t;
    const int r = static_cast<int>(rest % n_r);
    const int v = static_cast<int>(rest / n_r);
    h[i] = d[(static_cast<size_t>(t) * n_theta + v) * n_rp + r];
  }
}
__global__ void vol_to_dev_kernel(const float* __restrict__ zxy, float* __restrict__ yzx, int n_z,
                                  int n_x, int n_y) {
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % n_x);
    const size_t rest = i / n_x;
    const int z = static_cast<int>(rest % n_z);
    const int y = static_cast<int>(rest / n_z);
    yzx[i] = zxy[(static_cast<size_t>(z) * n_x + x) * n_y + y];
  }
}
__global__ void vol_to_host_kernel(const float* __restrict__ yzx, float* __restrict__ zxy, int n_z,
                                   int n_x, int n_y) {
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int y = static_cast<int>(i % n_y);
    const size_t rest = i / n_y;
    const int x = static_cast<int>(rest % n_x);
    const int z = static_cast<int>(rest / n_x);
    zxy[i] = yzx[(static_cast<size_t>(y) * n_z + z) * n_x + x];
  }
}

// e = y - yest - mu_theta (calculateMeasurementWeight, HAADF_ReconstructionEngine_Extra.cpp:693-771)
__global__ void error_from_projection_kernel(const float* __restrict__ y,
                                             const float* __restrict__ yest, float* __restrict__ e,
                                             const double* __restrict__ mu, int n_theta, int n_rp,
                                             int n_r, int n_t) {
  const size_t total = static_cast<size_t>(n_t) * n_theta * n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % n_rp);
    const int v = static_cast<int>((i / n_rp) % n_theta);
    e[i] = (r < n_r) ? static_cast<float>(static_cast<double>(y[i]) -
                                          static_cast<double>(yest[i]) - mu[v])
                     : 0.f;
  }
}

// Per-view FP64 sums.  kind 0 (jointEstimation, HAADF_ReconstructionEngine_Extra.cpp:474-517):
//   [0] sum y w, [1] sum w, [2] sum yh w, [3] sum yh w y, [4] sum y^2 w, [5] sum yh^2 w,
//   yh = (y - e - mu)/I.  kind 1 (updateWeights :825-833): [0] sum e^2.
template <int K>
__global__ void view_sums_kernel(const float* __restrict__ y, const float* __restrict__ e,
                                 const double* __restrict__ mu, const double* __restrict__ gain,
                                 const double* __restrict__ wv, double* __restrict__ partial,
                                 int n_theta, int n_rp, int n_r, int n_t, int n_chunk) {
  const int v = blockIdx.x, ch = blockIdx.y;
  const int t0 = static_cast<int>(static_cast<long long>(ch) * n_t / n_chunk);
  const int t1 = static_cast<int>(static_cast<long long>(ch + 1) * n_t / n_chunk);
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
    const double s = warp_sum_d(acc[k]);
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
__global__ void rebuild_error_kernel(const float* __restrict__ y, float* __restrict__ e,
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
    e[i] = static_cast<float>(yv - mu_new[v] - (gain_new[v] * yh));
  }
}

// QGGMRF prior term of computeCost (HAADF_ReconstructionEngine.cpp:1285-1359): 13 forward
// neighbours per voxel, FP64 accumulation.  Offsets are (dz, dx, dy) with weight index
// [dy+1][dz+1][dx+1].
__constant__ int c_fwd[13][3] = {{0, 0, 1},  {0, 1, -1}, {0, 1, 0},   {0, 1, 1},   {1, -1, 0},
                                 {1, 0, 0},  {1, 1, 0},  {1, -1, -1}, {1, -1, 1},  {1, 0, -1},
                                 {1, 1, -1}, {1, 1, 1},  {1, 0, 1}};

__global__ void prior_cost_kernel(const float* __restrict__ x, DevFilter q, int n_z, int n_x,
                                  int n_y, double* __restrict__ partial) {
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  double acc = 0.0;
  const double sig_p = q.sig_p, sig_pq = q.sig_pq;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int xi = static_cast<int>(i % n_x);
    const size_t rest = i / n_x;
    const int zi = static_cast<int>(rest % n_z);
    const int yi = static_cast<int>(rest / n_z);
    const double c = x[i];
    for (int k = 0; k < 13; ++k) {
      const int zz = zi + c_fwd[k][0], xx = xi + c_fwd[k][1], yy = yi + c_fwd[k][2];
      if (zz < 0 || zz >= n_z || xx < 0 || xx >= n_x || yy < 0 || yy >= n_y) continue;
      const double d = c - static_cast<double>(
                               x[(static_cast<size_t>(yy) * n_z + zz) * n_x + xx]);
      const double ad = fabs(d);
      const double num = (q.mrf_p == 2.f) ? ad * ad : static_cast<double>(powf(ad, q.mrf_p));
      const double den =
          q.mrf_c + static_cast<double>(powf(static_cast<float>(ad), q.mrf_p - q.mrf_q)) / sig_pq;
      const int fi = 9 * (c_fwd[k][2] + 1) + 3 * (c_fwd[k][0] + 1) + (c_fwd[k][1] + 1);
      acc += static_cast<double>(q.f[fi]) * ((num / sig_p) / den);
    }
  }
  acc = warp_sum_d(acc);
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

template <int NB, bool STAGE>
int launch_sweep_t(const SweepArgs& a, int nb, size_t smem, cudaStream_t s) {
  auto k = sweep_kernel<NB, STAGE>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return -3;
  k<<<nb, kWarps * 32, smem, s>>>(a);
  return ok_or(cudaGetLastError());
}

template <int NB>
int launch_ref_t(const RefOrderArgs& a, size_t smem, cudaStream_t s) {
  auto k = ref_order_kernel<NB>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return -3;
  k<<<1, 32, smem, s>>>(a);
  return ok_or(cudaGetLastError());
}

}  // namespace

size_t sweep_smem_bytes(int n_theta, int n_rs, int t_rows, int bins) {
  return smem_layout(n_theta, n_rs, t_rows, bins, n_rs > 0).total;
}

int launch_sweep(const SweepArgs& a, int nb, size_t smem, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool st = a.smem_rows != 0;
  switch (nb) {
    case 3:
      return st ? launch_sweep_t<3, true>(a, a.n_slices, smem, s)
                : launch_sweep_t<3, false>(a, a.n_slices, smem, s);
    case 5:
      return st ? launch_sweep_t<5, true>(a, a.n_slices, smem, s)
                : launch_sweep_t<5, false>(a, a.n_slices, smem, s);
    case 9:
      return st ? launch_sweep_t<9, true>(a, a.n_slices, smem, s)
                : launch_sweep_t<9, false>(a, a.n_slices, smem, s);
    default:
      return -7;
  }
}

int launch_ref_order(const RefOrderArgs& a, int nb, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = smem_layout(a.g.n_theta, 0, 0, a.g.bins, false).total;
  switch (nb) {
    case 3:
      return launch_ref_t<3>(a, smem, s);
    case 5:
      return launch_ref_t<5>(a, smem, s);
    case 9:
      return launch_ref_t<9>(a, smem, s);
    default:
      return -7;
  }
}

int launch_sino_to_dev(const float* h, float* d, int n_theta, int n_r, int n_rp, int n_t,
                       void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  sino_to_dev_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      h, d, n_theta, n_r, n_rp, n_t);
  return ok_or(cudaGetLastError());
}
int launch_sino_to_host(const float* d, float* h, int n_theta, int n_r, int n_rp, int n_t,
                        void* stream) {
  const size_t n = static_cast<size_t>(n_theta) * n_r * n_t;
  sino_to_host_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      d, h, n_theta, n_r, n_rp, n_t);
  return ok_or(cudaGetLastError());
}
int launch_vol_to_dev(const float* zxy, float* yzx, int n_z, int n_x, int n_y, void* stream) {
  const size_t n = static_cast<size_t>(n_z) * n_x * n_y;
  vol_to_dev_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(zxy, yzx,
                                                                                      n_z, n_x, n_y);
  return ok_or(cudaGetLastError());
}
int launch_vol_to_host(const float* yzx, float* zxy, int n_z, int n_x, int n_y, void* stream) {
  const size_t n = static_cast<size_t>(n_z) * n_x * n_y;
  vol_to_host_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      yzx, zxy, n_z, n_x, n_y);
  return ok_or(cudaGetLastError());
}
int launch_error_from_projection(const float* y, const float* yest, float* e, const double* mu,
                                 int n_theta, int n_rp, int n_r, int n_t, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  error_from_projection_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      y, yest, e, mu, n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}
int launch_view_sums(int kind, const float* y, const float* e, const double* mu,
                     const double* gain, const double* wv, double* partial, double* out,
                     int n_theta, int n_rp, int n_r, int n_t, int n_chunk, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid(n_theta, n_chunk);
  int K;
  if (kind == 0) {
    K = 6;
    view_sums_kernel<6><<<grid, 256, 0, s>>>(y, e, mu, gain, wv, partial, n_theta, n_rp, n_r, n_t,
                                             n_chunk);
  } else {
    K = 1;
    view_sums_kernel<1><<<grid, 256, 0, s>>>(y, e, mu, gain, wv, partial, n_theta, n_rp, n_r, n_t,
                                             n_chunk);
  }
  const int n = n_theta * K;
  view_sums_final_kernel<<<(n + 127) / 128, 128, 0, s>>>(partial, out, n_theta, n_chunk, K);
  return ok_or(cudaGetLastError());
}
int launch_rebuild_error(const float* y, float* e, const double* mu_old, const double* gain_old,
                         const double* mu_new, const double* gain_new, int n_theta, int n_rp,
                         int n_r, int n_t, void* stream) {
  const size_t n = static_cast<size_t>(n_t) * n_theta * n_rp;
  rebuild_error_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      y, e, mu_old, gain_old, mu_new, gain_new, n_theta, n_rp, n_r, n_t);
  return ok_or(cudaGetLastError());
}
int launch_prior_cost(const float* x, const DevFilter& f, int n_z, int n_x, int n_y,
                      double* partial, int n_blocks, void* stream) {
  prior_cost_kernel<<<n_blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, f, n_z, n_x, n_y,
                                                                            partial);
  return ok_or(cudaGetLastError());
}
int launch_reduce_stats(const double* in, int n_rows, int n_cols, double* out, void* stream) {
  reduce_rows_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(in, n_rows, n_cols, out);
  return ok_or(cudaGetLastError());
}

}  // namespace mbir
