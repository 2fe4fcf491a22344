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

// Detector coordinate of a voxel row at one view.  FP32: integer + fraction so that the
// per-voxel position keeps ~1e-7 bin accuracy; FP64: the coordinate itself.
struct RowBaseF {
  int ib;
  float fb;
};
struct RowBaseD {
  double base;
};
template <typename Real>
using RowBase = typename std::conditional<std::is_same<Real, float>::value, RowBaseF,
                                          RowBaseD>::type;

// u = j0 + f (f in [0,1)) for voxel column x: u = base(z) + x * bx with bx given as hi+lo.
__device__ __forceinline__ void detector_pos(int x, RowBaseF rb, float2 bx, double, int& j0,
                                             float& f) {
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
__device__ __forceinline__ void detector_pos(int x, RowBaseD rb, float2, double bxd, int& j0,
                                             double& f) {
  const double u = fma(static_cast<double>(x), bxd, rb.base);
  const double fl = floor(u);
  j0 = static_cast<int>(fl);
  f = u - fl;
}

template <typename Real>
__device__ __forceinline__ void compute_row_base(const DevTables& tab, int n_theta, int z,
                                                 RowBase<Real>* rb, int tid, int nthreads) {
  for (int v = tid; v < n_theta; v += nthreads) {
    const double b = tab.u0[v] - static_cast<double>(z) * tab.bz[v];
    if constexpr (std::is_same<Real, float>::value) {
      const double fl = floor(b);
      rb[v].ib = static_cast<int>(fl);
      rb[v].fb = static_cast<float>(b - fl);
    } else {
      rb[v].base = b;
    }
  }
}

// A-matrix entries of one voxel at one view (AMatrixCol.cpp:148-232): bins j in
// [floor(u-d), floor(u+d)] on the detector, value = linear interpolation of the detector
// response at |u - (j+0.5)|, kept when > 0.
template <typename Real, int NB>
__device__ __forceinline__ void view_footprint(const DevGeom& g, const Real* __restrict__ hrow,
                                               int j0, Real f, int& jlo, Real (&a)[NB]) {
  const Real hw = static_cast<Real>(g.half_width);
  const Real kr = static_cast<Real>(g.kr);
  const int lo = j0 + static_cast<int>(floor(f - hw));
  const int hi = j0 + static_cast<int>(floor(f + hw));
  jlo = lo;
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const int j = lo + b;
    Real v = Real(0);
    if (j <= hi && j >= 0 && j < g.n_r) {
      const Real delta = fabs(static_cast<Real>(j0 - j) + f - Real(0.5));
      const Real xr = delta * kr;
      const int idx = static_cast<int>(xr);
      if (idx < g.bins) {
        const Real t = xr - static_cast<Real>(idx);
        v = (Real(1) - t) * hrow[idx] + t * hrow[idx + 1];
      }
    }
    a[b] = v > Real(0) ? v : Real(0);
  }
}

// rho'(d)/d of the QGGMRF prior (QGGMRF_Functions.cpp:90-104 divided by d), or rho''(0)
// (:109-112) when d == 0.
template <typename Real>
__device__ __forceinline__ Real qggmrf_coef(const DevFilter& q, Real d0) {
  const Real P = static_cast<Real>(q.mrf_p), Q = static_cast<Real>(q.mrf_q);
  const Real c = static_cast<Real>(q.mrf_c), sp = static_cast<Real>(q.sig_p);
  if (d0 == Real(0)) return P / (sp * c);
  const Real ad = fabs(d0);
  const Real t1 = pow(ad, P - Q) / static_cast<Real>(q.sig_pq);
  const Real t3 = c + t1;
  Real r = (P - ((P - Q) * t1) / t3) / (t3 * sp);
  if (P != Real(2)) r *= pow(ad, P - Real(2));
  return r;
}

// One voxel (z, x, y) processed by one warp.  es points at the first detector row of slice y
// (row stride rs values between views, plane stride ps between t rows).  Returns in wst
// (lane 0): ROI sum|dx|, ROI sum|x|, zero-skipped, updated.
template <typename Real, int NB>
__device__ __forceinline__ void voxel_step(const DevGeom& g, const DevFilter& q,
                                           Real* __restrict__ vol, Real* es, int rs, int ps,
                                           const RowBase<Real>* rb, const Real* sH,
                                           const float2* sbx, const double* sbxd,
                                           const typename V2<Real>::type* sgw, int z, int x,
                                           int y, int tcount, const Real* hv, int mode,
                                           int iter_nonzero, int zero_skipping, int lane,
                                           double* wst) {
  using R2 = typename V2<Real>::type;
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t vidx = static_cast<size_t>(y) * plane + static_cast<size_t>(z) * g.n_x + x;
  const Real V = vol[vidx];
  const Real hw = static_cast<Real>(g.half_width);

  int jlo[kMaxViewsPerLane];
  Real a[kMaxViewsPerLane][NB];
  bool any = false;
#pragma unroll
  for (int i = 0; i < kMaxViewsPerLane; ++i) {
    const int v = lane + 32 * i;
    jlo[i] = 0;
#pragma unroll
    for (int b = 0; b < NB; ++b) a[i][b] = Real(0);
    if (v < g.n_theta) {
      int j0;
      Real f;
      detector_pos(x, rb[v], sbx ? sbx[v] : float2{0.f, 0.f}, sbxd ? sbxd[v] : 0.0, j0, f);
      const Real u = static_cast<Real>(j0) + f;
      if (!(u + hw < Real(0) || u - hw > static_cast<Real>(g.n_r))) {
        view_footprint<Real, NB>(g, sH + v * (g.bins + 1), j0, f, jlo[i], a[i]);
#pragma unroll
        for (int b = 0; b < NB; ++b) any |= (a[i][b] > Real(0));
      }
    }
  }
  if (!__any_sync(kFull, any)) return;  // empty A-column: the line is never visited

  if (mode == kModeProject) {
    if (V != Real(0)) {
#pragma unroll
      for (int i = 0; i < kMaxViewsPerLane; ++i) {
        const int v = lane + 32 * i;
        if (v >= g.n_theta) continue;
        const Real gain = sgw[v].x;
        for (int tr = 0; tr < tcount; ++tr) {
          const Real hh = hv[tr];
          Real* row = es + tr * ps + v * rs + jlo[i];
#pragma unroll
          for (int b = 0; b < NB; ++b)
            if (a[i][b] > Real(0)) row[b] += gain * (a[i][b] * hh * V);
        }
      }
    }
    return;
  }

  // 26-neighbourhood, one neighbour per lane (UpdateVoxels.cpp:283-306)
  Real nb = Real(0);
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
  if (zero_skipping && iter_nonzero && V == Real(0)) {
    if (!__any_sync(kFull, nb > Real(0))) {
      if (lane == 0) wst[2] += 1.0;
      return;
    }
  }
  // theta1 / theta2 (UpdateVoxels.cpp:343-369)
  Real t1 = Real(0), t2 = Real(0);
#pragma unroll
  for (int i = 0; i < kMaxViewsPerLane; ++i) {
    const int v = lane + 32 * i;
    if (v >= g.n_theta) continue;
    const R2 gw = sgw[v];
    for (int tr = 0; tr < tcount; ++tr) {
      const Real hh = hv[tr];
      const Real* row = es + tr * ps + v * rs + jlo[i];
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (a[i][b] > Real(0)) {
          const Real pe = gw.x * a[i][b] * hh;
          t2 += pe * pe * gw.y;
          t1 += row[b] * pe * gw.y;
        }
      }
    }
  }
  const Real theta1 = -warp_sum(t1);
  const Real theta2 = warp_sum(t2);
  // bracket (find_min_max, UpdateVoxels.cpp:47-63): over all 27 entries, centre and
  // out-of-range entries count as 0
  Real lo = warp_min(nb), hi = warp_max(nb);
  if (theta2 != Real(0)) {
    const Real cand = V - theta1 / theta2;
    lo = lo > cand ? cand : lo;
    hi = hi < cand ? cand : hi;
  }
  // QGGMRF surrogate, one iteration (QGGMRF_Functions.cpp:153-206)
  Real s1 = Real(0), s2 = Real(0);
  if (nvalid) {
    const Real tc = static_cast<Real>(q.f[lane]) * qggmrf_coef<Real>(q, V - nb);
    s1 = tc * nb;
    s2 = tc;
  }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  const Real u = (s1 + theta2 * V - theta1) / (s2 + theta2);
  Real nv = V + static_cast<Real>(q.mrf_alpha) * (u - V);
  nv = (nv < lo) ? lo : ((nv > hi) ? hi : nv);
  if (nv < Real(0)) nv = Real(0);  // positivity (UpdateVoxels.cpp:394-400)
  const Real dlt = nv - V;
  // error-sinogram scatter (UpdateVoxels.cpp:423-449)
  if (dlt != Real(0)) {
#pragma unroll
    for (int i = 0; i < kMaxViewsPerLane; ++i) {
      const int v = lane + 32 * i;
      if (v >= g.n_theta) continue;
      const Real gain = sgw[v].x;
      for (int tr = 0; tr < tcount; ++tr) {
        const Real hh = hv[tr];
        Real* row = es + tr * ps + v * rs + jlo[i];
#pragma unroll
        for (int b = 0; b < NB; ++b)
          if (a[i][b] > Real(0)) row[b] -= gain * (a[i][b] * hh * dlt);
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

struct SmemLayout {
  size_t bar, stats, rb, bx, bxd, gw, H, hv, es, total;
};

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

__host__ __device__ inline SmemLayout smem_layout(int n_theta, int n_rs, int t_rows, int bins,
                                                  bool stage, size_t real_bytes) {
  SmemLayout L;
  size_t o = 0;
  L.bar = o;
  o += 16;
  L.stats = o;
  o += sizeof(double) * kWarps * kStatSlots;
  L.rb = o;
  o = align_up(o + 8 * static_cast<size_t>(n_theta), 16);
  L.bx = o;
  o = align_up(o + sizeof(float2) * n_theta, 16);
  L.bxd = o;
  o = align_up(o + sizeof(double) * n_theta, 16);
  L.gw = o;
  o = align_up(o + 2 * real_bytes * n_theta, 16);
  L.H = o;
  o = align_up(o + real_bytes * n_theta * (bins + 1), 16);
  L.hv = o;
  o = align_up(o + real_bytes * kMaxTRows, 128);
  L.es = o;
  if (stage) o += real_bytes * static_cast<size_t>(t_rows) * n_theta * n_rs;
  L.total = align_up(o, 16);
  return L;
}

template <typename Real, int NB, bool STAGE>
__global__ void __launch_bounds__(kWarps * 32, 1) sweep_kernel(SweepArgs A) {
  using R2 = typename V2<Real>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  const DevGeom& g = A.g;
  const int y = A.colour + 2 * static_cast<int>(blockIdx.x);
  if (y >= g.n_y) return;
  const int tid = threadIdx.x, nthreads = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int tcount = A.tab.t_count[y], tfirst = A.tab.t_first[y];
  const SmemLayout L = smem_layout(g.n_theta, A.n_rs, tcount, g.bins, STAGE, sizeof(Real));
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L.bar);
  double* sstat = reinterpret_cast<double*>(smem + L.stats);
  RowBase<Real>* rb = reinterpret_cast<RowBase<Real>*>(smem + L.rb);
  float2* sbx = reinterpret_cast<float2*>(smem + L.bx);
  double* sbxd = reinterpret_cast<double*>(smem + L.bxd);
  R2* sgw = reinterpret_cast<R2*>(smem + L.gw);
  Real* sH = reinterpret_cast<Real*>(smem + L.H);
  Real* shv = reinterpret_cast<Real*>(smem + L.hv);
  const Real* gH = static_cast<const Real*>(A.tab.H);
  const R2* ggw = static_cast<const R2*>(A.tab.gw);
  const Real* ghv = static_cast<const Real*>(A.tab.hval);
  Real* const ge = static_cast<Real*>(A.e);
  Real* const gx = static_cast<Real*>(A.x);
  constexpr bool kF32 = std::is_same<Real, float>::value;

  for (int i = tid; i < g.n_theta * (g.bins + 1); i += nthreads) sH[i] = gH[i];
  for (int v = tid; v < g.n_theta; v += nthreads) {
    if (kF32) sbx[v] = A.tab.bx[v];
    else sbxd[v] = A.tab.bxd[v];
    sgw[v] = ggw[v];
  }
  if (tid < kMaxTRows) shv[tid] = ghv[y * kMaxTRows + tid];

  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  Real* es;
  int rs, ps;
  const int rows = tcount * g.n_theta;
  const uint32_t row_bytes = static_cast<uint32_t>(g.n_rp * sizeof(Real));
  if (STAGE) {
    es = reinterpret_cast<Real*>(smem + L.es);
    rs = A.n_rs;
    ps = g.n_theta * A.n_rs;
    if (A.mode == kModeProject) {
      for (int i = tid; i < tcount * ps; i += nthreads) es[i] = Real(0);
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
        bulk_g2s(es + tr * ps + v * rs,
                 ge + (static_cast<size_t>(tfirst + tr)) * sino_plane +
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
    es = ge + static_cast<size_t>(tfirst) * sino_plane;
    rs = g.n_rp;
    ps = static_cast<int>(sino_plane);
  }

  double wst[kStatSlots] = {0.0, 0.0, 0.0, 0.0};
  for (int rr = 0; rr < g.n_z; ++rr) {
    const int z = A.row_order[rr];
    __syncthreads();
    compute_row_base<Real>(A.tab, g.n_theta, z, rb, tid, nthreads);
    __syncthreads();
    for (int k = 0; k < A.stride; ++k) {
      for (int x = k + A.stride * warp; x < g.n_x; x += A.stride * kWarps)
        voxel_step<Real, NB>(g, A.flt, gx, es, rs, ps, rb, sH, kF32 ? sbx : nullptr,
                             kF32 ? nullptr : sbxd, sgw, z, x, y, tcount, shv, A.mode,
                             A.iter_nonzero, A.zero_skipping, lane, wst);
      __syncthreads();
    }
  }

  if (STAGE) {
    fence_proxy_async_smem();
    __syncthreads();
    for (int r = tid; r < rows; r += nthreads) {
      const int tr = r / g.n_theta, v = r % g.n_theta;
      bulk_s2g(ge + (static_cast<size_t>(tfirst + tr)) * sino_plane +
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

template <typename Real, int NB>
__global__ void __launch_bounds__(32, 1) ref_order_kernel(RefOrderArgs A) {
  using R2 = typename V2<Real>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  const DevGeom& g = A.g;
  const int lane = threadIdx.x;
  const SmemLayout L = smem_layout(g.n_theta, 0, 0, g.bins, false, sizeof(Real));
  RowBase<Real>* rb = reinterpret_cast<RowBase<Real>*>(smem + L.rb);
  float2* sbx = reinterpret_cast<float2*>(smem + L.bx);
  double* sbxd = reinterpret_cast<double*>(smem + L.bxd);
  R2* sgw = reinterpret_cast<R2*>(smem + L.gw);
  Real* sH = reinterpret_cast<Real*>(smem + L.H);
  const Real* gH = static_cast<const Real*>(A.tab.H);
  const R2* ggw = static_cast<const R2*>(A.tab.gw);
  const Real* ghv = static_cast<const Real*>(A.tab.hval);
  Real* const ge = static_cast<Real*>(A.e);
  Real* const gx = static_cast<Real*>(A.x);
  constexpr bool kF32 = std::is_same<Real, float>::value;
  for (int i = lane; i < g.n_theta * (g.bins + 1); i += 32) sH[i] = gH[i];
  for (int v = lane; v < g.n_theta; v += 32) {
    if (kF32) sbx[v] = A.tab.bx[v];
    else sbxd[v] = A.tab.bxd[v];
    sgw[v] = ggw[v];
  }
  __syncwarp();
  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  double wst[kStatSlots] = {0.0, 0.0, 0.0, 0.0};
  for (int n = 0; n < A.n_lines; ++n) {
    const int l = A.lines[n];
    const int z = l / g.n_x, x = l % g.n_x;
    __syncwarp();
    compute_row_base<Real>(A.tab, g.n_theta, z, rb, lane, 32);
    __syncwarp();
    for (int y = 0; y < g.n_y; ++y) {
      Real* es = ge + static_cast<size_t>(A.tab.t_first[y]) * sino_plane;
      voxel_step<Real, NB>(g, A.flt, gx, es, g.n_rp, static_cast<int>(sino_plane), rb, sH,
                           kF32 ? sbx : nullptr, kF32 ? nullptr : sbxd, sgw, z, x, y,
                           A.tab.t_count[y], ghv + y * kMaxTRows, kModeICD, A.iter_nonzero,
                           A.zero_skipping, lane, wst);
      __syncwarp();
    }
  }
  if (lane == 0)
    for (int s = 0; s < kStatSlots; ++s) A.stats[s] = wst[s];
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
    e[i] = static_cast<Real>(yv - mu_new[v] - (gain_new[v] * yh));
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
  const size_t total = static_cast<size_t>(n_z) * n_x * n_y;
  double acc = 0.0;
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
      double num, pq;
      if constexpr (std::is_same<Real, float>::value) {
        // FP32 elementwise power (relative error ~1e-7), FP64 accumulation
        num = (q.mrf_p == 2.0) ? ad * ad
                               : static_cast<double>(powf(static_cast<float>(ad),
                                                          static_cast<float>(q.mrf_p)));
        pq = static_cast<double>(
            powf(static_cast<float>(ad), static_cast<float>(q.mrf_p - q.mrf_q)));
      } else {
        num = pow(ad, q.mrf_p);
        pq = pow(ad, q.mrf_p - q.mrf_q);
      }
      const int fi = 9 * (c_fwd[k][2] + 1) + 3 * (c_fwd[k][0] + 1) + (c_fwd[k][1] + 1);
      acc += q.f[fi] * ((num / q.sig_p) / (q.mrf_c + pq / q.sig_pq));
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

template <typename Real, int NB, bool STAGE>
int launch_sweep_t(const SweepArgs& a, size_t smem, cudaStream_t s) {
  auto k = sweep_kernel<Real, NB, STAGE>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return -3;
  k<<<a.n_slices, kWarps * 32, smem, s>>>(a);
  return ok_or(cudaGetLastError());
}

template <typename Real>
int launch_sweep_r(const SweepArgs& a, int nb, size_t smem, cudaStream_t s) {
  const bool st = a.smem_rows != 0;
  switch (nb) {
    case 3:
      return st ? launch_sweep_t<Real, 3, true>(a, smem, s)
                : launch_sweep_t<Real, 3, false>(a, smem, s);
    case 5:
      return st ? launch_sweep_t<Real, 5, true>(a, smem, s)
                : launch_sweep_t<Real, 5, false>(a, smem, s);
    case 9:
      return st ? launch_sweep_t<Real, 9, true>(a, smem, s)
                : launch_sweep_t<Real, 9, false>(a, smem, s);
    default:
      return -7;
  }
}

template <typename Real, int NB>
int launch_ref_t(const RefOrderArgs& a, size_t smem, cudaStream_t s) {
  auto k = ref_order_kernel<Real, NB>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return -3;
  k<<<1, 32, smem, s>>>(a);
  return ok_or(cudaGetLastError());
}

template <typename Real>
int launch_ref_r(const RefOrderArgs& a, int nb, cudaStream_t s) {
  const size_t smem = smem_layout(a.g.n_theta, 0, 0, a.g.bins, false, sizeof(Real)).total;
  switch (nb) {
    case 3:
      return launch_ref_t<Real, 3>(a, smem, s);
    case 5:
      return launch_ref_t<Real, 5>(a, smem, s);
    case 9:
      return launch_ref_t<Real, 9>(a, smem, s);
    default:
      return -7;
  }
}

}  // namespace

size_t sweep_smem_bytes(int n_theta, int n_rs, int t_rows, int bins, int fp64) {
  return smem_layout(n_theta, n_rs, t_rows, bins, n_rs > 0, fp64 ? 8 : 4).total;
}

int launch_sweep(const SweepArgs& a, int nb, size_t smem, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a.fp64 ? launch_sweep_r<double>(a, nb, smem, s) : launch_sweep_r<float>(a, nb, smem, s);
}

int launch_ref_order(const RefOrderArgs& a, int nb, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return a.fp64 ? launch_ref_r<double>(a, nb, s) : launch_ref_r<float>(a, nb, s);
}

#define MBIR_DISPATCH(fp64, KERNEL, GRID, BLOCK, STREAM, ...)                             \
  do {                                                                                    \
    if (fp64)                                                                             \
      KERNEL<double><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__);                            \
    else                                                                                  \
      KERNEL<float><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__);                             \
  } while (0)

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
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid(n_theta, n_chunk);
  const int K = kind == 0 ? 6 : 1;
  if (fp64) {
    if (kind == 0)
      view_sums_kernel<double, 6><<<grid, 256, 0, s>>>(RP<double>(y), RP<double>(e), mu, gain, wv,
                                                        partial, n_theta, n_rp, n_r, n_t, n_chunk);
    else
      view_sums_kernel<double, 1><<<grid, 256, 0, s>>>(RP<double>(y), RP<double>(e), mu, gain, wv,
                                                        partial, n_theta, n_rp, n_r, n_t, n_chunk);
  } else {
    if (kind == 0)
      view_sums_kernel<float, 6><<<grid, 256, 0, s>>>(RP<float>(y), RP<float>(e), mu, gain, wv,
                                                       partial, n_theta, n_rp, n_r, n_t, n_chunk);
    else
      view_sums_kernel<float, 1><<<grid, 256, 0, s>>>(RP<float>(y), RP<float>(e), mu, gain, wv,
                                                       partial, n_theta, n_rp, n_r, n_t, n_chunk);
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
