// mbir_sweep.cuh -- the ICD sweep / forward-projection kernels (device code, templated on the
// real type).  Included by mbir_sweep_f32.cu and mbir_sweep_f64.cu, which instantiate them.
//
//   sweep_kernel      ICD sweep (and forward projection) over the voxel slices of one y-colour.
//                     One CTA owns one voxel slice y: the detector rows t of that slice (all
//                     views, all r) are staged into shared memory with TMA bulk copies and stay
//                     there for the whole sweep, so every theta1/theta2 gather and every
//                     error-sinogram scatter is an on-chip access.  Inside the slice the CTA
//                     walks the z-rows; for each row it caches the 9 neighbouring voxel rows
//                     (y-1..y+1, z-1..z+1) in shared memory and updates the voxels of one
//                     conflict-free class (x = k, k+S, ...: no two share a detector bin at any
//                     view, none are prior neighbours) in parallel, one voxel per group of G
//                     lanes.  The result equals the sequential ICD of that visit order.
//   ref_order_kernel  the reference's visit order (one voxel line after another, y in order)
//                     with the error sinogram in HBM; one warp, used for order-exact parity.
//
// Reference semantics: UpdateYSlice::execute (Code/MBIRLib/HAADF/
// HAADF_ReconstructionEngine_UpdateVoxels.cpp:149-484), the A-column of
// Code/MBIRLib/Common/AMatrixCol.cpp:82-239 and the QGGMRF surrogate of
// Code/MBIRLib/Reconstruction/QGGMRF_Functions.cpp:82-206.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "mbir_internal.h"

namespace mbir {
namespace sweep {

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
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the mbarrier phase; gives up after kWaitNs of wall time (or kWaitLimit polls).
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
  const uint32_t a = smem_u32(bar);
  const uint64_t t0 = global_ns();
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
    if ((i & 255u) == 255u && global_ns() - t0 > kWaitNs) return false;
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
__device__ __forceinline__ uint32_t dynamic_smem_bytes() {
  uint32_t v;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(v));
  return v;
}

// ---- reductions within aligned groups of G lanes (all 32 lanes take part) -----------------
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <int G, typename T>
__device__ __forceinline__ T group_min(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(kFull, v, o);
    v = w < v ? w : v;
  }
  return v;
}
template <int G, typename T>
__device__ __forceinline__ T group_max(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(kFull, v, o);
    v = w > v ? w : v;
  }
  return v;
}
template <int G>
__device__ __forceinline__ bool group_any(bool p, int lane) {
  const unsigned b = __ballot_sync(kFull, p);
  if constexpr (G == 32) {
    return b != 0u;
  } else {
    const unsigned m = ((1u << G) - 1u) << (lane & ~(G - 1));
    return (b & m) != 0u;
  }
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
__device__ __forceinline__ RowBase<Real> row_base(const DevTables& tab, int z, int v) {
  const double b = tab.u0[v] - static_cast<double>(z) * tab.bz[v];
  RowBase<Real> r;
  if constexpr (std::is_same<Real, float>::value) {
    const double fl = floor(b);
    r.ib = static_cast<int>(fl);
    r.fb = static_cast<float>(b - fl);
  } else {
    r.base = b;
  }
  return r;
}

template <typename Real>
__device__ __forceinline__ void compute_row_base(const DevTables& tab, int n_theta, int z,
                                                 RowBase<Real>* rb, int tid, int nthreads) {
  for (int v = tid; v < n_theta; v += nthreads) rb[v] = row_base<Real>(tab, z, v);
}

// A-matrix entries of one voxel at one view (AMatrixCol.cpp:148-232): bins j in
// [floor(u-d), floor(u+d)] on the detector, value = linear interpolation of the detector
// response at |u - (j+0.5)|, kept when > 0.
template <typename Real, int NB>
__device__ __forceinline__ void view_footprint(const DevGeom& g, Real hw, Real kr,
                                               const Real* __restrict__ hrow, int j0, Real f,
                                               int& jlo, Real (&a)[NB]) {
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

// |d|^e for the prior coefficient: FP32 uses the fast power intrinsic (a few ulp, far below the
// FP32 sweep's tolerance); FP64 keeps pow.
template <typename Real>
__device__ __forceinline__ Real prior_pow(Real a, Real e) {
  return pow(a, e);
}
template <>
__device__ __forceinline__ float prior_pow<float>(float a, float e) {
  return __powf(a, e);
}

// Bragg selector of one entry after the scatter (BFForwardModel.cpp:898-932): |e sqrt(w)| < T.
// FP32 compares e^2 w < T^2 (the same test for T >= 0, without a square root per entry).
template <typename Real>
__device__ __forceinline__ uint8_t bragg_selected(Real e, Real w, Real t) {
  return fabs(e * sqrt(w)) < t ? 1 : 0;
}
template <>
__device__ __forceinline__ uint8_t bragg_selected<float>(float e, float w, float t) {
  return e * e * w < t * t ? 1 : 0;
}

// Prior and footprint constants in the sweep's precision, converted from FP64 once per slice
// (on GB300 every FP64-to-FP32 conversion runs on the narrow FP64 pipe, so converting them per
// voxel cost ~2k cycles per voxel step).
template <typename Real>
struct PriorConst {
  Real P, Q, c, sp, sig_pq, inv_sig_pq, alpha, hw, kr;
};
template <typename Real>
__device__ __forceinline__ PriorConst<Real> prior_const(const DevFilter& q, const DevGeom& g) {
  PriorConst<Real> k;
  k.P = static_cast<Real>(q.mrf_p);
  k.Q = static_cast<Real>(q.mrf_q);
  k.c = static_cast<Real>(q.mrf_c);
  k.sp = static_cast<Real>(q.sig_p);
  k.sig_pq = static_cast<Real>(q.sig_pq);
  k.inv_sig_pq = static_cast<Real>(q.inv_sig_pq);
  k.alpha = static_cast<Real>(q.mrf_alpha);
  k.hw = static_cast<Real>(g.half_width);
  k.kr = static_cast<Real>(g.kr);
  return k;
}

// rho'(d)/d of the QGGMRF prior (QGGMRF_Functions.cpp:90-104 divided by d), or rho''(0)
// (:109-112) when d == 0.
template <typename Real>
__device__ __forceinline__ Real qggmrf_coef(const PriorConst<Real>& q, Real d0) {
  const Real P = q.P, Q = q.Q, c = q.c, sp = q.sp;
  if (d0 == Real(0)) return P / (sp * c);
  const Real ad = fabs(d0);
  const Real t1 = prior_pow<Real>(ad, P - Q) / q.sig_pq;
  const Real t3 = c + t1;
  Real r = (P - ((P - Q) * t1) / t3) / (t3 * sp);
  if (P != Real(2)) r *= prior_pow<Real>(ad, P - Real(2));
  return r;
}
// FP32: the same function as (P c + Q t1) / (t3^2 sigma^P) (P - (P-Q) t1/t3 = (P c + Q t1)/t3),
// one fast division instead of three IEEE divisions (relative error a few ulp).
template <>
__device__ __forceinline__ float qggmrf_coef<float>(const PriorConst<float>& q, float d0) {
  const float P = q.P, Q = q.Q, c = q.c, sp = q.sp;
  if (d0 == 0.f) return P / (sp * c);
  const float ad = fabsf(d0);
  const float t1 = __powf(ad, P - Q) * q.inv_sig_pq;
  const float t3 = c + t1;
  float r = __fdividef(P * c + Q * t1, t3 * t3 * sp);
  if (P != 2.f) r *= __powf(ad, P - 2.f);
  return r;
}

// round(|v| 2^32) as an unsigned 64-bit fixed-point value; for FP32 the product is exact in
// single precision, so the result equals the FP64 computation
template <typename Real>
__device__ __forceinline__ unsigned long long fix32(Real v) {
  return __double2ull_rn(fabs(static_cast<double>(v)) * kFixScale);
}
template <>
__device__ __forceinline__ unsigned long long fix32<float>(float v) {
  return __float2ull_rn(fabsf(v) * 4294967296.0f);
}

// Everything one CTA (or the reference-order warp) shares while it works on voxel slice y.
template <typename Real>
struct SliceCtx {
  using R2 = typename V2<Real>::type;
  const DevGeom* g;
  const DevFilter* q;
  Real* vol;                 // global volume [n_y][n_z][n_x]
  Real* es;                  // first detector row of the slice
  int rs, ps;                // row stride (between views), plane stride (between t rows)
  const RowBase<Real>* rb;   // current z-row's detector coordinates per view
  const Real* sH;            // [n_theta][bins+1]
  const float2* sbx;         // FP32 path
  const double* sbxd;        // FP64 path
  const R2* sgw;             // (gain, weight) per view
  const Real* hv;            // t-response of the slice
  const uint8_t* lineok;     // [n_z][n_x] A-column not empty
  Real* cache;               // [9][n_x] neighbour rows (dy,dz) or nullptr (read global)
  int tcount;
  int mode, iter_nonzero, zero_skipping;
  int inline_zs;             // run the zero-skipping test in group_step (candidates may be skipped)
  // bright field: per-entry weights (HBM), Bragg selector (shared memory or HBM)
  const Real* bw;
  int bw_rs, bw_ps;
  uint8_t* bs;
  int bs_rs, bs_ps;
  Real bt, bdt;              // T, delta*T
  unsigned long long* mag_fx;
  const float4* acol;        // A-column table (level-scheduled sweeps) or nullptr
  const PriorConst<Real>* pc;  // prior and footprint constants (shared memory)
  const Real* qf;            // prior weights [27] (shared memory)
  bool coherent;             // neighbour planes read from the volume bypass L1 (other CTAs of
                             // the launch write them)
};

// Zero skipping (UpdateVoxels.cpp:310-338, BFUpdateYSlice.cpp:238-262): after the first sweep a
// voxel that is 0 with no neighbour > 0 is not updated.  One thread, from the neighbour cache
// (rows outside the volume are cached as 0).
template <typename Real>
__device__ __forceinline__ bool zero_skipped(const SliceCtx<Real>& c, int x, Real V) {
  if (!(c.zero_skipping && c.iter_nonzero && V == Real(0))) return false;
  const int n_x = c.g->n_x;
#pragma unroll
  for (int r = 0; r < 9; ++r) {
    const Real* row = c.cache + r * n_x;
    if (row[x] > Real(0)) return false;
    if (x > 0 && row[x - 1] > Real(0)) return false;
    if (x + 1 < n_x && row[x + 1] > Real(0)) return false;
  }
  return true;
}

// Per-group accumulators: [0] ROI sum |dx|, [1] ROI sum |x| (fixed point, kFixScale),
// [2] zero-skipped, [3] updated.
struct GroupAcc {
  unsigned long long v[kStatSlots];
};

// One voxel (z, x, y) updated by one group of G lanes (G = 16: two voxels per warp).  All 32
// lanes of the warp call this together; `active` is false for a group with no voxel.  With
// INLINE_ZS the zero-skipping test runs here (reference order); otherwise the caller has
// already removed skipped voxels.
__device__ __forceinline__ float f4_at(const float4& q, int k) {
  return k == 0 ? q.x : (k == 1 ? q.y : (k == 2 ? q.z : q.w));
}

// With ACOL the voxel's A-column comes from the table (level-scheduled sweeps, FP32): the
// same values the in-kernel computation gives, loaded first so that their latency overlaps
// the neighbour loads.
template <typename Real, int NB, int G, int VPL, bool BF, bool INLINE_ZS, bool ACOL = false>
__device__ __forceinline__ void group_step(const SliceCtx<Real>& c, int z, int x_req, int y,
                                           bool active, int lane, GroupAcc& acc) {
  using R2 = typename V2<Real>::type;
  static_assert(!ACOL || std::is_same<Real, float>::value, "A-column table is FP32");
  const DevGeom& g = *c.g;
  const int gl = lane & (G - 1);
  const int x = active ? x_req : 0;
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t vidx = static_cast<size_t>(y) * plane + static_cast<size_t>(z) * g.n_x + x;
  constexpr int AW = acol_width(NB);
  float4 aq[ACOL ? VPL : 1][ACOL ? AW : 1];
  if constexpr (ACOL) {
    const float4* ac = c.acol + (static_cast<size_t>(z) * g.n_x + x) * g.n_theta * AW;
#pragma unroll
    for (int i = 0; i < VPL; ++i) {
      const int v = gl + G * i;
#pragma unroll
      for (int w = 0; w < AW; ++w)
        aq[i][w] = (active && v < g.n_theta) ? __ldg(ac + v * AW + w)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  const Real V = c.cache ? c.cache[4 * g.n_x + x] : c.vol[vidx];
  // scheduled lines (ACOL) all have a non-empty A-column
  bool live = active && (ACOL || c.lineok[static_cast<size_t>(z) * g.n_x + x] != 0);

  // 26-neighbourhood, entries k = gl, gl+G, ... (UpdateVoxels.cpp:283-306); centre and
  // out-of-range entries are 0 in the bracket, as in the reference
  constexpr int NNB = (27 + G - 1) / G;
  Real nb[NNB];
  bool nvalid[NNB];
  if (c.mode != kModeProject) {
    bool pos = false;
#pragma unroll
    for (int i = 0; i < NNB; ++i) {
      const int k = gl + G * i;
      nb[i] = Real(0);
      nvalid[i] = false;
      if (k < 27 && k != 13) {
        const int dy = k / 9 - 1, dz = (k / 3) % 3 - 1, dx = k % 3 - 1;
        const int yy = y + dy, zz = z + dz, xx = x + dx;
        if (yy >= 0 && yy < g.n_y && zz >= 0 && zz < g.n_z && xx >= 0 && xx < g.n_x) {
          if (c.cache) {
            nb[i] = c.cache[((dy + 1) * 3 + (dz + 1)) * g.n_x + xx];
          } else {
            const Real* src =
                c.vol + static_cast<size_t>(yy) * plane + static_cast<size_t>(zz) * g.n_x + xx;
            nb[i] = (c.coherent && dy != 0) ? __ldcg(src) : *src;
          }
          nvalid[i] = true;
          pos |= nb[i] > Real(0);
        }
      }
    }
    if (INLINE_ZS || c.inline_zs) {
      // the ballot runs on all 32 lanes: the two voxel groups of a warp may disagree
      const bool any_pos = group_any<G>(pos, lane);
      if (c.zero_skipping && c.iter_nonzero && V == Real(0) && !any_pos) {
        if (live && gl == 0) acc.v[2] += 1;
        live = false;
      }
    }
  } else {
    live = live && V != Real(0);
  }
  if (!__any_sync(kFull, live)) return;

  // QGGMRF surrogate sums of this lane's neighbours (QGGMRF_Functions.cpp:153-206): they need
  // only V and the neighbours, so their transcendental arithmetic is issued before the
  // footprint's memory traffic and overlaps it
  Real s1 = Real(0), s2 = Real(0);
  if (c.mode != kModeProject) {
#pragma unroll
    for (int i = 0; i < NNB; ++i) {
      if (nvalid[i]) {
        const Real tc =
            c.qf[gl + G * i] * qggmrf_coef<Real>(*c.pc, V - nb[i]);
        s1 += tc * nb[i];
        s2 += tc;
      }
    }
  }

  // A-column of the voxel, lanes over views (AMatrixCol.cpp:148-232)
  const Real hw = c.pc->hw;
  int jlo[VPL];
  Real a[VPL][NB];
#pragma unroll
  for (int i = 0; i < VPL; ++i) {
    const int v = gl + G * i;
    jlo[i] = 0;
#pragma unroll
    for (int b = 0; b < NB; ++b) a[i][b] = Real(0);
    if constexpr (ACOL) {
      if (v < g.n_theta && live) {
        jlo[i] = __float_as_int(aq[i][0].x);
#pragma unroll
        for (int b = 0; b < NB; ++b) a[i][b] = f4_at(aq[i][(b + 1) >> 2], (b + 1) & 3);
      }
      continue;
    }
    if (v < g.n_theta && live) {
      int j0;
      Real f;
      detector_pos(x, c.rb[v], c.sbx ? c.sbx[v] : float2{0.f, 0.f}, c.sbxd ? c.sbxd[v] : 0.0, j0,
                   f);
      const Real u = static_cast<Real>(j0) + f;
      if (!(u + hw < Real(0) || u - hw > static_cast<Real>(g.n_r)))
        view_footprint<Real, NB>(g, hw, c.pc->kr, c.sH + v * (g.bins + 1), j0, f, jlo[i], a[i]);
    }
  }

  if (c.mode == kModeProject) {
#pragma unroll
    for (int i = 0; i < VPL; ++i) {
      const int v = gl + G * i;
      if (v >= g.n_theta || !live) continue;
      const Real gain = c.sgw[v].x;
      for (int tr = 0; tr < c.tcount; ++tr) {
        const Real hh = c.hv[tr];
        Real* row = c.es + tr * c.ps + v * c.rs + jlo[i];
#pragma unroll
        for (int b = 0; b < NB; ++b)
          if (a[i][b] > Real(0)) row[b] += gain * (a[i][b] * hh * V);
      }
    }
    return;
  }

  // theta1 / theta2 (UpdateVoxels.cpp:343-369; BF: BFForwardModel::computeTheta,
  // BFForwardModel.cpp:851-892, entries the Bragg selector rejects weighted by
  // delta T / (|e| sqrt(w)))
  Real t1 = Real(0), t2 = Real(0);
  // One detector row per slice (delta_xy = delta_t, every fine level): the footprint's error
  // values (and, for bright field, weights and selector bytes) are gathered into registers in
  // one batch -- unconditional loads from a safe index, so they are all in flight together --
  // and reused by the scatter.
  const bool one_row = c.tcount == 1;
  constexpr int BV = BF ? VPL : 1, BN = BF ? NB : 1;
  Real ev[VPL][NB];
  Real wv[BV][BN];
  uint8_t sv[BV][BN];
  int eidx[VPL];
  if (one_row) {
    const Real hh = c.hv[0];
#pragma unroll
    for (int i = 0; i < VPL; ++i) {
      const int v = gl + G * i;
      const bool vok = v < g.n_theta && live;
      eidx[i] = vok ? v * c.rs + jlo[i] : 0;
      const int widx = vok ? v * c.bw_rs + jlo[i] : 0;
      const int sidx = vok ? v * c.bs_rs + jlo[i] : 0;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        const bool ok = vok && a[i][b] > Real(0);
        ev[i][b] = c.es[ok ? eidx[i] + b : 0];
        if constexpr (BF) {
          wv[i][b] = __ldg(c.bw + (ok ? widx + b : 0));
          sv[i][b] = c.bs[ok ? sidx + b : 0];
        }
      }
    }
#pragma unroll
    for (int i = 0; i < VPL; ++i) {
      const int v = gl + G * i;
      if (v >= g.n_theta || !live) continue;
      const R2 gw = c.sgw[v];
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        if (a[i][b] > Real(0)) {
          const Real pe = gw.x * a[i][b] * hh;
          if constexpr (BF) {
            const Real w = wv[i][b];
            if (sv[i][b]) {
              t2 += pe * pe * w;
              t1 += ev[i][b] * pe * w;
            } else {
              const Real qc = c.bdt / (fabs(ev[i][b]) * sqrt(w));
              t2 += qc * (pe * pe * w);
              t1 += qc * (ev[i][b] * pe * w);
            }
          } else {
            t2 += pe * pe * gw.y;
            t1 += ev[i][b] * pe * gw.y;
          }
        }
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < VPL; ++i) {
      const int v = gl + G * i;
      if (v >= g.n_theta || !live) continue;
      const R2 gw = c.sgw[v];
      for (int tr = 0; tr < c.tcount; ++tr) {
        const Real hh = c.hv[tr];
        const Real* row = c.es + tr * c.ps + v * c.rs + jlo[i];
        if constexpr (BF) {
          const Real* wr = c.bw + tr * c.bw_ps + v * c.bw_rs + jlo[i];
          const uint8_t* sr = c.bs + tr * c.bs_ps + v * c.bs_rs + jlo[i];
#pragma unroll
          for (int b = 0; b < NB; ++b) {
            if (a[i][b] > Real(0)) {
              const Real e0 = row[b];
              const Real w = __ldg(wr + b);
              const Real pe = gw.x * a[i][b] * hh;
              if (sr[b]) {
                t2 += pe * pe * w;
                t1 += e0 * pe * w;
              } else {
                const Real qc = c.bdt / (fabs(e0) * sqrt(w));
                t2 += qc * (pe * pe * w);
                t1 += qc * (e0 * pe * w);
              }
            }
          }
        } else {
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
    }
  }
  const Real theta1 = -group_sum<G>(t1);
  const Real theta2 = group_sum<G>(t2);
  // bracket (find_min_max, UpdateVoxels.cpp:47-63)
  Real lo = Real(0), hi = Real(0);
#pragma unroll
  for (int i = 0; i < NNB; ++i) {
    lo = nb[i] < lo ? nb[i] : lo;
    hi = nb[i] > hi ? nb[i] : hi;
  }
  lo = group_min<G>(lo);
  hi = group_max<G>(hi);
  if (theta2 != Real(0)) {
    const Real cand = V - theta1 / theta2;
    lo = lo > cand ? cand : lo;
    hi = hi < cand ? cand : hi;
  }
  // QGGMRF surrogate, one iteration (QGGMRF_Functions.cpp:153-206)
  s1 = group_sum<G>(s1);
  s2 = group_sum<G>(s2);
  const Real u = (s1 + theta2 * V - theta1) / (s2 + theta2);
  Real nv = V + c.pc->alpha * (u - V);
  nv = (nv < lo) ? lo : ((nv > hi) ? hi : nv);
  if (nv < Real(0)) nv = Real(0);  // positivity (UpdateVoxels.cpp:394-400, BFConstants.h)
  const Real dlt = nv - V;
  if (!live) return;
  // error-sinogram scatter (UpdateVoxels.cpp:423-449).  BF re-evaluates the selector of every
  // footprint entry even when the voxel did not change (BFForwardModel.cpp:898-932), so the
  // scatter runs then too.
  if (BF || dlt != Real(0)) {
    if (one_row) {
      const Real hh = c.hv[0];
#pragma unroll
      for (int i = 0; i < VPL; ++i) {
        const int v = gl + G * i;
        if (v >= g.n_theta) continue;
        const Real gain = c.sgw[v].x;
#pragma unroll
        for (int b = 0; b < NB; ++b)
          if (a[i][b] > Real(0)) {
            const Real ne = ev[i][b] - gain * (a[i][b] * hh * dlt);
            c.es[eidx[i] + b] = ne;
            if constexpr (BF)
              c.bs[v * c.bs_rs + jlo[i] + b] = bragg_selected<Real>(ne, wv[i][b], c.bt);
          }
      }
    } else {
#pragma unroll
      for (int i = 0; i < VPL; ++i) {
        const int v = gl + G * i;
        if (v >= g.n_theta) continue;
        const Real gain = c.sgw[v].x;
        for (int tr = 0; tr < c.tcount; ++tr) {
          const Real hh = c.hv[tr];
          Real* row = c.es + tr * c.ps + v * c.rs + jlo[i];
          if constexpr (BF) {
            const Real* wr = c.bw + tr * c.bw_ps + v * c.bw_rs + jlo[i];
            uint8_t* sr = c.bs + tr * c.bs_ps + v * c.bs_rs + jlo[i];
#pragma unroll
            for (int b = 0; b < NB; ++b)
              if (a[i][b] > Real(0)) {
                const Real ne = row[b] - gain * (a[i][b] * hh * dlt);
                row[b] = ne;
                sr[b] = bragg_selected<Real>(ne, __ldg(wr + b), c.bt);
              }
          } else {
#pragma unroll
            for (int b = 0; b < NB; ++b)
              if (a[i][b] > Real(0)) row[b] -= gain * (a[i][b] * hh * dlt);
          }
        }
      }
    }
  }
  if (gl == 0) {
    c.vol[vidx] = nv;
    if (c.cache) c.cache[4 * g.n_x + x] = nv;
    if (x >= g.roi_x0 && x <= g.roi_x1 && z >= g.roi_z0 && z <= g.roi_z1) {
      acc.v[0] += fix32<Real>(dlt);
      acc.v[1] += fix32<Real>(V);
    }
    acc.v[3] += 1;
    if constexpr (BF) {
      if (c.mag_fx != nullptr && dlt != Real(0))
        atomicAdd(c.mag_fx + static_cast<size_t>(z) * g.n_x + x,
                  fix32<Real>(dlt));
    }
  }
}

struct SmemLayout {
  size_t bar, ctl, stats, rb, bx, bxd, gw, H, hv, list, cls, okr, lv, flat, gofs, bits, cache, es,
      sel, total;
};

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr int kMaxGroups = kWarps * 32 / 16;  // voxel groups per CTA at G = 16

// n_sp > 0: the slice's selector rows are staged too (bright field).  sched: a scheduled call
// (no detector-response table, no row-walk lists or neighbour cache), which leaves more of the
// SM's L1 to the per-entry weights it gathers.
__host__ __device__ inline SmemLayout smem_layout(int n_theta, int n_x, int n_rs, int t_rows,
                                                  int bins, bool stage, size_t real_bytes,
                                                  int n_sp, bool sched = false) {
  if (sched) {
    n_x = 0;
    bins = -1;
  }
  SmemLayout L;
  size_t o = 0;
  L.bar = o;
  o += 16;
  L.ctl = o;  // class counters [2], zero-skip counter
  o += 16;
  L.stats = o;
  o += sizeof(unsigned long long) * kMaxGroups * kStatSlots;
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
  o = align_up(o + real_bytes * kMaxTRows, 16);
  L.list = o;  // class segments of the current row: S * ceil(n_x / S) <= 2 n_x + 2 slots
  o = align_up(o + sizeof(int) * (2 * static_cast<size_t>(n_x) + 2), 16);
  L.cls = o;   // candidates per class (S <= max(n_x, 2))
  o = align_up(o + sizeof(int) * (static_cast<size_t>(n_x) + 2), 16);
  L.okr = o;   // row flags: non-empty A-column and in the call's line list
  o = align_up(o + static_cast<size_t>(n_x), 16);
  L.lv = o;    // row flags: bit 0 live at row start, bit 1 live-or-reachable (period prefix)
  o = align_up(o + static_cast<size_t>(n_x), 16);
  L.flat = o;  // the row's candidates in step order
  o = align_up(o + sizeof(int) * (static_cast<size_t>(n_x) + 2), 16);
  L.gofs = o;  // step offsets into flat
  o = align_up(o + sizeof(int) * (static_cast<size_t>(n_x) + 4), 16);
  L.bits = o;  // candidates of the step being formed, one bit per x
  o = align_up(o + sizeof(unsigned) * ((static_cast<size_t>(n_x) + 31) / 32 + 2), 16);
  L.cache = o;
  o = align_up(o + real_bytes * 9 * static_cast<size_t>(n_x), 128);
  L.es = o;
  if (stage) o += real_bytes * static_cast<size_t>(t_rows) * n_theta * n_rs;
  o = align_up(o, 16);
  L.sel = o;
  if (stage && n_sp > 0) o += static_cast<size_t>(t_rows) * n_theta * n_sp;
  L.total = align_up(o, 16);
  return L;
}

// One voxel slice y of one reconstruction, processed by the whole CTA: stage the slice's
// detector rows (and, for bright field, its selector rows), walk the z-rows, update every
// conflict-free class, store the rows back.  Each class is first compacted: its candidate
// voxels that are updated (non-empty A-column, in the call's line list, not zero-skipped) are
// appended to a shared list, and the CTA's voxel groups then take the list in turns, so
// skipped voxels cost one thread's neighbour test instead of a group iteration.  Voxels of a
// class are independent (no shared detector bin, no prior neighbours), so the order in which
// the list is filled does not change any result.
// `phase` is the parity of the CTA's mbarrier (it alternates when a CTA processes several
// slices); `coherent` makes neighbour-row loads bypass L1 (needed when other CTAs of the same
// launch write neighbouring slices).  Writes the slice's four statistics to stat_out when it
// is not null.  Returns false when a bounded wait gave up (A.err is set).
template <typename Real, int NB, int G, int VPL, bool STAGE, bool BF>
__device__ __forceinline__ bool run_slice(const SweepArgs& A, int y, unsigned char* smem,
                                          uint32_t& phase, bool coherent, double* stat_out) {
  using R2 = typename V2<Real>::type;
  const DevGeom& g = A.g;
  const int tid = threadIdx.x, nthreads = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  constexpr int GPW = 32 / G;  // voxel groups per warp
  const int group = warp * GPW + (lane / G);
  const int n_groups = (nthreads / 32) * GPW;
  const int tcount = A.tab.t_count[y], tfirst = A.tab.t_first[y];
  const int n_sp = BF ? A.bfa.n_sp : 0;
  const bool sched_layout = BF && std::is_same<Real, float>::value && A.sched_lines != nullptr &&
                            A.acol != nullptr && A.mode != kModeProject;
  const SmemLayout L = smem_layout(g.n_theta, g.n_x, A.n_rs, tcount, g.bins, STAGE, sizeof(Real),
                                   n_sp, sched_layout);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L.bar);
  unsigned* ctl = reinterpret_cast<unsigned*>(smem + L.ctl);
  unsigned long long* sstat = reinterpret_cast<unsigned long long*>(smem + L.stats);
  RowBase<Real>* rb = reinterpret_cast<RowBase<Real>*>(smem + L.rb);
  float2* sbx = reinterpret_cast<float2*>(smem + L.bx);
  double* sbxd = reinterpret_cast<double*>(smem + L.bxd);
  R2* sgw = reinterpret_cast<R2*>(smem + L.gw);
  Real* sH = reinterpret_cast<Real*>(smem + L.H);
  Real* shv = reinterpret_cast<Real*>(smem + L.hv);
  int* list = reinterpret_cast<int*>(smem + L.list);
  Real* cache = reinterpret_cast<Real*>(smem + L.cache);
  const Real* gH = static_cast<const Real*>(A.tab.H);
  const R2* ggw = static_cast<const R2*>(A.tab.gw);
  const Real* ghv = static_cast<const Real*>(A.tab.hval);
  Real* const ge = static_cast<Real*>(A.e);
  Real* const gx = static_cast<Real*>(A.x);
  constexpr bool kF32 = std::is_same<Real, float>::value;

  __shared__ PriorConst<Real> s_pc;
  __shared__ Real s_qf[27];
  if (tid == 0) s_pc = prior_const<Real>(A.flt, A.g);
  if (tid < 27) s_qf[tid] = static_cast<Real>(A.flt.f[tid]);
  if (!sched_layout)  // scheduled calls read the A-column from its table
    for (int i = tid; i < g.n_theta * (g.bins + 1); i += nthreads) sH[i] = gH[i];
  for (int v = tid; v < g.n_theta; v += nthreads) {
    if (kF32)
      sbx[v] = A.tab.bx[v];
    else
      sbxd[v] = A.tab.bxd[v];
    sgw[v] = ggw[v];
  }
  if (tid < kMaxTRows) shv[tid] = ghv[y * kMaxTRows + tid];
  if (tid < 4) ctl[tid] = 0u;
  __syncthreads();  // constants and tables visible before any path uses them

  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  const size_t sel_plane = static_cast<size_t>(g.n_theta) * n_sp;
  Real* es;
  uint8_t* ssel = nullptr;
  int rs, ps, srs = 0, sps = 0;
  const int rows = tcount * g.n_theta;
  const uint32_t row_bytes = static_cast<uint32_t>(g.n_rp * sizeof(Real));
  if (STAGE) {
    es = reinterpret_cast<Real*>(smem + L.es);
    rs = A.n_rs;
    ps = g.n_theta * A.n_rs;
    if (BF) {
      ssel = smem + L.sel;
      srs = n_sp;
      sps = g.n_theta * n_sp;
    }
    if (A.mode == kModeProject) {
      for (int i = tid; i < tcount * ps; i += nthreads) es[i] = Real(0);
      __syncthreads();
    } else {
      const uint32_t total = static_cast<uint32_t>(rows) * (row_bytes + (BF ? n_sp : 0));
      if (tid == 0) mbar_expect_tx(bar, total);
      __syncthreads();
      for (int r = tid; r < rows; r += nthreads) {
        const int tr = r / g.n_theta, v = r % g.n_theta;
        bulk_g2s(es + tr * ps + v * rs,
                 ge + (static_cast<size_t>(tfirst + tr)) * sino_plane +
                     static_cast<size_t>(v) * g.n_rp,
                 row_bytes, bar);
        if (BF)
          bulk_g2s(ssel + tr * sps + v * srs,
                   A.bfa.sel + (static_cast<size_t>(tfirst + tr)) * sel_plane +
                       static_cast<size_t>(v) * n_sp,
                   static_cast<uint32_t>(n_sp), bar);
      }
      const bool ok = mbar_wait(bar, phase);
      phase ^= 1u;
      if (!__syncthreads_and(ok)) {
        if (tid == 0) atomicOr(A.err, 1);
        mbar_wait(bar, phase ^ 1u);  // give copies still in flight a second bounded chance
        return false;
      }
    }
  } else {
    es = ge + static_cast<size_t>(tfirst) * sino_plane;
    rs = g.n_rp;
    ps = static_cast<int>(sino_plane);
    if (BF) {
      ssel = A.bfa.sel + static_cast<size_t>(tfirst) * sel_plane;
      srs = n_sp;
      sps = static_cast<int>(sel_plane);
    }
  }

  SliceCtx<Real> c;
  c.g = &A.g;
  c.q = &A.flt;
  c.vol = gx;
  c.es = es;
  c.rs = rs;
  c.ps = ps;
  c.rb = rb;
  c.sH = sH;
  c.sbx = kF32 ? sbx : nullptr;
  c.sbxd = kF32 ? nullptr : sbxd;
  c.sgw = sgw;
  c.hv = shv;
  c.lineok = A.tab.lineok;
  c.cache = cache;
  c.tcount = tcount;
  c.mode = A.mode;
  c.iter_nonzero = A.iter_nonzero;
  c.zero_skipping = A.zero_skipping;
  c.bw = nullptr;
  c.bs = nullptr;
  c.mag_fx = nullptr;
  c.bw_rs = c.bw_ps = c.bs_rs = c.bs_ps = 0;
  c.bt = c.bdt = Real(0);
  c.acol = nullptr;
  c.coherent = coherent;
  c.pc = &s_pc;
  c.qf = s_qf;
  if (BF) {
    c.bw = static_cast<const Real*>(A.bfa.w) + static_cast<size_t>(tfirst) * sino_plane;
    c.bw_rs = g.n_rp;
    c.bw_ps = static_cast<int>(sino_plane);
    c.bs = ssel;
    c.bs_rs = srs;
    c.bs_ps = sps;
    c.bt = static_cast<Real>(A.bfa.bragg_t);
    c.bdt = static_cast<Real>(A.bfa.bragg_dt);
    c.mag_fx = A.bfa.mag_fx;
  }
  const uint8_t* active_lines = BF ? A.bfa.active : nullptr;
  int* cls = reinterpret_cast<int*>(smem + L.cls);
  int* flat = reinterpret_cast<int*>(smem + L.flat);
  int* gofs = reinterpret_cast<int*>(smem + L.gofs);
  unsigned* bits = reinterpret_cast<unsigned*>(smem + L.bits);
  uint8_t* okr = smem + L.okr;
  uint8_t* lv = smem + L.lv;
  const int S = A.stride;
  const int cap = (g.n_x + S - 1) / S;
  const bool project = A.mode == kModeProject;
  const bool zs_on = !project && A.zero_skipping && A.iter_nonzero;
  c.inline_zs = zs_on ? 1 : 0;

  const size_t vplane = static_cast<size_t>(g.n_z) * g.n_x;
  GroupAcc acc;
#pragma unroll
  for (int s2 = 0; s2 < kStatSlots; ++s2) acc.v[s2] = 0ull;
  unsigned skipped = 0;
  // Level schedule: the call's lines level by level, one CTA barrier per level; neighbours are
  // read from the volume (the slice's own plane is written only by this CTA, the planes y+-1
  // belong to the other colour and do not change during the launch), the zero-skipping test
  // runs at the visit, and the A-column comes from the table.
  bool scheduled = false;
  if constexpr (kF32 && BF) {  // only bright-field NHICD calls are scheduled
    if (A.sched_lines != nullptr && A.acol != nullptr && !project) {
      scheduled = true;
      c.cache = nullptr;
      c.acol = A.acol;
      const int n_levels = A.sched_count != nullptr ? __ldg(A.sched_count + 1) : A.n_levels;
      const int n_sl = __ldg(A.sched_lofs + n_levels);
      // the schedule (offsets, lines as z << 16 | x) in shared memory when it fits: after the
      // layout (the launch's room for it), or else in the row walk's lists, which this path
      // does not use
      const size_t sched_ints = static_cast<size_t>(n_levels) + 1 + n_sl;
      const size_t dyn = dynamic_smem_bytes();
      int* s_lofs = nullptr;
      int* s_zx = nullptr;
      if (L.total + sched_ints * sizeof(int) <= dyn)
        s_lofs = reinterpret_cast<int*>(smem + L.total);
      else if (sched_ints <= (L.es - L.list) / sizeof(int))
        s_lofs = reinterpret_cast<int*>(smem + L.list);
      if (s_lofs != nullptr) {
        s_zx = s_lofs + n_levels + 1;
        for (int i = tid; i <= n_levels; i += nthreads) s_lofs[i] = __ldg(A.sched_lofs + i);
        for (int i = tid; i < n_sl; i += nthreads) {
          const int l = __ldg(A.sched_lines + i);
          const int z = l / g.n_x;
          s_zx[i] = (z << 16) | (l - z * g.n_x);
        }
        __syncthreads();
      }
      for (int lv = 0; lv < n_levels; ++lv) {
        const int b = s_lofs ? s_lofs[lv] : __ldg(A.sched_lofs + lv);
        const int n = (s_lofs ? s_lofs[lv + 1] : __ldg(A.sched_lofs + lv + 1)) - b;
        for (int b0 = 0; b0 < n; b0 += n_groups) {
          const int i = b0 + group;
          const bool act = i < n;
          int z = 0, x = 0;
          if (act) {
            if (s_zx) {
              const int zx = s_zx[b + i];
              z = zx >> 16;
              x = zx & 0xffff;
            } else {
              const int l = __ldg(A.sched_lines + b + i);
              z = l / g.n_x;
              x = l - z * g.n_x;
            }
          }
          group_step<Real, NB, G, VPL, BF, false, true>(c, z, x, y, act, lane, acc);
        }
        __syncthreads();
      }
    }
  }
  for (int rr = 0; !scheduled && rr < g.n_z; ++rr) {
    const int z = A.row_order[rr];
    __syncthreads();
    compute_row_base<Real>(A.tab, g.n_theta, z, rb, tid, nthreads);
    // neighbour rows (y+dy, z+dz), dy, dz in {-1,0,1} (rows outside the volume read as 0),
    // loaded column by column: each thread also records whether its column holds a value > 0
    // (bit 2 of lv), from which the zero-skipping test of every voxel follows
    for (int x = tid; x < g.n_x; x += nthreads) {
      bool pos = false;
#pragma unroll
      for (int r = 0; r < 9; ++r) {
        const int yy = y + r / 3 - 1, zz = z + r % 3 - 1;
        Real v = Real(0);
        if (yy >= 0 && yy < g.n_y && zz >= 0 && zz < g.n_z) {
          const Real* src = gx + static_cast<size_t>(yy) * vplane + static_cast<size_t>(zz) * g.n_x + x;
          v = coherent ? __ldcg(src) : *src;
        }
        cache[r * g.n_x + x] = v;
        pos |= v > Real(0);
      }
      const size_t l = static_cast<size_t>(z) * g.n_x + x;
      okr[x] = (A.tab.lineok[l] && (active_lines == nullptr || active_lines[l])) ? 1 : 0;
      lv[x] = pos ? 4 : 0;
    }
    __syncthreads();
    // liveness at the start of the row (bit 0): projection needs V != 0; an ICD voxel that would
    // be zero-skipped now (V == 0, no neighbour > 0) is not live.  A voxel skipped at the start
    // of its row can still be updated if a same-row neighbour processed before it became
    // positive: within a stride period [mS, mS+S) classes run left to right, so reachability
    // is the period's prefix-OR, and the period's last voxel also follows the next period's
    // first one.  Bit 1 marks the candidates.  One thread per period.
    int any_cand = 0;
    for (int m = tid; m * S < g.n_x; m += nthreads) {
      const int x0 = m * S;
      const int x1 = min(x0 + S, g.n_x);
      auto live_at = [&](int x) -> int {
        if (!okr[x]) return 0;
        const Real V = cache[4 * g.n_x + x];
        if (project) return V != Real(0);
        if (!zs_on || V != Real(0)) return 1;
        const bool nbpos = (lv[x] & 4) || (x > 0 && (lv[x - 1] & 4)) ||
                           (x + 1 < g.n_x && (lv[x + 1] & 4));
        return nbpos ? 1 : 0;
      };
      int a = 0;
      for (int x = x0; x < x1; ++x) {
        const int l0 = live_at(x);
        a |= l0;
        int cand = zs_on ? a : l0;
        if (zs_on && x == x0 + S - 1 && x + 1 < g.n_x) cand |= live_at(x + 1);
        cand &= okr[x];
        any_cand |= cand;
        lv[x] = static_cast<uint8_t>((lv[x] & 4) | l0 | (cand << 1));
      }
    }
    if (!__syncthreads_or(any_cand)) {
      // nothing in this row can be updated: count its listed voxels as skipped
      if (!project)
        for (int x = tid; x < g.n_x; x += nthreads) skipped += okr[x];
      continue;
    }
    // compaction: warp w lists the candidates of classes w, w + warps, ... in ascending x
    for (int k = warp; k < S; k += nthreads / 32) {
      int base = 0;
      for (int m0 = 0; k + S * m0 < g.n_x; m0 += 32) {
        const int x = k + S * (m0 + lane);
        bool cand = false;
        if (x < g.n_x && okr[x]) {
          cand = ((lv[x] >> 1) & 1) != 0;
          if (!cand && !project) ++skipped;
        }
        const unsigned b = __ballot_sync(kFull, cand);
        if (cand) list[k * cap + base + __popc(b & ((1u << lane) - 1u))] = x;
        base += __popc(b);
      }
      if (lane == 0) cls[k] = base;
    }
    __syncthreads();
    // Dense rows: once a class holds more than 8 candidates, consecutive classes practically
    // always have candidates within S of each other and would not merge; each non-empty class
    // becomes a step as it is (class order, the same result as merged steps), the class lists
    // copied into the step list by all threads instead of the one-warp merge pass.
    int cmax = 0;
    for (int k = 0; k < S; ++k) cmax = max(cmax, static_cast<int>(cls[k]));
    const bool dense = cmax > 8;
    if (dense) {
      int off = 0, ns = 0;
      for (int k = 0; k < S; ++k) {
        const int n = cls[k];
        if (n == 0) continue;
        if (tid == 0) gofs[ns] = off;
        for (int j = tid; j < n; j += nthreads) flat[off + j] = list[k * cap + j];
        off += n;
        ++ns;
      }
      if (tid == 0) {
        gofs[ns] = off;
        ctl[0] = static_cast<unsigned>(ns);
      }
    }
    // Steps: consecutive classes are merged while none of the next class's candidates lies
    // within S of a candidate already in the step.  Voxels of one step are then pairwise
    // independent (no shared detector bin, no prior neighbours, no zero-skipping influence),
    // and independent updates commute, so a step gives exactly the result of running its
    // classes in order.  One warp forms the steps in class order.
    if (!dense && warp == 0) {
      const int words = (g.n_x + 31) >> 5;
      for (int w = lane; w < words; w += 32) bits[w] = 0u;
      __syncwarp();
      int ns = 0, nf = 0, step0 = 0;
      if (lane == 0) gofs[0] = 0;
      for (int k = 0; k < S; ++k) {
        const int n = cls[k];
        if (n == 0) continue;
        bool conf = false;
        for (int j = lane; j < n && !conf; j += 32) {
          const int x = list[k * cap + j];
          const int lo = max(x - S + 1, 0), hi = min(x + S - 1, g.n_x - 1);
          for (int w = lo >> 5; w <= (hi >> 5); ++w) {
            const int a = max(lo - (w << 5), 0), b = min(hi - (w << 5), 31);
            const unsigned mask =
                (b - a == 31) ? 0xffffffffu : (((1u << (b - a + 1)) - 1u) << a);
            if (bits[w] & mask) conf = true;
          }
        }
        if (__any_sync(kFull, conf) && nf > step0) {
          // close the step: clear the words holding its candidates, open the next one
          for (int j = step0 + lane; j < nf; j += 32) bits[flat[j] >> 5] = 0u;
          ++ns;
          step0 = nf;
          if (lane == 0) gofs[ns] = nf;
          __syncwarp();
        }
        for (int j = lane; j < n; j += 32) {
          const int x = list[k * cap + j];
          flat[nf + j] = x;
          atomicOr(&bits[x >> 5], 1u << (x & 31));
        }
        nf += n;
        __syncwarp();
      }
      if (lane == 0) {
        gofs[ns + 1] = nf;
        ctl[0] = static_cast<unsigned>(ns + 1);
      }
    }
    __syncthreads();
    const int n_steps = static_cast<int>(ctl[0]);
    for (int st = 0; st < n_steps; ++st) {
      const int b = gofs[st], n = gofs[st + 1] - b;
      for (int b0 = 0; b0 < n; b0 += n_groups) {
        const int i = b0 + group;
        const bool act = i < n;
        group_step<Real, NB, G, VPL, BF, false>(c, z, act ? flat[b + i] : 0, y, act, lane, acc);
      }
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
      if (BF && A.mode != kModeProject)
        bulk_s2g(A.bfa.sel + (static_cast<size_t>(tfirst + tr)) * sel_plane +
                     static_cast<size_t>(v) * n_sp,
                 ssel + tr * sps + v * srs, static_cast<uint32_t>(n_sp));
    }
    bulk_commit();
    bulk_wait_all();
  }
  if (stat_out != nullptr) {
    const int gl = lane & (G - 1);
    if (gl == 0)
      for (int s = 0; s < kStatSlots; ++s) sstat[group * kStatSlots + s] = acc.v[s];
    if (skipped) atomicAdd(ctl + 2, skipped);
    __syncthreads();
    if (tid < kStatSlots) {
      unsigned long long t = 0;
      for (int w = 0; w < n_groups; ++w) t += sstat[w * kStatSlots + tid];
      if (tid == 2) t += ctl[2];
      stat_out[tid] = tid < 2 ? static_cast<double>(t) / kFixScale : static_cast<double>(t);
    }
  }
  __syncthreads();
  return true;
}

__device__ __forceinline__ void init_slice_barrier(unsigned char* smem) {
  if (threadIdx.x == 0) {
    mbar_init(reinterpret_cast<uint64_t*>(smem), 1);
    fence_mbar_init();
  }
  __syncthreads();
}

// One launch = the slices of one y-colour of one reconstruction, one CTA per slice.
template <typename Real, int NB, int G, int VPL, bool STAGE, bool BF>
__global__ void __launch_bounds__(kWarps * 32, 1) sweep_kernel(SweepArgs A) {
  extern __shared__ __align__(128) unsigned char smem[];
  // slab launches (y_end > 0) start at y_first; whole-volume launches at the colour
  const int y = (A.y_end > 0 ? A.y_first : A.colour) + 2 * static_cast<int>(blockIdx.x);
  if (y >= (A.y_end > 0 ? A.y_end : A.g.n_y)) return;
  init_slice_barrier(smem);
  uint32_t phase = 0;
  run_slice<Real, NB, G, VPL, STAGE, BF>(
      A, y, smem, phase, false,
      A.stats != nullptr ? A.stats + static_cast<size_t>(blockIdx.x) * kStatSlots : nullptr);
}

// One slice of a batched series with its staging.
template <int NB, int G, int VPL, bool BF>
__device__ __forceinline__ void batch_slice(const SweepArgs& sA, int y, unsigned char* smem,
                                            uint32_t& phase, double* stat_out) {
  if (sA.smem_rows)
    run_slice<float, NB, G, VPL, true, BF>(sA, y, smem, phase, true, stat_out);
  else
    run_slice<float, NB, G, VPL, false, BF>(sA, y, smem, phase, true, stat_out);
}

// Many reconstructions of uneven size in one persistent launch per sweep (FP32).  CTAs pull
// (series, slice) items from a queue: first every colour-0 slice, then every colour-1 slice.
// A colour-1 slice needs the colour-0 neighbours y+-1 of its own series, so it waits (with a
// time bound) until all colour-0 slices of that series are done; those were taken from the
// queue earlier by running CTAs, so the wait always ends.  Launched cooperatively so every CTA
// is resident.  One launch covers the series of one voxel-group shape; it may use 256 threads
// per CTA (two CTAs per SM under the 128-register cap) or 512.  Bright-field and HAADF series
// run in separate launches.
template <int NB, int G, int VPL, bool BF>
__global__ void __launch_bounds__(kWarps * 32, 1) batch_sweep_kernel(BatchArgs B) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ SweepArgs sA;
  __shared__ int s_item;
  __shared__ int s_wait_ok;
  init_slice_barrier(smem);
  uint32_t phase = 0;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(B.queue, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= B.n_items) break;
    const int2 it = B.items[item];
    const int s = it.x, y = it.y;
    if (threadIdx.x == 0) {
      sA = B.series[s];
      int ok = 1;
      if (y & 1) {
        const uint64_t t0 = global_ns();
        unsigned ns = 64;
        for (;;) {
          int done;
          asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(done) : "l"(B.done + s) : "memory");
          if (done >= B.need[s]) break;
          if (global_ns() - t0 > B.wait_ns) {
            ok = 0;
            atomicOr(B.series[s].err, 2);
            break;
          }
          __nanosleep(ns);
          if (ns < 4096) ns <<= 1;
        }
      }
      s_wait_ok = ok;
    }
    __syncthreads();
    if (!s_wait_ok) continue;
    const int n0 = (sA.g.n_y + 1) / 2;
    const int slot = (y & 1) ? n0 + (y >> 1) : (y >> 1);
    double* stat_out = sA.stats + static_cast<size_t>(slot) * kStatSlots;
    batch_slice<NB, G, VPL, BF>(sA, y, smem, phase, stat_out);
    if (threadIdx.x == 0 && !(y & 1)) {
      __threadfence();
      atomicAdd(B.done + s, 1);
    }
  }
}

// The reference's visit order: voxel lines one after another in list order, y ascending
// (UpdateYSlice::execute / BFUpdateYSlice::execute with one task), one warp, error sinogram in
// HBM.  BF: the lines' update magnitudes restart at 0 (BFUpdateYSlice.cpp:171).
template <typename Real, int NB, int VPL, bool BF>
__global__ void __launch_bounds__(32, 1) ref_order_kernel(RefOrderArgs A) {
  using R2 = typename V2<Real>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  const DevGeom& g = A.g;
  const int lane = threadIdx.x;
  const SmemLayout L = smem_layout(g.n_theta, 0, 0, 0, g.bins, false, sizeof(Real), 0);
  RowBase<Real>* rb = reinterpret_cast<RowBase<Real>*>(smem + L.rb);
  float2* sbx = reinterpret_cast<float2*>(smem + L.bx);
  double* sbxd = reinterpret_cast<double*>(smem + L.bxd);
  R2* sgw = reinterpret_cast<R2*>(smem + L.gw);
  Real* sH = reinterpret_cast<Real*>(smem + L.H);
  const Real* gH = static_cast<const Real*>(A.tab.H);
  const R2* ggw = static_cast<const R2*>(A.tab.gw);
  const Real* ghv = static_cast<const Real*>(A.tab.hval);
  constexpr bool kF32 = std::is_same<Real, float>::value;
  __shared__ PriorConst<Real> s_pc;
  __shared__ Real s_qf[27];
  if (lane == 0) s_pc = prior_const<Real>(A.flt, A.g);
  if (lane < 27) s_qf[lane] = static_cast<Real>(A.flt.f[lane]);
  for (int i = lane; i < g.n_theta * (g.bins + 1); i += 32) sH[i] = gH[i];
  for (int v = lane; v < g.n_theta; v += 32) {
    if (kF32)
      sbx[v] = A.tab.bx[v];
    else
      sbxd[v] = A.tab.bxd[v];
    sgw[v] = ggw[v];
  }
  __syncwarp();
  SliceCtx<Real> c;
  c.g = &A.g;
  c.q = &A.flt;
  c.vol = static_cast<Real*>(A.x);
  c.rs = g.n_rp;
  c.ps = g.n_theta * g.n_rp;
  c.rb = rb;
  c.sH = sH;
  c.sbx = kF32 ? sbx : nullptr;
  c.sbxd = kF32 ? nullptr : sbxd;
  c.sgw = sgw;
  c.lineok = A.tab.lineok;
  c.cache = nullptr;
  c.mode = kModeICD;
  c.iter_nonzero = A.iter_nonzero;
  c.zero_skipping = A.zero_skipping;
  c.inline_zs = 1;
  c.bw = nullptr;
  c.bs = nullptr;
  c.mag_fx = nullptr;
  c.bw_rs = c.bw_ps = c.bs_rs = c.bs_ps = 0;
  c.bt = c.bdt = Real(0);
  c.acol = nullptr;
  c.coherent = false;
  c.pc = &s_pc;
  c.qf = s_qf;
  Real* const ge = static_cast<Real*>(A.e);
  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  const size_t sel_plane = BF ? static_cast<size_t>(g.n_theta) * A.bfa.n_sp : 0;
  if (BF) {
    c.bw_rs = g.n_rp;
    c.bw_ps = static_cast<int>(sino_plane);
    c.bs_rs = A.bfa.n_sp;
    c.bs_ps = static_cast<int>(sel_plane);
    c.bt = static_cast<Real>(A.bfa.bragg_t);
    c.bdt = static_cast<Real>(A.bfa.bragg_dt);
    c.mag_fx = A.bfa.mag_fx;
  }
  GroupAcc acc;
#pragma unroll
  for (int s = 0; s < kStatSlots; ++s) acc.v[s] = 0ull;
  for (int n = 0; n < A.n_lines; ++n) {
    const int l = A.lines[n];
    const int z = l / g.n_x, x = l % g.n_x;
    if (BF && c.mag_fx != nullptr && lane == 0) c.mag_fx[l] = 0ull;
    __syncwarp();
    compute_row_base<Real>(A.tab, g.n_theta, z, rb, lane, 32);
    __syncwarp();
    for (int y = 0; y < g.n_y; ++y) {
      c.es = ge + static_cast<size_t>(A.tab.t_first[y]) * sino_plane;
      c.tcount = A.tab.t_count[y];
      c.hv = ghv + y * kMaxTRows;
      if (BF) {
        c.bw = static_cast<const Real*>(A.bfa.w) + static_cast<size_t>(A.tab.t_first[y]) * sino_plane;
        c.bs = A.bfa.sel + static_cast<size_t>(A.tab.t_first[y]) * sel_plane;
      }
      group_step<Real, NB, 32, VPL, BF, true>(c, z, x, y, true, lane, acc);
      __syncwarp();
    }
  }
  if (lane == 0)
    for (int s = 0; s < kStatSlots; ++s)
      A.stats[s] = s < 2 ? static_cast<double>(acc.v[s]) / kFixScale : static_cast<double>(acc.v[s]);
}

// A-column table of every voxel line (z, x): per view the first bin and the NB footprint
// values, by the same arithmetic (and compile flags) as the in-kernel A-column of group_step,
// so a sweep that reads the table gives the same bits as one that computes it.
template <int NB>
__global__ void acol_kernel(DevGeom g, DevTables tab, float4* __restrict__ out) {
  constexpr int AW = acol_width(NB);
  const size_t n = static_cast<size_t>(g.n_z) * g.n_x * g.n_theta;
  const float hw = static_cast<float>(g.half_width);
  const float* H = static_cast<const float*>(tab.H);
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int v = static_cast<int>(i % g.n_theta);
    const size_t l = i / g.n_theta;
    const int z = static_cast<int>(l / g.n_x), x = static_cast<int>(l % g.n_x);
    int j0;
    float f;
    detector_pos(x, row_base<float>(tab, z, v), tab.bx[v], 0.0, j0, f);
    const float u = static_cast<float>(j0) + f;
    int jlo = 0;
    float a[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) a[b] = 0.f;
    if (!(u + hw < 0.f || u - hw > static_cast<float>(g.n_r)))
      view_footprint<float, NB>(g, hw, static_cast<float>(g.kr), H + v * (g.bins + 1), j0, f,
                                jlo, a);
    float t[AW * 4];
#pragma unroll
    for (int k = 0; k < AW * 4; ++k) t[k] = 0.f;
    t[0] = __int_as_float(jlo);
#pragma unroll
    for (int b = 0; b < NB; ++b) t[1 + b] = a[b];
#pragma unroll
    for (int w = 0; w < AW; ++w)
      out[i * AW + w] = make_float4(t[4 * w], t[4 * w + 1], t[4 * w + 2], t[4 * w + 3]);
  }
}

inline int ok_or(cudaError_t e) { return e == cudaSuccess ? 0 : -3; }

inline int launch_acol_t(const DevGeom& g, const DevTables& tab, int nb, float4* out,
                         cudaStream_t s) {
  const size_t n = static_cast<size_t>(g.n_z) * g.n_x * g.n_theta;
  const int grid = static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16));
  if (nb == 3)
    acol_kernel<3><<<grid, 256, 0, s>>>(g, tab, out);
  else if (nb == 5)
    acol_kernel<5><<<grid, 256, 0, s>>>(g, tab, out);
  else if (nb == 9)
    acol_kernel<9><<<grid, 256, 0, s>>>(g, tab, out);
  else
    return -7;
  return ok_or(cudaGetLastError());
}

template <typename Real, int NB, int G, int VPL, bool STAGE, bool BF>
int launch_sweep_t(const SweepArgs& a, size_t smem, cudaStream_t s) {
  auto k = sweep_kernel<Real, NB, G, VPL, STAGE, BF>;
  static const int lim = dyn_smem_limit(k);
  if (smem > static_cast<size_t>(lim)) return -3;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if (e != cudaSuccess) return -3;
  // shared-memory carveout just large enough for this launch: the rest of the SM's unified
  // L1/shared storage caches the gathered weights and neighbour rows
  static int per_sm = 0;
  if (per_sm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  }
  if (per_sm > 0) {
    const int pct = static_cast<int>(std::min<size_t>(100, (100 * (smem + 4096) + per_sm - 1) / per_sm));
    cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
  }
  k<<<a.n_slices, kWarps * 32, smem, s>>>(a);
  return ok_or(cudaGetLastError());
}
template <typename Real, int NB, int G, int VPL, bool STAGE>
int launch_sweep_m(const SweepArgs& a, size_t smem, cudaStream_t s) {
  return a.bf ? launch_sweep_t<Real, NB, G, VPL, STAGE, true>(a, smem, s)
              : launch_sweep_t<Real, NB, G, VPL, STAGE, false>(a, smem, s);
}

template <int NB, int G, int VPL, bool BF>
int launch_batch_t(const BatchArgs& b, size_t smem, int grid, int threads, cudaStream_t s) {
  auto k = batch_sweep_kernel<NB, G, VPL, BF>;
  static const int lim = dyn_smem_limit(k);
  if (smem > static_cast<size_t>(lim)) return -3;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if (e != cudaSuccess) return -3;
  if (threads != 256 && threads != kWarps * 32) threads = kWarps * 32;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem) != cudaSuccess ||
      per_sm < 1)
    return -3;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (grid <= 0 || grid > per_sm * sms) grid = per_sm * sms;
  BatchArgs arg = b;
  void* params[] = {&arg};
  e = cudaLaunchCooperativeKernel(reinterpret_cast<void*>(k), dim3(grid), dim3(threads), params,
                                  smem, s);
  return ok_or(e);
}

template <typename Real, int NB, int VPL>
int launch_ref_t(const RefOrderArgs& a, cudaStream_t s) {
  const size_t smem = smem_layout(a.g.n_theta, 0, 0, 0, a.g.bins, false, sizeof(Real), 0).total;
  auto launch = [&](auto kern) {
    const int lim = dyn_smem_limit(kern);
    if (smem > static_cast<size_t>(lim)) return -3;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return -3;
    kern<<<1, 32, smem, s>>>(a);
    return ok_or(cudaGetLastError());
  };
  return a.bf ? launch(ref_order_kernel<Real, NB, VPL, true>)
              : launch(ref_order_kernel<Real, NB, VPL, false>);
}

// FP32 sweep launch for one (STAGE, BF) pair: NB (footprint bins) and the lane shape select
// the instantiation.
template <bool STAGE, bool BF>
int launch_sweep_f32_pick(const SweepArgs& a, int nb, size_t smem, cudaStream_t s) {
  // explicit shape (1..4) when it covers the views, else the default for the view count
  const int shape = resolved_shape(a.shape, a.g.n_theta);
  if constexpr (!STAGE) {  // more than 160 views: 32 lanes x 8 views, slices in HBM
    if (shape == 5) {
      if (nb == 3) return launch_sweep_t<float, 3, 32, 8, STAGE, BF>(a, smem, s);
      if (nb == 5) return launch_sweep_t<float, 5, 32, 8, STAGE, BF>(a, smem, s);
      if (nb == 9) return launch_sweep_t<float, 9, 32, 8, STAGE, BF>(a, smem, s);
      return -7;
    }
  } else {
    if (shape == 5) return -7;
  }
  if (nb == 9) return launch_sweep_t<float, 9, 32, 5, STAGE, BF>(a, smem, s);
  if (nb == 3) {
    if (shape == 1) return launch_sweep_t<float, 3, 16, 4, STAGE, BF>(a, smem, s);
    if (shape == 2) return launch_sweep_t<float, 3, 32, 2, STAGE, BF>(a, smem, s);
    if (shape == 3) return launch_sweep_t<float, 3, 32, 3, STAGE, BF>(a, smem, s);
    return launch_sweep_t<float, 3, 32, 5, STAGE, BF>(a, smem, s);
  }
  if (nb == 5) {
    if (shape == 1) return launch_sweep_t<float, 5, 16, 4, STAGE, BF>(a, smem, s);
    if (shape == 2) return launch_sweep_t<float, 5, 32, 2, STAGE, BF>(a, smem, s);
    if (shape == 3) return launch_sweep_t<float, 5, 32, 3, STAGE, BF>(a, smem, s);
    return launch_sweep_t<float, 5, 32, 5, STAGE, BF>(a, smem, s);
  }
  return -7;
}

// group = 2 * (shape - 1) + bf: the voxel-group shape of every series in the launch (1 = 16x4,
// 2 = 32x2, 3 = 32x3, 4 = 32x5) and whether they are bright field
template <int NB, bool BF>
int launch_batch_shape(const BatchArgs& b, int shape, int threads, size_t smem, int grid,
                       cudaStream_t s) {
  if (shape == 1) return launch_batch_t<NB, 16, 4, BF>(b, smem, grid, threads, s);
  if (shape == 2) return launch_batch_t<NB, 32, 2, BF>(b, smem, grid, threads, s);
  if (shape == 3) return launch_batch_t<NB, 32, 3, BF>(b, smem, grid, threads, s);
  return launch_batch_t<NB, 32, 5, BF>(b, smem, grid, threads, s);
}
template <int NB>
int launch_batch_pick(const BatchArgs& b, int group, int threads, size_t smem, int grid,
                      cudaStream_t s) {
  return (group & 1) ? launch_batch_shape<NB, true>(b, group / 2 + 1, threads, smem, grid, s)
                     : launch_batch_shape<NB, false>(b, group / 2 + 1, threads, smem, grid, s);
}

}  // namespace sweep
}  // namespace mbir
