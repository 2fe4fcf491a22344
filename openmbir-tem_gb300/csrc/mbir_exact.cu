// mbir_exact.cu -- reference-exact FP64 kernels (compiled with -fmad=false).
//
// ICD iterates of this algorithm are chaotic with respect to rounding: the zero-skipping test
// and the positivity/bracket clips turn last-bit differences into whole-voxel differences, so
// even two FP64 runs that only sum theta1 in a different order drift apart by ~3e-4 after five
// outer iterations.  To reproduce the reference's iterates, this mode performs every
// floating-point operation of the reference path in the reference's order and association:
//   * A-matrix values by the formula of AMatrixCol.cpp:148-232 (r = x cos - z sin, ...);
//   * forward projection summed voxel line by voxel line in (z, x) order
//     (HAADF_ForwardProject.cpp:94-118), one thread per measurement;
//   * theta1/theta2 and the surrogate sums accumulated sequentially in the reference's entry and
//     neighbour order (_UpdateVoxels.cpp:343-369, QGGMRF_Functions.cpp:170-190);
//   * per-view sums of jointEstimation / updateWeights sequentially over r then t
//     (_Extra.cpp:474-517, :825-833);
//   * powers by a pinned double-double method instead of a math library's pow (the oracle
//     evaluates them the same way in this mode).
// Only the elementwise parts run in parallel.  It is a parity mode, not a fast path.
#include <cuda_runtime.h>

#include <algorithm>

#include "mbir_internal.h"

namespace mbir {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kPerView = 9;                 // bins per view for delta_xz <= 4 delta_r
constexpr int kMaxEntries = kPerView * 160;  // A-column entries of one voxel line

struct ExactCol {
  int n;
  int idx[kMaxEntries];   // theta * n_r + r
  double val[kMaxEntries];
};

// AMatrixCol::calculateAMatrixColumnPartial for view i of voxel (row, col): appends the view's
// entries (value > 0) in ascending bin order.  Returns the number written.
__device__ int amatrix_view(const ExactArgs& A, int row, int col, int i, int* idx, double* val) {
  const DevGeom& g = A.g;
  const double x = A.x0 + (static_cast<double>(col) + 0.5) * A.delta_xz;
  const double z = A.z0 + (static_cast<double>(row) + 0.5) * A.delta_xz;
  const double r = x * A.cosv[i] - z * A.sinv[i];
  const double rmin = r - A.delta_xz, rmax = r + A.delta_xz;
  if (rmax < A.R0 || rmin > A.RMax) return 0;
  int imin = static_cast<int>(floor(((rmin - A.R0) / A.delta_r)));
  int imax = static_cast<int>(floor((rmax - A.R0) / A.delta_r));
  if (imax >= g.n_r) imax = g.n_r - 1;
  if (imin < 0) imin = 0;
  const double* H = A.H + static_cast<size_t>(i) * g.bins;
  int n = 0;
  for (int j = imin; j <= imax; j++) {
    const double rc = (A.R0 + ((static_cast<double>(j)) + 0.5) * (A.delta_r));
    const double dr = fabs(r - rc);
    const int idr = static_cast<int>(floor((dr / A.offset_r)));
    if (idr >= 0 && idr < g.bins) {
      const double w1 = dr - idr * A.offset_r;
      const double w2 = (idr + 1) * A.offset_r - dr;
      const int ii = idr + 1 < g.bins ? idr + 1 : g.bins - 1;
      const double f1 = (w2 / A.offset_r) * H[idr] + (w1 / A.offset_r) * H[ii];
      if (f1 > 0) {
        idx[n] = i * g.n_r + j;
        val[n] = f1;
        n++;
      }
    }
  }
  return n;
}

// Builds the ordered A-column of voxel line (row, col) in shared memory with one warp.
__device__ void build_column(const ExactArgs& A, int row, int col, ExactCol* c) {
  const int lane = threadIdx.x & 31;
  int base = 0;
  for (int v0 = 0; v0 < A.g.n_theta; v0 += 32) {
    const int v = v0 + lane;
    int li[kPerView];
    double lv[kPerView];
    int n = 0;
    if (v < A.g.n_theta) n = amatrix_view(A, row, col, v, li, lv);
    int incl = n;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += t;
    }
    const int off = base + incl - n;
    for (int k = 0; k < n; k++) {
      c->idx[off + k] = li[k];
      c->val[off + k] = lv[k];
    }
    base += __shfl_sync(kFull, incl, 31);
  }
  if (lane == 0) c->n = base;
  __syncwarp();
}

// ---- pinned power function ------------------------------------------------------------
// The reference calls the C library's pow; its last bit differs between libraries (and
// from CUDA's pow), and the iterates amplify that.  This mode evaluates x^y by double-double
// arithmetic built from IEEE add/mul/div only (Knuth two-sum; Dekker exact product with
// Veltkamp splitting; this file is compiled without fused multiply-adds):
//   ln x = k ln2 + 2 atanh(s), s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)), by the power series
//   of atanh to s^45;  e^t = 2^k (1 + expm1(r)), expm1 by its Taylor series at r/256 to the
//   14th power followed by eight doublings expm1(2u) = expm1(u) (2 + expm1(u)).
// The result is the double nearest to x^y except within ~1e-30 of a rounding boundary.
struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD dd(double hi, double lo = 0.0) { return DD{hi, lo}; }
__device__ __forceinline__ DD two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return DD{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DD fast_sum(double a, double b) {
  const double s = a + b;
  return DD{s, b - (s - a)};
}
__device__ __forceinline__ void vsplit(double a, double& hi, double& lo) {
  const double t = 134217729.0 * a;  // 2^27 + 1
  hi = t - (t - a);
  lo = a - hi;
}
__device__ __forceinline__ DD two_prod(double a, double b) {
  const double p = a * b;
  double ah, al, bh, bl;
  vsplit(a, ah, al);
  vsplit(b, bh, bl);
  return DD{p, (((ah * bh) - p) + (ah * bl) + (al * bh)) + (al * bl)};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  const DD t = two_sum(a.lo, b.lo);
  s.lo = s.lo + t.hi;
  s = fast_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return fast_sum(s.hi, s.lo);
}
__device__ __forceinline__ DD dd_mul(DD a, DD b) {
  DD p = two_prod(a.hi, b.hi);
  p.lo = p.lo + ((a.hi * b.lo) + (a.lo * b.hi));
  return fast_sum(p.hi, p.lo);
}
__device__ DD dd_div(DD a, DD b) {
  const double q1 = a.hi / b.hi;
  DD r = dd_add(a, dd_mul(b, dd(-q1)));
  const double q2 = r.hi / b.hi;
  r = dd_add(r, dd_mul(b, dd(-q2)));
  const double q3 = r.hi / b.hi;
  return dd_add(fast_sum(q1, q2), dd(q3));
}
constexpr double kLn2Hi = 6.93147180559945286227e-01;  // ln 2 = kLn2Hi + kLn2Lo
constexpr double kLn2Lo = 2.31904681384629955842e-17;

__device__ DD dd_log(double x) {
  int k;
  double m = frexp(x, &k);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    k = k - 1;
  }
  const DD s = dd_div(dd(m - 1.0), two_sum(m, 1.0));
  const DD s2 = dd_mul(s, s);
  DD acc = dd_div(dd(1.0), dd(45.0));
  for (int n = 21; n >= 0; n--) acc = dd_add(dd_mul(acc, s2), dd_div(dd(1.0), dd(2.0 * n + 1.0)));
  const DD lm = dd_mul(dd_mul(s, acc), dd(2.0));
  return dd_add(dd_mul(DD{kLn2Hi, kLn2Lo}, dd(static_cast<double>(k))), lm);
}
__device__ double dd_exp(DD t) {
  const double kf = floor(t.hi / kLn2Hi + 0.5);
  DD r = dd_add(t, dd_mul(DD{kLn2Hi, kLn2Lo}, dd(-kf)));
  r.hi = ldexp(r.hi, -8);
  r.lo = ldexp(r.lo, -8);
  DD term = r, sum = r;
  for (int n = 2; n <= 14; n++) {
    term = dd_div(dd_mul(term, r), dd(static_cast<double>(n)));
    sum = dd_add(sum, term);
  }
  for (int i = 0; i < 8; i++) sum = dd_mul(sum, dd_add(sum, dd(2.0)));
  sum = dd_add(sum, dd(1.0));
  return ldexp(sum.hi, static_cast<int>(kf));
}
__device__ double pinned_pow(double x, double y) {
  if (y == 0.0) return 1.0;
  if (x == 0.0) return 0.0;
  if (y == 1.0) return x;
  return dd_exp(dd_mul(dd_log(x), dd(y)));
}

// rho'(d)/d exactly as QGGMRF::Derivative (QGGMRF_Functions.cpp:90-104) divided by d
__device__ double exact_coef(const DevFilter& q, double d0) {
  if (d0 == 0) return q.mrf_p / (q.sig_p * q.mrf_c);
  const double P = q.mrf_p, Q = q.mrf_q;
  const double t1 = pinned_pow(fabs(d0), P - Q) / q.sig_pq;
  const double t2 = pinned_pow(fabs(d0), P - 1);
  const double t3 = q.mrf_c + t1;
  double der;
  if (d0 < 0)
    der = ((-1 * t2 / (t3 * q.sig_p)) * (P - ((P - Q) * t1) / (t3)));
  else
    der = ((t2 / (t3 * q.sig_p)) * (P - ((P - Q) * t1) / (t3)));
  return der / d0;
}

__global__ void __launch_bounds__(32, 1) exact_icd_kernel(ExactArgs A) {
  __shared__ ExactCol col;
  __shared__ double ev[kMaxEntries * 2];  // e values of the column for up to two t rows
  __shared__ double nbs[27];
  __shared__ double prm[27];
  __shared__ unsigned char bfl[27];
  __shared__ double s_new;
  __shared__ int s_skip;
  const DevGeom& g = A.g;
  const int lane = threadIdx.x;
  double* vol = A.x;   // [y][z][x]
  double* e = A.e;     // [t][theta][n_rp]
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  double st[kStatSlots] = {0, 0, 0, 0};
  const size_t sel_plane = A.bf ? static_cast<size_t>(g.n_theta) * A.n_sp : 0;
  for (int n = 0; n < A.n_lines; ++n) {
    const int l = A.lines[n];
    const int jn = l / g.n_x, kn = l % g.n_x;
    if (A.bf && lane == 0) A.mag[l] = 0;  // BFUpdateYSlice.cpp:171
    build_column(A, jn, kn, &col);
    if (col.n == 0) continue;
    for (int i = 0; i < g.n_y; ++i) {
      // neighbourhood (UpdateVoxels.cpp:283-306), flags as the reference sets them
      if (lane < 27) {
        const int p = lane / 9 - 1, q = (lane / 3) % 3 - 1, r = lane % 3 - 1;
        double v = 0;
        unsigned char f = 0;
        if (i + p >= 0 && i + p < g.n_y && jn + q >= 0 && jn + q < g.n_z && kn + r >= 0 &&
            kn + r < g.n_x) {
          v = vol[static_cast<size_t>(i + p) * plane + static_cast<size_t>(jn + q) * g.n_x + kn + r];
          f = 1;
        }
        if (lane == 13) v = 0;
        nbs[lane] = v;
        bfl[lane] = f;
      }
      __syncwarp();
      const size_t vidx = static_cast<size_t>(i) * plane + static_cast<size_t>(jn) * g.n_x + kn;
      const double V = vol[vidx];
      if (lane == 0) {
        int skip = 0;
        if (A.zero_skipping == 1 && V == 0.0 && A.iter_nonzero) {
          skip = 1;
          for (int a = 0; a < 27; a++)
            if (nbs[a] > 0.0) skip = 0;
        }
        s_skip = skip;
      }
      __syncwarp();
      if (s_skip) {
        if (lane == 0) st[2] += 1;
        __syncwarp();
        continue;
      }
      const int t0 = A.t_first[i], tc = A.t_count[i];
      const double* hv = A.hval + i * kMaxTRows;
      // gather the column's error-sinogram values (read only; summed in order below)
      const bool pre = tc <= 2;
      if (pre)
        for (int q = lane; q < col.n; q += 32) {
          const int id = col.idx[q];
          const int th = id / g.n_r, r = id % g.n_r;
          for (int a = 0; a < tc; a++)
            ev[q * 2 + a] = e[static_cast<size_t>(t0 + a) * sino_plane +
                              static_cast<size_t>(th) * g.n_rp + r];
        }
      // surrogate coefficients in parallel (independent per neighbour)
      if (lane < 27) {
        const int a = lane;
        prm[a] = (a != 13 && bfl[a] == 1) ? exact_coef(A.flt, V - nbs[a]) : 0.0;
      }
      __syncwarp();
      if (lane == 0) {
        // theta1 / theta2 in the reference's order
        double th1 = 0.0, th2 = 0.0;
        for (int q = 0; q < col.n; q++) {
          const int id = col.idx[q];
          const int th = id / g.n_r, r = id % g.n_r;
          const double k0 = A.gain[th] * (col.val[q]);
          for (int a = 0; a < tc; a++) {
            const size_t ei = static_cast<size_t>(t0 + a) * sino_plane +
                              static_cast<size_t>(th) * g.n_rp + r;
            const double evv = pre ? ev[q * 2 + a] : e[ei];
            if (A.bf) {
              // BFForwardModel::computeTheta (BFForwardModel.cpp:866-887)
              const double w = A.bw[ei];
              const size_t si = static_cast<size_t>(t0 + a) * sel_plane +
                                static_cast<size_t>(th) * A.n_sp + r;
              if (A.bsel[si] == 1) {
                const double pe = k0 * hv[a];
                th2 += (pe * pe * w);
                th1 += (evv * pe * w);
              } else {
                const double qc = (A.bragg_delta * A.bragg_t) / (fabs(evv) * sqrt(w));
                const double pe = k0 * hv[a];
                th2 += qc * (pe * pe * w);
                th1 += qc * (evv * pe * w);
              }
            } else {
              double pe = k0 * hv[a];
              if (A.bfm) pe *= A.bfm[ei];  // with bright-field data (_UpdateVoxels.cpp:358-364)
              th2 += (pe * pe * A.weight[th]);
              th1 += (evv * pe * A.weight[th]);
            }
          }
        }
        th1 *= -1;
        double low = nbs[0], high = nbs[0];
        for (int a = 0; a < 27; a++) {
          if (nbs[a] < low) low = nbs[a];
          if (nbs[a] > high) high = nbs[a];
        }
        if (th2 != 0) {
          low = (low > (V - (th1 / th2)) ? (V - (th1 / th2)) : low);
          high = (high < (V - (th1 / th2)) ? (V - (th1 / th2)) : high);
        }
        double temp1 = 0, temp2 = 0;
        for (int a = 0; a < 27; a++) {
          if (a != 13 && bfl[a] == 1) {
            const double tcst = A.flt.f[a] * prm[a];
            temp1 += tcst * nbs[a];
            temp2 += tcst;
          }
        }
        const double u = (temp1 + (th2 * V) - th1) / (temp2 + th2);
        double nv = V + A.flt.mrf_alpha * (u - V);
        nv = (nv < low) ? low : ((nv > high) ? high : nv);
        if (nv < 0.0) nv = 0.0;
        s_new = nv;
        vol[vidx] = nv;
        if (A.bf) A.mag[l] = A.mag[l] + fabs(nv - V);
        if (kn >= g.roi_x0 && kn <= g.roi_x1 && jn >= g.roi_z0 && jn <= g.roi_z1) {
          st[0] += fabs(nv - V);
          st[1] += fabs(V);
        }
        st[3] += 1;
      }
      __syncwarp();
      const double nv = s_new;
      // scatter: every entry is written once, so entries can be updated in parallel
      for (int q = lane; q < col.n; q += 32) {
        const int id = col.idx[q];
        const int th = id / g.n_r, r = id % g.n_r;
        for (int a = 0; a < tc; a++) {
          const size_t ei = static_cast<size_t>(t0 + a) * sino_plane +
                            static_cast<size_t>(th) * g.n_rp + r;
          const double k2 = (A.gain[th] * (col.val[q] * hv[a] * (nv - V)));
          if (A.bfm)
            e[ei] -= (A.bfm[ei] * k2);  // with bright-field data (_UpdateVoxels.cpp:442-446)
          else
            e[ei] -= k2;
          if (A.bf) {  // BFForwardModel::updateErrorSinogram (BFForwardModel.cpp:921-929)
            const size_t si = static_cast<size_t>(t0 + a) * sel_plane +
                              static_cast<size_t>(th) * A.n_sp + r;
            A.bsel[si] = (fabs(e[ei] * sqrt(A.bw[ei])) < A.bragg_t) ? 1 : 0;
          }
        }
      }
      __syncwarp();
    }
  }
  if (lane == 0)
    for (int s = 0; s < kStatSlots; ++s) A.stats[s] = st[s];
}

// Y_Est of HAADF_ForwardProject::operator() (HAADF_ForwardProject.cpp:94-118), one thread per
// measurement (theta, r, t), terms added in the reference's (z, x) order.
__global__ void exact_project_kernel(ExactArgs A, double* yest) {
  const DevGeom& g = A.g;
  const size_t total = static_cast<size_t>(g.n_t) * g.n_theta * g.n_r;
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  for (size_t w = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; w < total;
       w += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int j = static_cast<int>(w % g.n_r);
    const int th = static_cast<int>((w / g.n_r) % g.n_theta);
    const int t = static_cast<int>(w / (static_cast<size_t>(g.n_r) * g.n_theta));
    double acc = 0.0;
    // slices whose voxel-line response covers row t
    for (int i = 0; i < g.n_y; i++) {
      const int a = t - A.t_first[i];
      if (a < 0 || a >= A.t_count[i]) continue;
      const double h = A.hval[i * kMaxTRows + a];
      for (int z = 0; z < g.n_z; z++) {
        // voxels whose footprint can reach bin j at this view: |r - Rc(j)| < delta_xz + delta_r
        const double zc = A.z0 + (static_cast<double>(z) + 0.5) * A.delta_xz;
        const double rcj = A.R0 + (static_cast<double>(j) + 0.5) * A.delta_r;
        const double c = A.cosv[th], s = A.sinv[th];
        int xlo = 0, xhi = g.n_x - 1;
        if (fabs(c) > 1e-12) {
          const double xa = (rcj + zc * s - (A.delta_xz + A.delta_r)) / c;
          const double xb = (rcj + zc * s + (A.delta_xz + A.delta_r)) / c;
          const double lo = fmin(xa, xb), hi = fmax(xa, xb);
          xlo = max(0, static_cast<int>(floor((lo - A.x0) / A.delta_xz - 0.5)) - 1);
          xhi = min(g.n_x - 1, static_cast<int>(ceil((hi - A.x0) / A.delta_xz - 0.5)) + 1);
        }
        for (int x = xlo; x <= xhi; x++) {
          if (!A.lineok[static_cast<size_t>(z) * g.n_x + x]) continue;
          int idx[kPerView];
          double val[kPerView];
          const int n = amatrix_view(A, z, x, th, idx, val);
          for (int k = 0; k < n; k++)
            if (idx[k] == th * g.n_r + j) {
              const double xv = A.x[static_cast<size_t>(i) * plane + static_cast<size_t>(z) * g.n_x + x];
              acc += (A.gain[th] * (val[k] * h * xv));
            }
        }
      }
    }
    yest[(static_cast<size_t>(t) * g.n_theta + th) * g.n_rp + j] = acc;
  }
}

// Sequential per-view sums in the reference's order (r outer, t inner).  kind 0: the six
// jointEstimation sums, kind 1: sum e^2 * 1 of updateWeights.
__global__ void exact_view_sums_kernel(ExactArgs A, int kind, const double* y, const double* mu,
                                       double* out) {
  const DevGeom& g = A.g;
  const int th = blockIdx.x * blockDim.x + threadIdx.x;
  if (th >= g.n_theta) return;
  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  if (kind == 1) {
    double sum = 0;
    for (int r = 0; r < g.n_r; r++)
      for (int t = 0; t < g.n_t; t++) {
        const double ev = A.e[static_cast<size_t>(t) * sino_plane + static_cast<size_t>(th) * g.n_rp + r];
        sum += (ev * ev * 1.0);
      }
    out[th] = sum;
    return;
  }
  double a = 0, b = 0, cc = 0, d = 0, num = 0, den = 0;
  const double wv = A.weight[th];
  for (int r = 0; r < g.n_r; r++)
    for (int t = 0; t < g.n_t; t++) {
      const size_t i = static_cast<size_t>(t) * sino_plane + static_cast<size_t>(th) * g.n_rp + r;
      const double yv = y[i];
      double ye = yv - A.e[i] - mu[th];
      ye /= A.gain[th];
      num += (yv * wv);
      den += (wv);
      a += (ye * wv);
      b += (ye * wv * yv);
      cc += (yv * yv * wv);
      d += (ye * ye * wv);
    }
  out[th * 6 + 0] = num;
  out[th * 6 + 1] = den;
  out[th * 6 + 2] = a;
  out[th * 6 + 3] = b;
  out[th * 6 + 4] = cc;
  out[th * 6 + 5] = d;
}

// calculateMeasurementWeight's error with bright-field data (_Extra.cpp:722-727):
// e = y - m Y_Est - mu, one thread per measurement
__global__ void exact_bfa_error_kernel(ExactArgs A, const double* y, const double* yest,
                                       const double* mu) {
  const DevGeom& g = A.g;
  const size_t total = static_cast<size_t>(g.n_t) * g.n_theta * g.n_rp;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % g.n_rp);
    const int v = static_cast<int>((i / g.n_rp) % g.n_theta);
    A.e[i] = (r < g.n_r) ? y[i] - A.bfm[i] * yest[i] - mu[v] : 0.0;
  }
}

// jointEstimation with bright-field data, offsets only (_Extra.cpp:643-668): per view (one
// thread) the error's weighted mean over r then t, taken off the error and added to mu
__global__ void exact_bfa_offsets_kernel(ExactArgs A, double* mu) {
  const DevGeom& g = A.g;
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.n_theta) return;
  const size_t plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  const double w = A.weight[v];
  double num_sum = 0, den_sum = 0;
  for (int r = 0; r < g.n_r; r++)
    for (int t = 0; t < g.n_t; t++) {
      const size_t i = static_cast<size_t>(t) * plane + static_cast<size_t>(v) * g.n_rp + r;
      num_sum += (A.e[i] * w);
      den_sum += w;
    }
  const double a = num_sum / den_sum;
  for (int r = 0; r < g.n_r; r++)
    for (int t = 0; t < g.n_t; t++)
      A.e[static_cast<size_t>(t) * plane + static_cast<size_t>(v) * g.n_rp + r] -= a;
  mu[v] += a;
}

}  // namespace

int launch_exact_bfa_error(const ExactArgs& a, const double* y, const double* yest,
                           const double* mu, void* stream) {
  const size_t n = static_cast<size_t>(a.g.n_t) * a.g.n_theta * a.g.n_rp;
  const int grid = static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16));
  exact_bfa_error_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, y, yest, mu);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_exact_bfa_offsets(const ExactArgs& a, double* mu, void* stream) {
  exact_bfa_offsets_kernel<<<(a.g.n_theta + 63) / 64, 64, 0, static_cast<cudaStream_t>(stream)>>>(
      a, mu);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_exact_icd(const ExactArgs& a, void* stream) {
  exact_icd_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_exact_project(const ExactArgs& a, double* yest, void* stream) {
  const size_t total = static_cast<size_t>(a.g.n_t) * a.g.n_theta * a.g.n_r;
  int grid = static_cast<int>((total + 127) / 128);
  if (grid > 152 * 16) grid = 152 * 16;
  exact_project_kernel<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(a, yest);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_exact_view_sums(const ExactArgs& a, int kind, const double* y, const double* mu,
                           double* out, void* stream) {
  exact_view_sums_kernel<<<(a.g.n_theta + 63) / 64, 64, 0, static_cast<cudaStream_t>(stream)>>>(
      a, kind, y, mu, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace mbir
