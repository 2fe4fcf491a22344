/*
 * mbir_oracle.c -- CPU restatement (FP64) of OpenMBIR-TEM's HAADF reconstruction path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GB300 engine.  Loaded by tests/, by
 * __graft_entry__.smoke() and by the cpu_baseline leg of bench.py; never by the product.
 *
 * All paths below are relative to the reference project root (Code/MBIRLib/...).
 * Arithmetic is FP64 throughout, in the reference's loop order, so that the restatement
 * reproduces the reference bit for bit: it is pinned to the reference's own programs built from
 * their sources (mbir_oracle.h says how).
 */
#include "mbir_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define M_PI_2_ (M_PI / 2.0)
#define M_PI_4_ (M_PI / 4.0)

#define IDX3(i, j, k) (9 * (i) + 3 * (j) + (k))

/* 26-neighbour prior weights, indexed [dy+1][dz+1][dx+1]
 * (HAADF/HAADF_ReconstructionEngine.cpp:266-294, same table in _UpdateVoxels.cpp:556-585). */
static const double k_filter[27] = {
  0.0302, 0.0370, 0.0302, 0.0370, 0.0523, 0.0370, 0.0302, 0.0370, 0.0302,
  0.0370, 0.0523, 0.0370, 0.0523, 0.0000, 0.0523, 0.0370, 0.0523, 0.0370,
  0.0302, 0.0370, 0.0302, 0.0370, 0.0523, 0.0370, 0.0302, 0.0370, 0.0302};

struct orc_ctx {
  orc_params p;
  int n_theta, n_r, n_t;
  double delta_r, delta_t, R0, RMax, T0, TMax;
  int n_x, n_y, n_z;
  double delta_xz, delta_xy, x0, y0, z0, length_x, length_y, length_z;
  double offset_r, offset_t;
  double* angles_deg;
  double* cosv;
  double* sinv;
  double* profile;
  double* beam;
  double* H;
  double* Ht;
  int* vlr_first;
  int* vlr_count;
  double* vlr_val; /* [n_y][vlr_cap] */
  int vlr_cap;
  int* col_start;
  int* col_count;
  int* col_index;
  double* col_val;
  double* counts;
  double* x;
  double* e;
  double* w;
  double* yest;
  double* I;
  double* mu;
  double* alpha;
  double* init_gain;
  double* init_offset;
  double* init_var;
  unsigned char* mask;
  double* mag_map;
  double sig_p, sig_pq, sig_q;
  /* bright field */
  unsigned char* sel;  /* Bragg selector [n_theta][n_r][n_t] */
  double* filt_map;    /* VSC-filtered mag map [n_z][n_x] */
  double bragg_t;      /* current Bragg threshold T */
  int counts_logged;   /* processRawCounts applied */
  /* HAADF with bright-field data: the bright-field counts + BF_OFFSET [n_theta][n_r][n_t]
   * (NULL without) */
  double* bfm;
};

/* ---------------------------------------------------------------------------------------
 * Pinned power function.  The reference calls the C library's pow, whose last bit differs
 * between libraries (and from CUDA's); ICD iterates amplify such differences.  With
 * pinned_pow set, x^y is evaluated here by double-double arithmetic from plain IEEE
 * additions, multiplications and divisions only (Knuth's two-sum, Dekker's exact product with
 * Veltkamp splitting): ln x = k ln2 + 2 atanh((m-1)/(m+1)) by its power series, and
 * e^t = 2^k (1 + expm1(r)) with expm1 by its Taylor series at r/256 followed by eight
 * doublings expm1(2u) = expm1(u) (2 + expm1(u)).  The result is the double nearest to
 * x^y except in cases closer than ~1e-30 to a rounding boundary, and is the same on every
 * machine that does not fuse multiply-adds.
 * ------------------------------------------------------------------------------------- */
typedef struct {
  double hi, lo;
} dd_t;

static dd_t dd_make(double hi, double lo) {
  dd_t r;
  r.hi = hi;
  r.lo = lo;
  return r;
}
static dd_t dd_two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  return dd_make(s, (a - (s - bb)) + (b - bb));
}
static dd_t dd_fast_sum(double a, double b) {
  double s = a + b;
  return dd_make(s, b - (s - a));
}
static void dd_split(double a, double* hi, double* lo) {
  double t = 134217729.0 * a; /* 2^27 + 1 */
  *hi = t - (t - a);
  *lo = a - *hi;
}
static dd_t dd_two_prod(double a, double b) {
  double p = a * b, ah, al, bh, bl;
  dd_split(a, &ah, &al);
  dd_split(b, &bh, &bl);
  return dd_make(p, (((ah * bh) - p) + (ah * bl) + (al * bh)) + (al * bl));
}
static dd_t dd_add(dd_t a, dd_t b) {
  dd_t s = dd_two_sum(a.hi, b.hi);
  dd_t t = dd_two_sum(a.lo, b.lo);
  s.lo = s.lo + t.hi;
  s = dd_fast_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return dd_fast_sum(s.hi, s.lo);
}
static dd_t dd_mul(dd_t a, dd_t b) {
  dd_t p = dd_two_prod(a.hi, b.hi);
  p.lo = p.lo + ((a.hi * b.lo) + (a.lo * b.hi));
  return dd_fast_sum(p.hi, p.lo);
}
static dd_t dd_div(dd_t a, dd_t b) {
  double q1 = a.hi / b.hi;
  dd_t r = dd_add(a, dd_mul(b, dd_make(-q1, 0.0)));
  double q2 = r.hi / b.hi;
  r = dd_add(r, dd_mul(b, dd_make(-q2, 0.0)));
  double q3 = r.hi / b.hi;
  return dd_add(dd_fast_sum(q1, q2), dd_make(q3, 0.0));
}
static const double kLn2Hi = 6.93147180559945286227e-01; /* ln 2 = kLn2Hi + kLn2Lo */
static const double kLn2Lo = 2.31904681384629955842e-17;

static dd_t dd_log(double x) { /* x > 0 and finite */
  int k;
  double m = frexp(x, &k);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    k = k - 1;
  }
  dd_t s = dd_div(dd_make(m - 1.0, 0.0), dd_two_sum(m, 1.0));
  dd_t s2 = dd_mul(s, s);
  dd_t acc = dd_div(dd_make(1.0, 0.0), dd_make(45.0, 0.0));
  for (int n = 21; n >= 0; n--)
    acc = dd_add(dd_mul(acc, s2), dd_div(dd_make(1.0, 0.0), dd_make(2.0 * n + 1.0, 0.0)));
  dd_t lm = dd_mul(dd_mul(s, acc), dd_make(2.0, 0.0));
  return dd_add(dd_mul(dd_make(kLn2Hi, kLn2Lo), dd_make((double)k, 0.0)), lm);
}
static double dd_exp(dd_t t) {
  double kf = floor(t.hi / kLn2Hi + 0.5);
  dd_t r = dd_add(t, dd_mul(dd_make(kLn2Hi, kLn2Lo), dd_make(-kf, 0.0)));
  r.hi = ldexp(r.hi, -8);
  r.lo = ldexp(r.lo, -8);
  dd_t term = r, sum = r;
  for (int n = 2; n <= 14; n++) {
    term = dd_div(dd_mul(term, r), dd_make((double)n, 0.0));
    sum = dd_add(sum, term);
  }
  for (int i = 0; i < 8; i++) sum = dd_mul(sum, dd_add(sum, dd_make(2.0, 0.0)));
  sum = dd_add(sum, dd_make(1.0, 0.0));
  return ldexp(sum.hi, (int)kf);
}
double orc_pinned_pow(double x, double y) {
  if (y == 0.0) return 1.0;
  if (x == 0.0) return 0.0;
  if (y == 1.0) return x;
  return dd_exp(dd_mul(dd_log(x), dd_make(y, 0.0)));
}

static double q_pow(const orc_ctx* c, double x, double y) {
  return c->p.pinned_pow ? orc_pinned_pow(x, y) : pow(x, y);
}

/* ---------------------------------------------------------------------------------------
 * QGGMRF prior (Reconstruction/QGGMRF_Functions.cpp:82-206)
 * ------------------------------------------------------------------------------------- */
static double q_value(const orc_ctx* c, double delta) {
  /* QGGMRF_Functions.cpp:82-85 */
  return (q_pow(c, fabs(delta), c->p.mrf_p) / c->sig_p) /
         (c->p.mrf_c + q_pow(c, fabs(delta), c->p.mrf_p - c->p.mrf_q) / c->sig_pq);
}

static double q_derivative(const orc_ctx* c, double delta) {
  /* QGGMRF_Functions.cpp:90-104 */
  double P = c->p.mrf_p, Q = c->p.mrf_q;
  double t1 = q_pow(c, fabs(delta), P - Q) / c->sig_pq;
  double t2 = q_pow(c, fabs(delta), P - 1);
  double t3 = c->p.mrf_c + t1;
  if (delta < 0) return ((-1 * t2 / (t3 * c->sig_p)) * (P - ((P - Q) * t1) / (t3)));
  return ((t2 / (t3 * c->sig_p)) * (P - ((P - Q) * t1) / (t3)));
}

static double q_second_at_zero(const orc_ctx* c) {
  /* QGGMRF_Functions.cpp:109-112 */
  return c->p.mrf_p / (c->sig_p * c->p.mrf_c);
}

static double clip(double x, double a, double b) { return (x < a) ? a : ((x > b) ? b : x); }

/* QGGMRF::FunctionalSubstitution with QGGMRF_ITER = 1 (QGGMRF_Functions.cpp:153-206);
 * ComputeParameters inlined (:118-147).  umin is NOT clamped at zero: POSITIVITY_CONSTRAINT
 * is not visible in that translation unit. */
static double q_substitution(const orc_ctx* c, double umin, double umax, double V,
                             const unsigned char* bf, const double* nb, double theta1,
                             double theta2) {
  double ref = V, temp1 = 0, temp2 = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) {
        int id = IDX3(i, j, k);
        if ((i != 1 || j != 1 || k != 1) && bf[id] == 1) {
          double d0 = ref - nb[id];
          double prm = (d0 != 0) ? q_derivative(c, d0) / d0 : q_second_at_zero(c);
          double tc = k_filter[id] * prm;
          temp1 += tc * nb[id];
          temp2 += tc;
        }
      }
  double u = (temp1 + (theta2 * V) - theta1) / (temp2 + theta2);
  return clip(ref + c->p.mrf_alpha * (u - ref), umin, umax);
}

/* ---------------------------------------------------------------------------------------
 * Geometry and tables
 * ------------------------------------------------------------------------------------- */

/* GenericFilters/InitialReconstructionInitializer.cpp:98-167 (non-FORWARD_PROJECT_MODE) and
 * the sinogram extents of GenericFilters/MRCSinogramInitializer.cpp:302-305. */
static void geometry_init(orc_ctx* c) {
  const orc_params* p = &c->p;
  c->R0 = -(c->n_r * c->delta_r) / 2;
  c->RMax = (c->n_r * c->delta_r) / 2;
  c->T0 = -(c->n_t * c->delta_t) / 2;
  c->TMax = (c->n_t * c->delta_t) / 2;

  c->delta_xz = c->delta_r * p->delta_xz_factor;
  c->delta_xy = c->delta_xz;
  double mx = fabs(c->angles_deg[0]);
  for (int i = 1; i < c->n_theta; i++)
    if (fabs(c->angles_deg[i]) > mx) mx = fabs(c->angles_deg[i]);
  if (mx > 75.0) mx = 75.0; /* ReconstructionConstants.h:80 k_MaxAngleStretch */
  mx = mx * M_PI / 180.0;
  double lz = p->length_z;
  lz *= p->z_stretch;
  lz /= (p->interpolate_factor * c->delta_r);
  lz = floor(lz + 0.5) * p->interpolate_factor * c->delta_r;
  c->length_z = lz;
  c->length_x = c->n_r * c->delta_r;
  if (p->extend_object) {
    double lx = p->x_shrink_factor * ((c->n_r * c->delta_r) / cos(mx)) + lz * tan(mx);
    lx /= (p->interpolate_factor * c->delta_r);
    c->length_x = floor(lx + 0.5) * p->interpolate_factor * c->delta_r;
  }
  c->length_y = c->n_t * c->delta_t; /* (yEnd - yStart + 1) * delta_t */
  c->n_x = (int)(uint16_t)floor(c->length_x / c->delta_xz);
  c->n_z = (int)(uint16_t)floor(lz / c->delta_xz);
  c->n_y = (int)(uint16_t)floor(c->length_y / c->delta_xy);
  c->x0 = -c->length_x / 2;
  c->z0 = -lz / 2;
  c->y0 = -c->length_y / 2;
}

/* HAADF_ReconstructionEngine::calculateVoxelProfile (HAADF_ReconstructionEngine.cpp:957-1029)
 * for one view with the angle (radians) the profile is built from. */
static void voxel_profile_row(const orc_ctx* c, double angle, double* out) {
  double mvli;
  while (angle > M_PI_2_) angle -= M_PI_2_;
  while (angle < 0) angle += M_PI_2_;
  if (angle <= M_PI_4_)
    mvli = c->delta_xz / cos(angle);
  else
    mvli = c->delta_xz / cos(M_PI_2_ - angle);
  double temp = cos(M_PI_4_);
  double dist1 = temp * cos((M_PI_4_ - angle));
  double dist2 = temp * fabs((cos((M_PI_4_ + angle))));
  double lc = 1 - dist1, ln = 1 - dist2, rn = 1 + dist2, rc = 1 + dist1;
  int PR = c->p.profile_resolution;
  for (int j = 0; j < PR; j++) {
    double t = 2.0 * j / PR;
    double v;
    if (t <= lc || t >= rc)
      v = 0;
    else if (t > rn)
      v = mvli * (rc - t) / (rc - rn);
    else if (t >= ln)
      v = mvli;
    else
      v = mvli * (t - lc) / (ln - lc);
    out[j] = v;
  }
}

static void tables_init(orc_ctx* c) {
  int nt = c->n_theta, bins = c->p.response_bins, PR = c->p.profile_resolution,
      BR = c->p.beam_resolution;
  /* angles: the engine converts to radians in place once before calculateSinCos
   * (HAADF_ReconstructionEngine.cpp:464-471) and, in the HAADF engine, a second time before
   * the profile that feeds DetectorResponse (:499, :978). */
  c->cosv = (double*)calloc(nt, sizeof(double));
  c->sinv = (double*)calloc(nt, sizeof(double));
  c->profile = (double*)calloc((size_t)nt * PR, sizeof(double));
  for (int i = 0; i < nt; i++) {
    double rad = c->angles_deg[i] * (M_PI / 180.0);
    c->cosv[i] = cos(rad); /* DetectorParameters.cpp:60-73 */
    c->sinv[i] = sin(rad);
    double prof_angle = c->p.compat_double_angle ? rad * (M_PI / 180.0) : rad;
    voxel_profile_row(c, prof_angle, c->profile + (size_t)i * PR);
  }
  /* HAADF_ReconstructionEngine.cpp:467-470 */
  c->offset_r = ((c->delta_xz / sqrt(3.0)) + c->delta_r / 2) / bins;
  c->offset_t = ((c->delta_xz / 2) + c->delta_t / 2) / bins;
  double beam_width = c->delta_r;
  /* DetectorParameters::initializeBeamProfile (DetectorParameters.cpp:78-100) */
  c->beam = (double*)calloc(BR, sizeof(double));
  double sum = 0;
  for (int i = 0; i < BR; i++) {
    c->beam[i] = 0.54 - 0.46 * cos((2.0 * M_PI / BR) * i);
    sum = sum + c->beam[i];
  }
  for (int i = 0; i < BR; i++) {
    c->beam[i] /= sum;
    c->beam[i] /= c->delta_t;
  }
  /* DetectorResponse::execute (GenericFilters/DetectorResponse.cpp:66-127) */
  c->H = (double*)calloc((size_t)nt * bins, sizeof(double));
  double r0 = -(beam_width) / 2;
  double step = beam_width / BR;
  double tc = (PR) / (2 * c->delta_xz);
  for (int k = 0; k < nt; k++) {
    for (int i = 0; i < bins; i++) {
      double pcr = i * c->offset_r;
      double rmin = pcr - c->delta_xz;
      double s = 0;
      for (int pp = 0; pp < BR; pp++) {
        double r = r0 + pp * step;
        if (r < rmin) continue;
        int pi = (int)floor((r - rmin) * tc);
        if (pi < 0) pi = 0;
        if (pi >= PR) pi = PR - 1;
        s += c->profile[(size_t)k * PR + pi] * c->beam[pp];
      }
      c->H[(size_t)k * bins + i] = s;
    }
  }
  /* HAADF_ForwardModel::initializeHt (HAADF/HAADF_ForwardModel.cpp:408-451); identical for
   * every view, so one row is kept. */
  c->Ht = (double*)calloc(bins, sizeof(double));
  for (int i = 0; i < bins; i++) {
    double pct = i * c->offset_t, v;
    if (c->delta_xy >= c->delta_t) {
      if (pct <= ((c->delta_xy / 2) - (c->delta_t / 2)))
        v = c->delta_t;
      else
        v = -1 * pct + (c->delta_xy / 2) + c->delta_t / 2;
    } else {
      if (pct <= c->delta_t / 2 - c->delta_xy / 2)
        v = c->delta_xy;
      else
        v = -pct + (c->delta_xy / 2) + c->delta_t / 2;
    }
    if (v < 0) v = 0;
    c->Ht[i] = v;
  }
  /* storeVoxelResponse (HAADF_ReconstructionEngine_Extra.cpp:329-404) */
  c->vlr_cap = (int)(c->delta_xy / c->delta_t) + 2;
  c->vlr_first = (int*)calloc(c->n_y, sizeof(int));
  c->vlr_count = (int*)calloc(c->n_y, sizeof(int));
  c->vlr_val = (double*)calloc((size_t)c->n_y * c->vlr_cap, sizeof(double));
  for (int i = 0; i < c->n_y; i++) {
    double y = ((double)i + 0.5) * c->delta_xy + c->y0;
    double t = y;
    double tmin = (t - c->delta_xy / 2) > c->T0 ? t - c->delta_xy / 2 : c->T0;
    double tmax = (t + c->delta_xy / 2) <= c->TMax ? t + c->delta_xy / 2 : c->TMax;
    int smin = (int16_t)(uint16_t)floor((tmin - c->T0) / c->delta_t);
    int smax = (int16_t)(uint16_t)floor((tmax - c->T0) / c->delta_t);
    if (smin < 0) smin = 0;
    if (smax >= c->n_t) smax = c->n_t - 1;
    c->vlr_first[i] = -1;
    for (int it = smin; it <= smax; it++) {
      double ct = ((double)it + 0.5) * c->delta_t + c->T0;
      double dt = fabs(ct - t);
      int idt = (uint16_t)floor(dt / c->offset_t);
      double pt;
      if (idt < bins) {
        double w3 = dt - (double)(idt)*c->offset_t;
        double w4 = ((double)idt + 1) * c->offset_t - dt;
        int tt = idt + 1 < bins ? idt + 1 : bins - 1;
        pt = (w4 / c->offset_t) * c->Ht[idt] + (w3 / c->offset_t) * c->Ht[tt];
      } else {
        pt = 0;
      }
      if (pt != 0 && c->vlr_count[i] < c->vlr_cap) {
        if (c->vlr_count[i] == 0) c->vlr_first[i] = it;
        c->vlr_val[(size_t)i * c->vlr_cap + c->vlr_count[i]] = pt;
        c->vlr_count[i]++;
      }
    }
    if (c->vlr_first[i] < 0) c->vlr_first[i] = 0;
  }
}

/* AMatrixCol::calculateAMatrixColumnPartial (Common/AMatrixCol.cpp:82-239, duplicated at
 * HAADF_ReconstructionEngine.cpp:1369-1524), AREA_WEIGHTED branch.  The t-direction part of
 * that loop does not change the value (index_delta_t is fixed at 0), so it is omitted. */
int orc_amatrix_column(const orc_ctx* c, int row, int col, int32_t* index, double* value,
                       int cap) {
  int bins = c->p.response_bins, count = 0;
  double x = c->x0 + ((double)col + 0.5) * c->delta_xz;
  double z = c->z0 + ((double)row + 0.5) * c->delta_xz;
  for (int i = 0; i < c->n_theta; i++) {
    double r = x * c->cosv[i] - z * c->sinv[i];
    double rmin = r - c->delta_xz, rmax = r + c->delta_xz;
    if (rmax < c->R0 || rmin > c->RMax) continue;
    int imin = (int)floor(((rmin - c->R0) / c->delta_r));
    int imax = (int)floor((rmax - c->R0) / c->delta_r);
    if (imax >= c->n_r) imax = c->n_r - 1;
    if (imin < 0) imin = 0;
    for (int j = imin; j <= imax; j++) {
      double rc = (c->R0 + (((double)j) + 0.5) * (c->delta_r));
      double dr = fabs(r - rc);
      int idr = (int)floor((dr / c->offset_r));
      if (idr >= 0 && idr < bins) {
        double w1 = dr - idr * c->offset_r;
        double w2 = (idr + 1) * c->offset_r - dr;
        int ii = idr + 1 < bins ? idr + 1 : bins - 1;
        double f1 = (w2 / c->offset_r) * c->H[(size_t)i * bins + idr] +
                    (w1 / c->offset_r) * c->H[(size_t)i * bins + ii];
        if (f1 > 0 && count < cap) {
          index[count] = i * c->n_r + j;
          value[count] = f1;
          count++;
        }
      }
    }
  }
  return count;
}

int orc_voxel_line_response(const orc_ctx* c, int y, int32_t* t_first, double* value, int cap) {
  int n = c->vlr_count[y];
  *t_first = c->vlr_first[y];
  for (int i = 0; i < n && i < cap; i++) value[i] = c->vlr_val[(size_t)y * c->vlr_cap + i];
  return n;
}

static void columns_init(orc_ctx* c) {
  int nl = c->n_z * c->n_x;
  int cap = 3 * c->n_theta * ((int)ceil(3 * c->delta_xz / c->delta_r) + 1);
  int32_t* ti = (int32_t*)malloc(sizeof(int32_t) * cap);
  double* tv = (double*)malloc(sizeof(double) * cap);
  c->col_start = (int*)calloc(nl + 1, sizeof(int));
  c->col_count = (int*)calloc(nl, sizeof(int));
  size_t total = 0, alloc = (size_t)nl * 2 * c->n_theta + 16;
  c->col_index = (int*)malloc(sizeof(int) * alloc);
  c->col_val = (double*)malloc(sizeof(double) * alloc);
  for (int z = 0; z < c->n_z; z++)
    for (int x = 0; x < c->n_x; x++) {
      int l = z * c->n_x + x;
      int n = orc_amatrix_column(c, z, x, ti, tv, cap);
      if (total + n > alloc) {
        alloc = (total + n) * 2;
        c->col_index = (int*)realloc(c->col_index, sizeof(int) * alloc);
        c->col_val = (double*)realloc(c->col_val, sizeof(double) * alloc);
      }
      c->col_start[l] = (int)total;
      c->col_count[l] = n;
      for (int q = 0; q < n; q++) {
        c->col_index[total + q] = ti[q];
        c->col_val[total + q] = tv[q];
      }
      total += n;
    }
  c->col_start[nl] = (int)total;
  free(ti);
  free(tv);
}

#define X3(c, zz, xx, yy) ((c)->x[((size_t)(zz) * (c)->n_x + (xx)) * (c)->n_y + (yy)])
#define S3(c, arr, th_, r_, t_) ((c)->arr[((size_t)(th_) * (c)->n_r + (r_)) * (c)->n_t + (t_)])

orc_ctx* orc_create(const orc_params* p, const double* counts, const double* tilts_deg,
                    int n_theta, int n_r, int n_t, double delta_r, double delta_t) {
  orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
  c->p = *p;
  c->n_theta = n_theta;
  c->n_r = n_r;
  c->n_t = n_t;
  c->delta_r = delta_r;
  c->delta_t = delta_t;
  c->angles_deg = (double*)malloc(sizeof(double) * n_theta);
  memcpy(c->angles_deg, tilts_deg, sizeof(double) * n_theta);
  size_t ns = (size_t)n_theta * n_r * n_t;
  c->counts = (double*)malloc(sizeof(double) * ns);
  memcpy(c->counts, counts, sizeof(double) * ns);
  geometry_init(c);
  tables_init(c);
  columns_init(c);
  size_t nv = (size_t)c->n_z * c->n_x * c->n_y;
  c->x = (double*)calloc(nv, sizeof(double));
  c->e = (double*)calloc(ns, sizeof(double));
  c->w = (double*)calloc(ns, sizeof(double));
  c->yest = (double*)calloc(ns, sizeof(double));
  c->I = (double*)calloc(n_theta, sizeof(double));
  c->mu = (double*)calloc(n_theta, sizeof(double));
  c->alpha = (double*)calloc(n_theta, sizeof(double));
  c->init_gain = (double*)calloc(n_theta, sizeof(double));
  c->init_offset = (double*)calloc(n_theta, sizeof(double));
  c->init_var = (double*)calloc(n_theta, sizeof(double));
  c->mag_map = (double*)calloc((size_t)c->n_z * c->n_x, sizeof(double));
  c->mask = (unsigned char*)calloc((size_t)c->n_z * c->n_x, 1);
  c->filt_map = (double*)calloc((size_t)c->n_z * c->n_x, sizeof(double));
  c->sel = (unsigned char*)malloc(ns);
  memset(c->sel, 1, ns);
  c->bragg_t = p->bragg_threshold;
  /* HAADF_QGGMRFPriorModel.cpp:10-21 (c, P and alpha come from params) */
  c->sig_p = pow(p->sigma_x, p->mrf_p);
  c->sig_pq = pow(p->sigma_x, (p->mrf_p - p->mrf_q));
  c->sig_q = pow(p->sigma_x, p->mrf_q);
  /* initializeROIMask (HAADF_ReconstructionEngine_Extra.cpp:227-248) */
  for (int i = 0; i < c->n_z; i++)
    for (int j = 0; j < c->n_x; j++) {
      double x = c->x0 + ((double)j + 0.5) * c->delta_xz;
      double z = c->z0 + ((double)i + 0.5) * c->delta_xz;
      c->mask[(size_t)i * c->n_x + j] =
          (x >= -(c->n_r * c->delta_r) / 2 && x <= (c->n_r * c->delta_r) / 2 &&
           z >= -c->length_z / 2 && z <= c->length_z / 2)
              ? 1
              : 0;
    }
  return c;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  void* ptrs[] = {c->angles_deg, c->cosv,     c->sinv,       c->profile,     c->beam,
                  c->H,          c->Ht,       c->vlr_first,  c->vlr_count,   c->vlr_val,
                  c->col_start,  c->col_count, c->col_index, c->col_val,     c->counts,
                  c->x,          c->e,        c->w,          c->yest,        c->I,
                  c->mu,         c->alpha,    c->init_gain,  c->init_offset, c->init_var,
                  c->mask,       c->mag_map,  c->filt_map,   c->sel,       c->bfm};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
  free(c);
}

/* initializeBrightFieldData (HAADF_ReconstructionEngine_Extra.cpp:84-176): the bright-field
 * tilt series of the same size, BF_OFFSET (HAADFConstants.h:49) added to every count; from
 * then on the forward model carries BF_Flag.  bf_counts: [n_theta][n_r][n_t]. */
void orc_set_bf_assist(orc_ctx* c, const double* bf_counts) {
  size_t ns = (size_t)c->n_theta * c->n_r * c->n_t;
  free(c->bfm);
  c->bfm = NULL;
  if (!bf_counts) return;
  c->bfm = (double*)malloc(sizeof(double) * ns);
  for (size_t i = 0; i < ns; i++) c->bfm[i] = bf_counts[i] + 32768.0;
}

void orc_dims(const orc_ctx* c, int32_t* dims, double* geo) {
  dims[0] = c->n_z;
  dims[1] = c->n_x;
  dims[2] = c->n_y;
  if (geo) {
    geo[0] = c->delta_xz;
    geo[1] = c->delta_xy;
    geo[2] = c->x0;
    geo[3] = c->y0;
    geo[4] = c->z0;
    geo[5] = c->length_x;
    geo[6] = c->length_y;
    geo[7] = c->length_z;
  }
}
void orc_offsets(const orc_ctx* c, double* o) {
  o[0] = c->offset_r;
  o[1] = c->offset_t;
}
double* orc_volume(orc_ctx* c) { return c->x; }
double* orc_error(orc_ctx* c) { return c->e; }
double* orc_weight(orc_ctx* c) { return c->w; }
double* orc_yest(orc_ctx* c) { return c->yest; }
double* orc_gain(orc_ctx* c) { return c->I; }
double* orc_offset(orc_ctx* c) { return c->mu; }
double* orc_variance(orc_ctx* c) { return c->alpha; }
double* orc_counts(orc_ctx* c) { return c->counts; }
const double* orc_detector_response(const orc_ctx* c) { return c->H; }
const double* orc_ht(const orc_ctx* c) { return c->Ht; }
const double* orc_voxel_profile(const orc_ctx* c) { return c->profile; }
const double* orc_mag_map(const orc_ctx* c) { return c->mag_map; }

/* InitialReconstructionInitializer::initializeData (:74-90), then the zeroing of voxel lines
 * with an empty A column (HAADF_ReconstructionEngine.cpp:614-625). */
void orc_init_volume(orc_ctx* c, const double* vol) {
  size_t nv = (size_t)c->n_z * c->n_x * c->n_y;
  if (vol)
    memcpy(c->x, vol, sizeof(double) * nv);
  else
    for (size_t i = 0; i < nv; i++) c->x[i] = c->p.default_recon_value;
  for (int z = 0; z < c->n_z; z++)
    for (int x = 0; x < c->n_x; x++)
      if (c->col_count[z * c->n_x + x] == 0)
        for (int y = 0; y < c->n_y; y++) X3(c, z, x, y) = 0.0;
}

/* createInitialGainsData / createInitialOffsetsData / createInitialVariancesData
 * (HAADF/HAADF_ForwardModel.cpp:248-402), ComputeInitialOffsets::execute
 * (GenericFilters/ComputeInitialOffsets.cpp:58-186) and gainAndOffsetInitialization
 * (HAADF_ReconstructionEngine_Extra.cpp:280-307). */
int orc_init_nuisance(orc_ctx* c) {
  int nt = c->n_theta;
  for (int i = 0; i < nt; i++) c->init_gain[i] = c->p.target_gain;
  if (c->p.use_default_offset) {
    for (int i = 0; i < nt; i++) c->init_offset[i] = c->p.default_offset;
  } else {
    double* avg = (double*)calloc((size_t)(nt > 0 ? nt : 1), sizeof(double));
    double* tg = (double*)calloc((size_t)(nt > 0 ? nt : 1), sizeof(double));
    for (int th = 0; th < nt; th++) {
      double sum = 0;
      for (int r = 0; r < c->n_r; r++)
        for (int t = 0; t < c->n_t; t++) sum += S3(c, counts, th, r, t);
      sum /= (c->n_r * c->n_t);
      avg[th] = sum;
      tg[th] = 1.0 / cos(c->angles_deg[th] * M_PI / 180);
    }
    double pm[2][2];
    for (int i = 0; i < 2; i++)
      for (int j = 0; j < 2; j++) {
        pm[i][j] = 0;
        for (int k = 0; k < nt; k++) {
          double a = (i == 0) ? tg[k] : 1.0, b = (j == 0) ? tg[k] : 1.0;
          pm[i][j] += a * b;
        }
      }
    double det = pm[0][0] * pm[1][1] - (pm[0][1] * pm[0][1]);
    double inv[2][2];
    inv[0][0] = pm[1][1] / det;
    inv[1][1] = pm[0][0] / det;
    inv[0][1] = -pm[1][0] / det;
    inv[1][0] = -pm[0][1] / det;
    double tv[2] = {0, 0};
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < nt; k++) tv[j] += ((j == 0) ? tg[k] : 1.0) * avg[k];
    double est[2] = {0, 0};
    for (int i = 0; i < 2; i++)
      for (int k = 0; k < 2; k++) est[i] += inv[i][k] * tv[k];
    for (int i = 0; i < nt; i++) c->init_offset[i] = est[1];
    free(avg);
    free(tg);
  }
  for (int i = 0; i < nt; i++) c->init_var[i] = c->p.default_variance;
  double sum = 0;
  for (int k = 0; k < nt; k++) {
    c->I[k] = c->init_gain[k];
    c->mu[k] = c->init_offset[k];
    sum += c->I[k];
  }
  sum /= nt;
  if (sum - c->p.target_gain > 1e-5) {
    double t = c->p.target_gain / sum;
    for (int k = 0; k < nt; k++) c->I[k] = c->init_gain[k] * t;
  }
  /* BF: BFReconstructionEngine::execute creates the nuisance parameters from the raw counts
   * (:374) and only then takes the log (processRawCounts :385,
   * BFForwardModel.cpp:939-972): counts += bf_offset; y = -log(counts / BF_MAX), BF_MAX = 1.
   * A negative count ends that (theta, r) row early, as the reference's break does. */
  if (c->p.modality == 1 && !c->counts_logged) {
    for (int th = 0; th < nt; th++)
      for (int r = 0; r < c->n_r; r++)
        for (int t = 0; t < c->n_t; t++) {
          double* v = &S3(c, counts, th, r, t);
          *v += c->p.bf_offset;
          if (*v < 0) break;
          *v = -log(*v / 1.0);
        }
    c->counts_logged = 1;
  }
  return 0;
}

/* HAADF_ForwardProject::operator() (HAADF/HAADF_ForwardProject.cpp:80-120), run serially
 * over z in order so that the FP64 sum is deterministic. */
void orc_forward_project(orc_ctx* c) {
  size_t ns = (size_t)c->n_theta * c->n_r * c->n_t;
  memset(c->yest, 0, sizeof(double) * ns);
  for (int j = 0; j < c->n_z; j++)
    for (int k = 0; k < c->n_x; k++) {
      int l = j * c->n_x + k;
      if (c->col_count[l] <= 0) continue;
      for (int i = 0; i < c->n_y; i++)
        for (int q = 0; q < c->col_count[l]; q++) {
          int id = c->col_index[c->col_start[l] + q];
          int th = id / c->n_r, r = id % c->n_r;
          int t0 = c->vlr_first[i];
          for (int a = 0; a < c->vlr_count[i]; a++) {
            double tt = (c->I[th] * (c->col_val[c->col_start[l] + q] *
                                     c->vlr_val[(size_t)i * c->vlr_cap + a] * X3(c, j, k, i)));
            S3(c, yest, th, r, t0 + a) += tt;
          }
        }
    }
}

/* calculateMeasurementWeight (HAADF_ReconstructionEngine_Extra.cpp:693-771) with
 * IDENTITY_NOISE_MODEL (HAADFConstants.h:56) and no bright-field data. */
void orc_measurement_weight(orc_ctx* c) {
  if (c->p.modality == 1) {
    /* BFForwardModel::calculateMeasurementWeight (BFForwardModel.cpp:328-385): no
     * IDENTITY_NOISE_MODEL in the BF build, so w = BF_MAX / exp(y), divided by alpha */
    for (int th = 0; th < c->n_theta; th++) {
      if (c->p.noise_estimation) c->alpha[th] = c->init_var[th];
      for (int r = 0; r < c->n_r; r++)
        for (int t = 0; t < c->n_t; t++) {
          S3(c, e, th, r, t) = S3(c, counts, th, r, t) - S3(c, yest, th, r, t) - c->mu[th];
          double w = 1.0 / exp(S3(c, counts, th, r, t));
          S3(c, sel, th, r, t) = 1;
          if (c->p.noise_estimation) w /= c->alpha[th];
          S3(c, w, th, r, t) = w;
        }
    }
    return;
  }
  for (int th = 0; th < c->n_theta; th++) {
    if (c->p.noise_model) c->alpha[th] = c->init_var[th];
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        if (c->bfm) /* :722-727 */
          S3(c, e, th, r, t) =
              S3(c, counts, th, r, t) - S3(c, bfm, th, r, t) * S3(c, yest, th, r, t) - c->mu[th];
        else
          S3(c, e, th, r, t) = S3(c, counts, th, r, t) - S3(c, yest, th, r, t) - c->mu[th];
        double w = 1.0;
        if (c->p.noise_model) w /= c->alpha[th];
        S3(c, w, th, r, t) = w;
      }
  }
}

/* One voxel of UpdateYSlice::execute (HAADF_ReconstructionEngine_UpdateVoxels.cpp:265-460). */
static void update_voxel(orc_ctx* c, int jn, int kn, int i, int outer, int inner, double* stats,
                         double* mag) {
  double nb[27];
  unsigned char bf[27];
  memset(nb, 0, sizeof(nb));
  memset(bf, 0, sizeof(bf));
  for (int p = -1; p <= 1; p++)
    for (int q = -1; q <= 1; q++)
      for (int r = -1; r <= 1; r++)
        if (i + p >= 0 && i + p < c->n_y && jn + q >= 0 && jn + q < c->n_z && kn + r >= 0 &&
            kn + r < c->n_x) {
          nb[IDX3(p + 1, q + 1, r + 1)] = X3(c, q + jn, r + kn, p + i);
          bf[IDX3(p + 1, q + 1, r + 1)] = 1;
        }
  nb[IDX3(1, 1, 1)] = 0.0;
  double V = X3(c, jn, kn, i);
  /* zero skipping :310-338 */
  int zs = 0;
  if (c->p.zero_skipping == 1 && V == 0.0 && (inner > 0 || outer > 0)) {
    zs = 1;
    for (int a = 0; a < 27; a++)
      if (nb[a] > 0.0) zs = 0;
  }
  if (zs) {
    stats[2] += 1;
    return;
  }
  int l = jn * c->n_x + kn;
  int base = c->col_start[l], cnt = c->col_count[l];
  int t0 = c->vlr_first[i], tc = c->vlr_count[i];
  const double* hv = c->vlr_val + (size_t)i * c->vlr_cap;
  double th1 = 0.0, th2 = 0.0;
  for (int q = 0; q < cnt; q++) {
    int id = c->col_index[base + q];
    int th = id / c->n_r, r = id % c->n_r;
    double k0 = c->I[th] * (c->col_val[base + q]);
    for (int a = 0; a < tc; a++) {
      size_t ei = ((size_t)th * c->n_r + r) * c->n_t + (t0 + a);
      double pe = k0 * hv[a];
      if (c->bfm) pe *= c->bfm[ei]; /* :358-364 */
      th2 += (pe * pe * c->w[ei]);
      th1 += (c->e[ei] * pe * c->w[ei]);
    }
  }
  th1 *= -1;
  /* find_min_max (:47-63) over all 27 entries (centre and out-of-range entries are 0) */
  double low = nb[0], high = nb[0];
  for (int a = 0; a < 27; a++) {
    if (nb[a] < low) low = nb[a];
    if (nb[a] > high) high = nb[a];
  }
  if (th2 != 0) {
    low = (low > (V - (th1 / th2)) ? (V - (th1 / th2)) : low);
    high = (high < (V - (th1 / th2)) ? (V - (th1 / th2)) : high);
  }
  double nv = q_substitution(c, low, high, V, bf, nb, th1, th2);
  if (nv < 0.0) nv = 0.0; /* POSITIVITY_CONSTRAINT :394-400 */
  X3(c, jn, kn, i) = nv;
  mag[l] += fabs(nv - V);
  if (c->mask[l] == 1) {
    stats[0] += fabs(nv - V);
    stats[1] += fabs(V);
  }
  stats[3] += 1;
  for (int q = 0; q < cnt; q++) {
    int id = c->col_index[base + q];
    int th = id / c->n_r, r = id % c->n_r;
    for (int a = 0; a < tc; a++) {
      size_t ei = ((size_t)th * c->n_r + r) * c->n_t + (t0 + a);
      double k2 = (c->I[th] * (c->col_val[base + q] * hv[a] * (nv - V)));
      if (c->bfm)
        c->e[ei] -= (c->bfm[ei] * k2); /* :442-446 */
      else
        c->e[ei] -= k2;
    }
  }
}

/* ---------------------------------------------------------------------------------------
 * MT19937 (Matsumoto & Nishimura 1998), the generator behind boost::mt19937; restated here
 * from the published algorithm.
 * ------------------------------------------------------------------------------------- */
typedef struct {
  uint32_t mt[624];
  int idx;
} mt_state;

static void mt_seed(mt_state* s, uint32_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 624; i++)
    s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->idx = 624;
}

static uint32_t mt_next(mt_state* s) {
  if (s->idx >= 624) {
    for (int i = 0; i < 624; i++) {
      uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
      s->mt[i] = s->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    s->idx = 0;
  }
  uint32_t y = s->mt[s->idx++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

/* Visit order of UpdateYSlice::execute (HAADF_ReconstructionEngine_UpdateVoxels.cpp:151-241):
 * uniform_int over the full uint32 range returns the raw generator output; each draw picks
 * Counter[draw % remaining] and moves the last entry into its place. */
void orc_visit_order(uint32_t seed, int n_z, int n_x, int32_t* out) {
  int size = n_z * n_x;
  int32_t* counter = (int32_t*)malloc(sizeof(int32_t) * size);
  for (int j = 0; j < size; j++) counter[j] = j;
  mt_state s;
  mt_seed(&s, seed);
  int n = 0;
  for (int j = 0; j < n_z; j++)
    for (int k = 0; k < n_x; k++) {
      uint32_t index = mt_next(&s) % (uint32_t)size;
      int kn = counter[index] % n_x;
      int jn = counter[index] / n_x;
      counter[index] = counter[size - 1];
      size--;
      out[n++] = jn * n_x + kn;
    }
  free(counter);
}

void orc_icd_sweep_lines(orc_ctx* c, const int32_t* lines, int n_lines, int outer, int inner,
                         double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (size_t i = 0; i < (size_t)c->n_z * c->n_x; i++) c->mag_map[i] = 0;
  for (int n = 0; n < n_lines; n++) {
    int l = lines[n];
    if (c->col_count[l] <= 0) continue;
    int jn = l / c->n_x, kn = l % c->n_x;
    for (int i = 0; i < c->n_y; i++) update_voxel(c, jn, kn, i, outer, inner, stats, c->mag_map);
  }
}

void orc_icd_sweep_reference(orc_ctx* c, uint32_t seed, int outer, int inner, double* stats) {
  int nl = c->n_z * c->n_x;
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * nl);
  orc_visit_order(seed, c->n_z, c->n_x, order);
  orc_icd_sweep_lines(c, order, nl, outer, inner, stats);
  free(order);
}

/* updateVoxels with OpenMBIR_USE_PARALLEL_ALGORITHMS (_UpdateVoxels.cpp:666-723): the y range is
 * split round-robin by count into one contiguous range per worker; every worker walks the same
 * random line order over its own y range.  Neighbour reads across range boundaries race exactly
 * as in the reference; the per-line update magnitudes are kept per worker and summed. */
typedef struct {
  orc_ctx* c;
  const int32_t* order;
  int n_lines, y0, y1, outer, inner;
  int bf;
  double st[4];
  double* mag;
} orc_task;

static void bf_update_voxel(orc_ctx* c, int jn, int kn, int i, int outer, int inner,
                            double* stats, double* mag);

static void* orc_task_run(void* arg) {
  orc_task* t = (orc_task*)arg;
  orc_ctx* c = t->c;
  for (int n = 0; n < t->n_lines; n++) {
    int l = t->order[n];
    if (c->col_count[l] <= 0) continue;
    int jn = l / c->n_x, kn = l % c->n_x;
    for (int i = t->y0; i < t->y1; i++) {
      if (t->bf)
        bf_update_voxel(c, jn, kn, i, t->outer, t->inner, t->st, t->mag);
      else
        update_voxel(c, jn, kn, i, t->outer, t->inner, t->st, t->mag);
    }
  }
  return NULL;
}

void orc_icd_sweep_reference_mt(orc_ctx* c, uint32_t seed, int outer, int inner, int n_threads,
                                double* stats) {
  int nl = c->n_z * c->n_x;
  if (n_threads < 1) n_threads = 1;
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * nl);
  orc_visit_order(seed, c->n_z, c->n_x, order);
  int* ycount = (int*)calloc(n_threads, sizeof(int));
  for (int y = 0, t = 0; y < c->n_y; ++y) {
    ycount[t]++;
    if (++t == n_threads) t = 0;
  }
  orc_task* tasks = (orc_task*)calloc(n_threads, sizeof(orc_task));
  pthread_t* th = (pthread_t*)calloc(n_threads, sizeof(pthread_t));
  int ystart = 0, used = 0;
  for (int t = 0; t < n_threads; t++) {
    if (ycount[t] == 0) continue;
    orc_task* k = &tasks[used];
    k->c = c;
    k->order = order;
    k->n_lines = nl;
    k->y0 = ystart;
    k->y1 = ystart + ycount[t];
    k->outer = outer;
    k->inner = inner;
    k->mag = (double*)calloc(nl, sizeof(double));
    ystart = k->y1;
    used++;
  }
  for (int t = 0; t < used; t++) pthread_create(&th[t], NULL, orc_task_run, &tasks[t]);
  for (int t = 0; t < used; t++) pthread_join(th[t], NULL);
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (int l = 0; l < nl; l++) c->mag_map[l] = 0;
  for (int t = 0; t < used; t++) {
    for (int s = 0; s < 4; s++) stats[s] += tasks[t].st[s];
    for (int l = 0; l < nl; l++) c->mag_map[l] += tasks[t].mag[l];
    free(tasks[t].mag);
  }
  free(tasks);
  free(th);
  free(ycount);
  free(order);
}

void orc_icd_sweep_slices(orc_ctx* c, const int32_t* row_order, int stride, int outer, int inner,
                          double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (size_t i = 0; i < (size_t)c->n_z * c->n_x; i++) c->mag_map[i] = 0;
  for (int colour = 0; colour < 2; colour++)
    for (int i = colour; i < c->n_y; i += 2)
      for (int rr = 0; rr < c->n_z; rr++) {
        int z = row_order[rr];
        for (int k = 0; k < stride; k++)
          for (int x = k; x < c->n_x; x += stride)
            if (c->col_count[z * c->n_x + x] > 0)
              update_voxel(c, z, x, i, outer, inner, stats, c->mag_map);
      }
}

/* jointEstimation, gain+offset branch (HAADF_ReconstructionEngine_Extra.cpp:419-636). */
int orc_joint_estimation(orc_ctx* c) {
  if (c->bfm) {
    /* with bright-field data only the offsets are estimated (:429, :643-668): per view the
     * weighted mean of the error, taken off the error and added to the offset */
    for (int th = 0; th < c->n_theta; th++) {
      double num_sum = 0, den_sum = 0;
      for (int r = 0; r < c->n_r; r++)
        for (int t = 0; t < c->n_t; t++) {
          num_sum += (S3(c, e, th, r, t) * S3(c, w, th, r, t));
          den_sum += S3(c, w, th, r, t);
        }
      double a = num_sum / den_sum;
      for (int r = 0; r < c->n_r; r++)
        for (int t = 0; t < c->n_t; t++) S3(c, e, th, r, t) -= a;
      c->mu[th] += a;
    }
    return 0;
  }
  int nt = c->n_theta;
  double* Qk = (double*)calloc((size_t)nt * 3, sizeof(double));
  double* bk = (double*)calloc((size_t)nt * 2, sizeof(double));
  double* d1 = (double*)calloc(nt, sizeof(double));
  double* d2 = (double*)calloc(nt, sizeof(double));
  for (int th = 0; th < nt; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        double v = S3(c, counts, th, r, t) - S3(c, e, th, r, t) - c->mu[th];
        S3(c, yest, th, r, t) = v / c->I[th];
      }
  for (int th = 0; th < nt; th++) {
    double a = 0, b = 0, cc = 0, d = 0, num = 0, den = 0;
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        double y = S3(c, counts, th, r, t), w = S3(c, w, th, r, t), ye = S3(c, yest, th, r, t);
        num += (y * w);
        den += (w);
        a += (ye * w);
        b += (ye * w * y);
        cc += (y * y * w);
        d += (ye * ye * w);
      }
    bk[th * 2 + 1] = num;
    bk[th * 2 + 0] = b;
    Qk[th * 3 + 2] = den;
    Qk[th * 3 + 1] = a;
    Qk[th * 3 + 0] = d;
    d1[th] = num / den;
    d2[th] = a / den;
    (void)cc;
  }
  double sum1 = 0, sum2 = 0;
  for (int th = 0; th < nt; th++) {
    sum1 += (1.0 / (Qk[th * 3 + 0] - Qk[th * 3 + 1] * d2[th]));
    sum2 += ((bk[th * 2 + 0] - Qk[th * 3 + 1] * d1[th]) / (Qk[th * 3 + 0] - Qk[th * 3 + 1] * d2[th]));
  }
  double lm = (-nt * c->p.target_gain + sum2) / sum1;
  for (int th = 0; th < nt; th++) {
    double ni = (-1 * lm - Qk[th * 3 + 1] * d1[th] + bk[th * 2 + 0]) /
                (Qk[th * 3 + 0] - Qk[th * 3 + 1] * d2[th]);
    c->I[th] = ni;
    c->mu[th] = d1[th] - d2[th] * c->I[th];
  }
  for (int th = 0; th < nt; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++)
        S3(c, e, th, r, t) =
            S3(c, counts, th, r, t) - c->mu[th] - (c->I[th] * S3(c, yest, th, r, t));
  free(Qk);
  free(bk);
  free(d1);
  free(d2);
  return 0;
}

/* updateWeights (HAADF_ReconstructionEngine_Extra.cpp:795-881), IDENTITY_NOISE_MODEL. */
void orc_update_weights(orc_ctx* c) {
  for (int th = 0; th < c->n_theta; th++) {
    double sum = 0;
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) S3(c, w, th, r, t) = 1.0;
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        double e = S3(c, e, th, r, t);
        sum += (e * e * S3(c, w, th, r, t));
      }
    sum /= (c->n_r * c->n_t);
    c->alpha[th] = sum;
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) S3(c, w, th, r, t) = 1.0 / c->alpha[th];
  }
}

/* computeCost, QGGMRF branch (HAADF_ReconstructionEngine.cpp:1147-1364). */
static double prior_cost(const orc_ctx* c);

double orc_cost(const orc_ctx* c, double* parts) {
  double cost = 0, temp = 0;
  for (int i = 0; i < c->n_theta; i++)
    for (int j = 0; j < c->n_r; j++)
      for (int k = 0; k < c->n_t; k++) {
        double ev = S3(c, e, i, j, k);
        cost += (ev * ev * S3(c, w, i, j, k));
      }
  cost /= 2;
  double data = cost;
  temp = prior_cost(c);
  cost += temp;
  double noise = 0;
  if (c->p.noise_model) {
    double tn = 0;
    for (int i = 0; i < c->n_theta; i++)
      for (int j = 0; j < c->n_r; j++)
        for (int k = 0; k < c->n_t; k++) {
          double w = S3(c, w, i, j, k);
          if (w != 0) tn += log(2 * M_PI * (1.0 / w));
        }
    tn /= 2;
    noise = tn;
    cost += tn;
  }
  if (parts) {
    parts[0] = data;
    parts[1] = temp;
    parts[2] = noise;
  }
  return cost;
}

/* QGGMRF prior term of computeCost (HAADF_ReconstructionEngine.cpp:1285-1359; the same
 * 13-neighbour loop is QGGMRF::PriorModelCost, BF_QGGMRFPriorModel.cpp:162-262). */
static double prior_cost(const orc_ctx* c) {
  double temp = 0;
#define XV(zz, xx, yy) X3(c, zz, xx, yy)
#define ACC(fi, z2, x2, y2) temp += k_filter[fi] * q_value(c, XV(i, j, k) - XV(z2, x2, y2))
  for (int i = 0; i < c->n_z; i++)
    for (int j = 0; j < c->n_x; j++)
      for (int k = 0; k < c->n_y; k++) {
        if (k + 1 < c->n_y) ACC(IDX3(2, 1, 1), i, j, k + 1);
        if (j + 1 < c->n_x) {
          if (k - 1 >= 0) ACC(IDX3(0, 1, 2), i, j + 1, k - 1);
          ACC(IDX3(1, 1, 2), i, j + 1, k);
          if (k + 1 < c->n_y) ACC(IDX3(2, 1, 2), i, j + 1, k + 1);
        }
        if (i + 1 < c->n_z) {
          if (j - 1 >= 0) ACC(IDX3(1, 2, 0), i + 1, j - 1, k);
          ACC(IDX3(1, 2, 1), i + 1, j, k);
          if (j + 1 < c->n_x) ACC(IDX3(1, 2, 2), i + 1, j + 1, k);
          if (j - 1 >= 0) {
            if (k - 1 >= 0) ACC(IDX3(0, 2, 0), i + 1, j - 1, k - 1);
            if (k + 1 < c->n_y) ACC(IDX3(2, 2, 0), i + 1, j - 1, k + 1);
          }
          if (k - 1 >= 0) ACC(IDX3(0, 2, 1), i + 1, j, k - 1);
          if (j + 1 < c->n_x) {
            if (k - 1 >= 0) ACC(IDX3(0, 2, 2), i + 1, j + 1, k - 1);
            if (k + 1 < c->n_y) ACC(IDX3(2, 2, 2), i + 1, j + 1, k + 1);
          }
          if (k + 1 < c->n_y) ACC(IDX3(2, 2, 1), i + 1, j, k + 1);
        }
      }
#undef ACC
#undef XV
  return temp;
}

/* HAADF_ReconstructionEngine::execute outer/inner loops (HAADF_ReconstructionEngine.cpp:706-815)
 * with RegularRandomOrderUpdate and the ROI stop rule of updateVoxels (_UpdateVoxels.cpp:765-787). */
int orc_run(orc_ctx* c, uint32_t seed, double* cost_log, int n_cost) {
  return orc_run_seeded(c, seed, 0u, cost_log, n_cost);
}

/* The same with sweep k drawing its order from seed + k * seed_step: the reference reseeds from
 * its millisecond clock at every sweep, so consecutive sweeps visit the lines in new orders
 * (seed_step = 0: one order for every sweep, the clock frozen). */
int orc_run_seeded(orc_ctx* c, uint32_t seed, uint32_t seed_step, double* cost_log, int n_cost) {
  int sweeps = 0;
  double stop = c->p.stop_threshold;
  int num_iter = c->p.inner_iterations;
  for (int outer = 0; outer < c->p.outer_iterations; outer++) {
    if (outer != 0) num_iter = 1;
    int status = 1;
    for (int inner = 0; inner < num_iter; inner++) {
      double st[4];
      orc_icd_sweep_reference(c, seed + (uint32_t)sweeps * seed_step, outer, inner, st);
      if (cost_log && sweeps < n_cost) cost_log[sweeps] = orc_cost(c, NULL);
      sweeps++;
      status = 1;
      if (st[1] > 0 && (st[0] / st[1]) < stop) {
        stop *= c->p.threshold_reduction_factor;
        status = 0;
        break;
      }
    }
    if (c->p.joint_estimation) orc_joint_estimation(c);
    if (c->p.noise_model) {
      orc_update_weights(c);
      if (status == 0 && outer >= 1) break;
    } else if (status == 0 && outer >= 1) {
      break;
    }
  }
  return sweeps;
}

/* =========================================================================================
 * Bright field (Code/MBIRLib/BrightField/...)
 * ========================================================================================= */
unsigned char* orc_selector(orc_ctx* c) { return c->sel; }
double* orc_filt_map(orc_ctx* c) { return c->filt_map; }
void orc_set_bragg(orc_ctx* c, double t) { c->bragg_t = t; }
double orc_get_bragg(const orc_ctx* c) { return c->bragg_t; }

/* boost::uniform_int<uint32_t>(0, range) drawn from mt19937 (boost's integer bucket method:
 * the raw 32-bit draw divided by bucket_size, redrawn when the quotient exceeds range). */
static uint32_t boost_uniform(mt_state* s, uint32_t range) {
  const uint32_t brange = 0xffffffffu;
  if (range == 0) return 0;
  if (range == brange) return mt_next(s);
  uint32_t bucket = brange / (range + 1u);
  if (brange % (range + 1u) == range) ++bucket;
  for (;;) {
    uint32_t r = mt_next(s) / bucket;
    if (r <= range) return r;
  }
}

/* VoxelUpdateList::GenRandList (Common/VoxelUpdateList.cpp:157-215): newIndexes starts as
 * the identity; for i = 1..n-1 it is swapped with a uniform position in [0, n-1]; element i
 * of the input goes to position newIndexes[i].  The reference seeds with the clock; here the
 * seed is explicit. */
void orc_rand_list_perm(uint32_t seed, int n, int32_t* idx) {
  for (int i = 0; i < n; i++) idx[i] = i;
  if (n < 2) return;
  mt_state s;
  mt_seed(&s, seed);
  for (int i = 1; i < n; i++) {
    uint32_t r = boost_uniform(&s, (uint32_t)(n - 1));
    if (r >= (uint32_t)n) continue;
    int32_t t = idx[i];
    idx[i] = idx[r];
    idx[r] = t;
  }
}

/* One voxel of BFUpdateYSlice::execute (BrightField/BFUpdateYSlice.cpp:185-322) with
 * BFForwardModel::computeTheta (BFForwardModel.cpp:851-892) and updateErrorSinogram
 * (:898-932): entries rejected by the Bragg selector enter theta1/theta2 with the weight
 * delta*T / (|e| sqrt(w)); the scatter re-evaluates the selector as |e sqrt(w)| < T. */
static void bf_update_voxel(orc_ctx* c, int jn, int kn, int i, int outer, int inner,
                            double* stats, double* mag) {
  double nb[27];
  unsigned char bf[27];
  memset(nb, 0, sizeof(nb));
  memset(bf, 0, sizeof(bf));
  for (int p = -1; p <= 1; p++)
    for (int q = -1; q <= 1; q++)
      for (int r = -1; r <= 1; r++)
        if (i + p >= 0 && i + p < c->n_y && jn + q >= 0 && jn + q < c->n_z && kn + r >= 0 &&
            kn + r < c->n_x) {
          nb[IDX3(p + 1, q + 1, r + 1)] = X3(c, q + jn, r + kn, p + i);
          bf[IDX3(p + 1, q + 1, r + 1)] = 1;
        }
  nb[IDX3(1, 1, 1)] = 0.0;
  double V = X3(c, jn, kn, i);
  int zs = 0;
  if (c->p.zero_skipping == 1 && V == 0.0 && (inner > 0 || outer > 0)) {
    zs = 1;
    for (int a = 0; a < 27; a++)
      if (nb[a] > 0.0) zs = 0;
  }
  if (zs) {
    stats[2] += 1;
    return;
  }
  const double T = c->bragg_t, dlt = c->p.bragg_delta;
  int l = jn * c->n_x + kn;
  int base = c->col_start[l], cnt = c->col_count[l];
  int t0 = c->vlr_first[i], tc = c->vlr_count[i];
  const double* hv = c->vlr_val + (size_t)i * c->vlr_cap;
  double th1 = 0.0, th2 = 0.0;
  for (int q = 0; q < cnt; q++) {
    int id = c->col_index[base + q];
    int th = id / c->n_r, r = id % c->n_r;
    double k0 = c->I[th] * (c->col_val[base + q]);
    for (int a = 0; a < tc; a++) {
      size_t ei = ((size_t)th * c->n_r + r) * c->n_t + (t0 + a);
      double ev = c->e[ei], w = c->w[ei];
      if (c->sel[ei] == 1) {
        double pe = k0 * hv[a];
        th2 += (pe * pe * w);
        th1 += (ev * pe * w);
      } else {
        double qc = (dlt * T) / (fabs(ev) * sqrt(w));
        double pe = k0 * hv[a];
        th2 += qc * (pe * pe * w);
        th1 += qc * (ev * pe * w);
      }
    }
  }
  th1 *= -1;
  double low = nb[0], high = nb[0];
  for (int a = 0; a < 27; a++) {
    if (nb[a] < low) low = nb[a];
    if (nb[a] > high) high = nb[a];
  }
  if (th2 != 0) {
    low = (low > (V - (th1 / th2)) ? (V - (th1 / th2)) : low);
    high = (high < (V - (th1 / th2)) ? (V - (th1 / th2)) : high);
  }
  double nv = q_substitution(c, low, high, V, bf, nb, th1, th2);
  if (nv < 0.0) nv = 0.0; /* POSITIVITY_CONSTRAINT (BFConstants.h) */
  X3(c, jn, kn, i) = nv;
  mag[l] = mag[l] + fabs(nv - V);
  if (c->mask[l] == 1) {
    stats[0] += fabs(nv - V);
    stats[1] += fabs(V);
  }
  stats[3] += 1;
  double d = nv - V;
  for (int q = 0; q < cnt; q++) {
    int id = c->col_index[base + q];
    int th = id / c->n_r, r = id % c->n_r;
    for (int a = 0; a < tc; a++) {
      size_t ei = ((size_t)th * c->n_r + r) * c->n_t + (t0 + a);
      double k2 = (c->I[th] * (c->col_val[base + q] * hv[a] * (d)));
      c->e[ei] -= k2;
      c->sel[ei] = (fabs(c->e[ei] * sqrt(c->w[ei])) < T) ? 1 : 0;
    }
  }
}

/* One updateVoxels call (BFReconstructionEngine_Extra.cpp:476-859) with one worker: the
 * lines' magnitudes restart at 0, then every line sweeps y = 0..n_y-1 in list order. */
void orc_bf_sweep_lines(orc_ctx* c, const int32_t* lines, int n_lines, int outer, int inner,
                        double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (int n = 0; n < n_lines; n++) c->mag_map[lines[n]] = 0;
  for (int n = 0; n < n_lines; n++) {
    int l = lines[n];
    c->mag_map[l] = 0;
    if (c->col_count[l] <= 0) continue;
    for (int y = 0; y < c->n_y; y++)
      bf_update_voxel(c, l / c->n_x, l % c->n_x, y, outer, inner, stats, c->mag_map);
  }
}

void orc_bf_sweep_slices(orc_ctx* c, const unsigned char* active, const int32_t* row_order,
                         int stride, int outer, int inner, double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  size_t nl = (size_t)c->n_z * c->n_x;
  for (size_t l = 0; l < nl; l++)
    if (active[l]) c->mag_map[l] = 0;
  for (int colour = 0; colour < 2; colour++)
    for (int i = colour; i < c->n_y; i += 2)
      for (int rr = 0; rr < c->n_z; rr++) {
        int z = row_order[rr];
        for (int k = 0; k < stride; k++)
          for (int x = k; x < c->n_x; x += stride) {
            int l = z * c->n_x + x;
            if (active[l] && c->col_count[l] > 0)
              bf_update_voxel(c, z, x, i, outer, inner, stats, c->mag_map);
          }
      }
}

/* The same call with every voxel slice visiting the call's lines in the given order (the
 * GPU's scheduled calls: colour classes one after another); slices in colour order as above. */
void orc_bf_sweep_slices_order(orc_ctx* c, const int32_t* lines, int n_lines, int outer,
                               int inner, double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (int n = 0; n < n_lines; n++) c->mag_map[lines[n]] = 0;
  for (int colour = 0; colour < 2; colour++)
    for (int i = colour; i < c->n_y; i += 2)
      for (int n = 0; n < n_lines; n++) {
        int l = lines[n];
        if (c->col_count[l] > 0)
          bf_update_voxel(c, l / c->n_x, l % c->n_x, i, outer, inner, stats, c->mag_map);
      }
}

/* ComputeVSC (BFReconstructionEngine_Extra.cpp:888-947): 5x5 Hamming window
 * (BFReconstructionEngine.cpp:157-185) over the update-magnitude map, zero outside. */
static const double k_hamming[5][5] = {{0.0013, 0.0086, 0.0159, 0.0086, 0.0013},
                                       {0.0086, 0.0581, 0.1076, 0.0581, 0.0086},
                                       {0.0159, 0.1076, 0.1993, 0.1076, 0.0159},
                                       {0.0086, 0.0581, 0.1076, 0.0581, 0.0086},
                                       {0.0013, 0.0086, 0.0159, 0.0086, 0.0013}};
void orc_bf_vsc(orc_ctx* c) {
  for (int i = 0; i < c->n_z; i++)
    for (int j = 0; j < c->n_x; j++) {
      double f = 0;
      for (int p = -2; p <= 2; p++)
        for (int q = -2; q <= 2; q++)
          if (i + p >= 0 && i + p < c->n_z && j + q >= 0 && j + q < c->n_x)
            f += k_hamming[p + 2][q + 2] * c->mag_map[(size_t)(i + p) * c->n_x + (j + q)];
      c->filt_map[(size_t)i * c->n_x + j] = f;
    }
}

static int cmp_double(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* SetNonHomThreshold (BFReconstructionEngine_Extra.cpp:954-1011): the order statistic at
 * position N - N/20 (ascending, 0-based) of the filtered map.  RandomizedSelect's random
 * pivots do not change the value it returns; this takes it from a sorted copy.  (For N < 20
 * the reference's position is out of range; here it is clamped to N-1.) */
double orc_bf_nh_threshold(const orc_ctx* c) {
  size_t n = (size_t)c->n_z * c->n_x;
  double* a = (double*)malloc(sizeof(double) * n);
  memcpy(a, c->filt_map, sizeof(double) * n);
  qsort(a, n, sizeof(double), cmp_double);
  size_t k = n - n / 20;
  if (k >= n) k = n - 1;
  double t = a[k];
  free(a);
  return t;
}

/* GenNonHomList (BFReconstructionEngine_Extra.cpp:1016-1047) before its randomisation: lines
 * whose filtered magnitude exceeds the threshold, z-major. */
int orc_bf_nh_lines(const orc_ctx* c, double threshold, int32_t* lines) {
  int n = 0;
  for (int j = 0; j < c->n_z; j++)
    for (int k = 0; k < c->n_x; k++)
      if (c->filt_map[(size_t)j * c->n_x + k] > threshold) lines[n++] = j * c->n_x + k;
  return n;
}

/* roiVolumeSum (BFReconstructionEngine_Extra.cpp:1200-1215) */
double orc_roi_volume_sum(const orc_ctx* c) {
  double sum = 0;
  for (int j = 0; j < c->n_z; j++)
    for (int k = 0; k < c->n_x; k++)
      if (c->mask[(size_t)j * c->n_x + k] == 1)
        for (int i = 0; i < c->n_y; i++) sum += X3(c, j, k, i);
  return sum;
}

/* the ROI sum of stopCriteria (BFReconstructionEngine_Extra.cpp:1239-1248) */
double orc_roi_mag_sum(const orc_ctx* c) {
  double sum = 0;
  for (int j = 0; j < c->n_z; j++)
    for (int k = 0; k < c->n_x; k++)
      if (c->mask[(size_t)j * c->n_x + k] == 1) sum += c->mag_map[(size_t)j * c->n_x + k];
  return sum;
}

/* BFForwardModel::jointEstimation (BFForwardModel.cpp:390-441): per view, the offset
 * (log dosage) step alpha = num/den over selected entries (e w, w) and rejected ones
 * (T delta sign(e) sqrt(w), T delta sqrt(w) / |e|); e -= alpha, mu += alpha. */
void orc_bf_joint_estimation(orc_ctx* c) {
  const double T = c->bragg_t, dl = c->p.bragg_delta;
  for (int th = 0; th < c->n_theta; th++) {
    double num = 0, den = 0;
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        double ev = S3(c, e, th, r, t), w = S3(c, w, th, r, t);
        if (S3(c, sel, th, r, t) == 1) {
          num += (ev * w);
          den += w;
        } else {
          num += (T * dl * ev / fabs(ev)) * sqrt(w);
          den += ((T * dl * sqrt(w)) / fabs(ev));
        }
      }
    double a = num / den;
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) S3(c, e, th, r, t) -= a;
    c->mu[th] += a;
  }
}

/* BFForwardModel::updateWeights (BFForwardModel.cpp:447-511): one variance for all views. */
void orc_bf_update_weights(orc_ctx* c) {
  const double T = c->bragg_t, dl = c->p.bragg_delta;
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) S3(c, w, th, r, t) *= c->alpha[th];
  double sum1 = 0, sum2 = 0;
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        double ev = S3(c, e, th, r, t), w = S3(c, w, th, r, t);
        if (S3(c, sel, th, r, t) == 1)
          sum1 += (ev * ev * w);
        else
          sum2 += fabs(ev) * sqrt(c->alpha[th] * w);
      }
  double upd = (sum1 + (dl * T) * sum2) / (c->n_theta * c->n_r * c->n_t);
  for (int th = 0; th < c->n_theta; th++) c->alpha[th] = upd;
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) S3(c, w, th, r, t) /= c->alpha[th];
}

/* BFForwardModel::updateSelector (BFForwardModel.cpp:517-531) */
void orc_bf_update_selector(orc_ctx* c) {
  const double T = c->bragg_t;
  size_t ns = (size_t)c->n_theta * c->n_r * c->n_t;
  for (size_t i = 0; i < ns; i++) c->sel[i] = (c->e[i] * c->e[i] * c->w[i] < T * T) ? 1 : 0;
}

/* ---- bright-field slabs: the y-range task split of updateVoxels
 * (BFReconstructionEngine_Extra.cpp:624-752) with the tasks' magnitude maps and the estimates'
 * sums added over slabs by the caller.  Rows [t0, t1) are the slab's detector rows. */

/* the call's lines restart their magnitudes (BFUpdateYSlice.cpp:171) */
void orc_bf_reset_mag(orc_ctx* c, const unsigned char* active) {
  size_t nl = (size_t)c->n_z * c->n_x;
  for (size_t l = 0; l < nl; l++)
    if (active[l]) c->mag_map[l] = 0;
}

/* one colour of orc_bf_sweep_slices over slices [y0, y1) (magnitudes accumulate) */
void orc_bf_sweep_colour(orc_ctx* c, const unsigned char* active, const int32_t* row_order,
                         int stride, int colour, int y0, int y1, int outer, int inner,
                         double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (int i = y0; i < y1; i++) {
    if ((i & 1) != colour) continue;
    for (int rr = 0; rr < c->n_z; rr++) {
      int z = row_order[rr];
      for (int k = 0; k < stride; k++)
        for (int x = k; x < c->n_x; x += stride) {
          int l = z * c->n_x + x;
          if (active[l] && c->col_count[l] > 0)
            bf_update_voxel(c, z, x, i, outer, inner, stats, c->mag_map);
        }
    }
  }
}

/* orc_bf_joint_estimation's per-view numerator and denominator over rows [t0, t1), [theta][2] */
void orc_bf_offset_sums(const orc_ctx* c, int t0, int t1, double* out) {
  const double T = c->bragg_t, dl = c->p.bragg_delta;
  for (int th = 0; th < c->n_theta; th++) {
    double num = 0, den = 0;
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) {
        double ev = S3(c, e, th, r, t), w = S3(c, w, th, r, t);
        if (S3(c, sel, th, r, t) == 1) {
          num += (ev * w);
          den += w;
        } else {
          num += (T * dl * ev / fabs(ev)) * sqrt(w);
          den += ((T * dl * sqrt(w)) / fabs(ev));
        }
      }
    out[th * 2] = num;
    out[th * 2 + 1] = den;
  }
}

static void bf_selector_rows(orc_ctx* c, int t0, int t1) {
  const double T = c->bragg_t;
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) {
        double ev = S3(c, e, th, r, t);
        S3(c, sel, th, r, t) = (ev * ev * S3(c, w, th, r, t) < T * T) ? 1 : 0;
      }
}

/* the offset steps from sums added over slabs: e -= num/den on rows [t0, t1), mu += num/den,
 * then the selector of those rows */
void orc_bf_apply_offsets(orc_ctx* c, const double* sums, int t0, int t1) {
  for (int th = 0; th < c->n_theta; th++) {
    double a = sums[th * 2] / sums[th * 2 + 1];
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) S3(c, e, th, r, t) -= a;
    c->mu[th] += a;
  }
  bf_selector_rows(c, t0, t1);
}

/* orc_bf_update_weights' two sums over rows [t0, t1), after w *= alpha on those rows, and the
 * number of entries they cover */
void orc_bf_variance_sums(orc_ctx* c, int t0, int t1, double* out3) {
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) S3(c, w, th, r, t) *= c->alpha[th];
  double sum1 = 0, sum2 = 0;
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) {
        double ev = S3(c, e, th, r, t), w = S3(c, w, th, r, t);
        if (S3(c, sel, th, r, t) == 1)
          sum1 += (ev * ev * w);
        else
          sum2 += fabs(ev) * sqrt(c->alpha[th] * w);
      }
  out3[0] = sum1;
  out3[1] = sum2;
  out3[2] = (double)c->n_theta * c->n_r * (t1 - t0);
}

/* the common variance from sums added over slabs (the two sums over the entries they cover);
 * w /= it on rows [t0, t1), then their selector */
void orc_bf_apply_variance(orc_ctx* c, const double* sums, int t0, int t1) {
  const double T = c->bragg_t, dl = c->p.bragg_delta;
  double upd = (sums[0] + (dl * T) * sums[1]) / sums[2];
  for (int th = 0; th < c->n_theta; th++) c->alpha[th] = upd;
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) S3(c, w, th, r, t) /= c->alpha[th];
  bf_selector_rows(c, t0, t1);
}

/* orc_roi_volume_sum over slices [y0, y1) */
double orc_roi_volume_sum_range(const orc_ctx* c, int y0, int y1) {
  double sum = 0;
  for (int j = 0; j < c->n_z; j++)
    for (int k = 0; k < c->n_x; k++)
      if (c->mask[(size_t)j * c->n_x + k] == 1)
        for (int i = y0; i < y1; i++) sum += X3(c, j, k, i);
  return sum;
}

/* BFReconstructionEngine::computeCost (BFReconstructionEngine.cpp:1084-1097) =
 * BFForwardModel::forwardCost (BFForwardModel.cpp:812-846) + QGGMRF::PriorModelCost.
 * parts: [0] data, [1] prior, [2] noise. */
double orc_bf_cost(const orc_ctx* c, double* parts) {
  const double T = c->bragg_t, dl = c->p.bragg_delta;
  double cost = 0;
  for (int i = 0; i < c->n_theta; i++)
    for (int j = 0; j < c->n_r; j++)
      for (int k = 0; k < c->n_t; k++) {
        double ev = S3(c, e, i, j, k), w = S3(c, w, i, j, k);
        if (S3(c, sel, i, j, k) == 1)
          cost += (ev * ev * w);
        else
          cost += (2 * T * dl * fabs(ev) * sqrt(w) + T * T * (1 - 2 * dl));
      }
  cost /= 2;
  double data = cost, noise = 0;
  if (c->p.noise_estimation) {
    /* (N_theta N_r N_t / 2) in integer arithmetic, as the reference writes it */
    noise = (double)((c->n_theta * c->n_r * c->n_t) / 2) * log(c->alpha[0]);
    cost += noise;
  }
  double prior = prior_cost(c);
  if (parts) {
    parts[0] = data;
    parts[1] = prior;
    parts[2] = noise;
  }
  return cost + prior;
}

#define K_NHOM 20      /* MBIR::Constants::k_NumHomogeniousIter (ReconstructionConstants.h:76) */
#define K_NNHOM 20     /* k_NumNonHomogeniousIter (:77) */
#define K_DEF_BRAGG 5e10 /* DefBraggThreshold (BFConstants.h) */

/* BFReconstructionEngine::execute outer/inner loops (BFReconstructionEngine.cpp:555-858) with
 * NHICD (even calls: the next 1/20 of a random permutation of all lines; odd calls: lines
 * whose filtered update magnitude is in the top 1/20), the Bragg threshold schedule, the
 * stop rule of stopCriteria and the nuisance updates.  Each call visits its list in the order
 * of orc_rand_list_perm(seed + 1 + call) (the reference: GenRandList per worker, clock seed). */
static int bf_run_impl(orc_ctx* c, uint32_t seed, uint32_t list_seed_step, int max_calls);

int orc_bf_run(orc_ctx* c, uint32_t seed, int max_calls) { return bf_run_impl(c, seed, 1u, max_calls); }

/* The reference seeds every list generator from the millisecond clock
 * (VoxelUpdateList.cpp:171-172); with the clock frozen at one value every list draw starts from
 * the same seed, which this entry point reproduces. */
int orc_bf_run_fixed_seed(orc_ctx* c, uint32_t seed, int max_calls) {
  return bf_run_impl(c, seed, 0u, max_calls);
}

static int bf_run_impl(orc_ctx* c, uint32_t seed, uint32_t list_seed_step, int max_calls) {
  const int nl = c->n_z * c->n_x;
  int32_t* perm = (int32_t*)malloc(sizeof(int32_t) * (nl > 0 ? nl : 1));
  int32_t* master = (int32_t*)malloc(sizeof(int32_t) * (nl > 0 ? nl : 1));
  int32_t* list = (int32_t*)malloc(sizeof(int32_t) * (nl > 0 ? nl : 1));
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (nl > 0 ? nl : 1));
  orc_rand_list_perm(seed, nl, perm);
  for (int i = 0; i < nl; i++) master[perm[i]] = i;
  int num_iter = c->p.inner_iterations;
  double des_t = 0, temp_t;
  if (num_iter > 1) {
    des_t = c->p.bragg_threshold;
    temp_t = K_DEF_BRAGG;
  } else {
    temp_t = c->p.bragg_threshold;
  }
  c->bragg_t = temp_t;
  for (int i = 0; i < nl; i++) c->mag_map[i] = 0;
  uint32_t listsel = 0, eff = 0;
  double prev_mag = 0, stop = c->p.stop_threshold;
  int calls = 0, done = 0;
  for (int outer = 0; outer < c->p.outer_iterations && !done; outer++) {
    if (outer > 0) {
      num_iter = 1;
      c->bragg_t = temp_t;
    }
    int status = 1;
    for (int inner = 0; inner < num_iter; inner++) {
      if (num_iter > 1 && inner == 0) c->bragg_t = K_DEF_BRAGG;
      int n = 0;
      if (!c->p.nhicd) {
        memcpy(list, master, sizeof(int32_t) * nl);
        n = nl;
      } else if (eff % 2 == 0) {
        listsel %= K_NHOM;
        int n_el = (int)floor((double)nl / K_NHOM);
        if (listsel == K_NHOM - 1) n_el += nl - n_el * K_NHOM;
        int start = (int)(floor((double)nl / K_NHOM) * listsel);
        memcpy(list, master + start, sizeof(int32_t) * n_el);
        n = n_el;
        listsel++;
      } else {
        orc_bf_vsc(c);
        n = orc_bf_nh_lines(c, orc_bf_nh_threshold(c), list);
      }
      /* The worker's GenRandList of the call's list (BFReconstructionEngine_Extra.cpp:691).  A
       * non-homogeneous list was already randomised once by GenNonHomList (:1044); both draws
       * happen within the same millisecond of the reference's clock and so use one seed. */
      const uint32_t call_seed = list_seed_step ? seed + 1u + (uint32_t)calls : seed;
      orc_rand_list_perm(call_seed, n, perm);
      const int nh_call = c->p.nhicd && (eff % 2 == 1);
      if (nh_call) {
        for (int i = 0; i < n; i++) order[perm[i]] = list[i];
        memcpy(list, order, sizeof(int32_t) * n);
      }
      for (int i = 0; i < n; i++) order[perm[i]] = list[i];
      double st[4];
      orc_bf_sweep_lines(c, order, n, outer, inner, st);
      status = 1;
      int check = c->p.nhicd ? (eff % K_NNHOM == 0) : 1;
      if (check && eff > 0 && prev_mag > 0) {
        double ratio = fabs(orc_roi_mag_sum(c)) / fabs(prev_mag);
        if (ratio < stop) {
          stop *= c->p.threshold_reduction_factor;
          status = 0;
        }
      }
      if (!c->p.nhicd || eff % K_NNHOM == 0) prev_mag = orc_roi_volume_sum(c);
      eff++;
      calls++;
      if (max_calls > 0 && calls >= max_calls) {
        done = 1;
        break;
      }
      if (status == 0) break;
      if (inner == num_iter - 1 && inner != 0) {
        temp_t = des_t;
        c->bragg_t = temp_t;
      }
    }
    if (done) break;
    if (status == 0 && outer >= 1) break;
    if (c->p.outer_iterations > 1) {
      if (c->p.joint_estimation) {
        orc_bf_joint_estimation(c);
        orc_bf_update_selector(c);
      }
      if (c->p.noise_estimation) {
        orc_bf_update_weights(c);
        orc_bf_update_selector(c);
      }
    }
  }
  free(perm);
  free(master);
  free(list);
  free(order);
  return calls;
}

/* updateVoxels of the BF engine with OpenMBIR_USE_PARALLEL_ALGORITHMS
 * (BFReconstructionEngine_Extra.cpp:654-753): contiguous y ranges, one per worker, every worker
 * walking the call's lines over its range (the reference gives each worker its own random order
 * of the list; here they share the given order).  Per-worker magnitudes are summed into the
 * lines of the call.  Used to time the reference's CPU path. */
void orc_bf_sweep_lines_mt(orc_ctx* c, const int32_t* lines, int n_lines, int outer, int inner,
                           int n_threads, double* stats) {
  int nl = c->n_z * c->n_x;
  if (n_threads < 1) n_threads = 1;
  int* ycount = (int*)calloc(n_threads, sizeof(int));
  for (int y = 0, t = 0; y < c->n_y; ++y) {
    ycount[t]++;
    if (++t == n_threads) t = 0;
  }
  orc_task* tasks = (orc_task*)calloc(n_threads, sizeof(orc_task));
  pthread_t* th = (pthread_t*)calloc(n_threads, sizeof(pthread_t));
  int ystart = 0, used = 0;
  for (int t = 0; t < n_threads; t++) {
    if (ycount[t] == 0) continue;
    orc_task* k = &tasks[used];
    k->c = c;
    k->order = lines;
    k->n_lines = n_lines;
    k->y0 = ystart;
    k->y1 = ystart + ycount[t];
    k->outer = outer;
    k->inner = inner;
    k->bf = 1;
    k->mag = (double*)calloc(nl, sizeof(double));
    ystart = k->y1;
    used++;
  }
  for (int t = 0; t < used; t++) pthread_create(&th[t], NULL, orc_task_run, &tasks[t]);
  for (int t = 0; t < used; t++) pthread_join(th[t], NULL);
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (int n = 0; n < n_lines; n++) c->mag_map[lines[n]] = 0;
  for (int t = 0; t < used; t++) {
    for (int s = 0; s < 4; s++) stats[s] += tasks[t].st[s];
    for (int n = 0; n < n_lines; n++) c->mag_map[lines[n]] += tasks[t].mag[lines[n]];
    free(tasks[t].mag);
  }
  free(tasks);
  free(th);
  free(ycount);
}

/* =========================================================================================
 * y-slab sharding support (test infrastructure for the multi-rank driver): one colour phase of
 * the slice-order sweep restricted to slices y in [y0, y1), per-view sums over a detector-row
 * range, and the nuisance update with the error rebuild of jointEstimation.
 * ========================================================================================= */
void orc_icd_sweep_colour(orc_ctx* c, const int32_t* row_order, int stride, int colour, int y0,
                          int y1, int outer, int inner, double* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  for (int i = y0; i < y1; i++) {
    if ((i & 1) != colour) continue;
    for (int rr = 0; rr < c->n_z; rr++) {
      int z = row_order[rr];
      for (int k = 0; k < stride; k++)
        for (int x = k; x < c->n_x; x += stride)
          if (c->col_count[z * c->n_x + x] > 0)
            update_voxel(c, z, x, i, outer, inner, stats, c->mag_map);
    }
  }
}

/* kind 0: the six sums of jointEstimation per view ([theta][6]: y w, w, yh w, yh w y, y^2 w,
 * yh^2 w with yh = (y - e - mu)/I); kind 1: sum e^2 per view.  Rows t in [t0, t1). */
void orc_view_sums(const orc_ctx* c, int kind, int t0, int t1, double* out) {
  for (int th = 0; th < c->n_theta; th++) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int r = 0; r < c->n_r; r++)
      for (int t = t0; t < t1; t++) {
        double ev = S3(c, e, th, r, t);
        if (kind == 1) {
          s[0] += ev * ev;
        } else {
          double y = S3(c, counts, th, r, t), w = S3(c, w, th, r, t);
          double yh = (y - ev - c->mu[th]) / c->I[th];
          s[0] += (y * w);
          s[1] += (w);
          s[2] += (yh * w);
          s[3] += (yh * w * y);
          s[4] += (y * y * w);
          s[5] += (yh * yh * w);
        }
      }
    if (kind == 1)
      out[th] = s[0];
    else
      for (int k = 0; k < 6; k++) out[th * 6 + k] = s[k];
  }
}

/* new gain/offset (and variance) per view; e = y - mu' - I' yh, yh = (y - e - mu)/I
 * (HAADF_ReconstructionEngine_Extra.cpp:600-612); weights 1/alpha (identity noise model) */
void orc_apply_nuisance(orc_ctx* c, const double* gain, const double* offset,
                        const double* variance) {
  for (int th = 0; th < c->n_theta; th++)
    for (int r = 0; r < c->n_r; r++)
      for (int t = 0; t < c->n_t; t++) {
        double yv = S3(c, counts, th, r, t);
        double yh = (yv - S3(c, e, th, r, t) - c->mu[th]) / c->I[th];
        S3(c, e, th, r, t) = yv - offset[th] - (gain[th] * yh);
        if (variance) S3(c, w, th, r, t) = 1.0 / variance[th];
      }
  for (int th = 0; th < c->n_theta; th++) {
    c->I[th] = gain[th];
    c->mu[th] = offset[th];
    if (variance) c->alpha[th] = variance[th];
  }
}
