// mbir_sweep_f32_sched.cu -- FP32 bright-field NHICD calls run from a colour schedule, with the
// loads of the next classes issued while the current class is updated.
//
// A scheduled call (BFUpdateYSlice::execute over the call's lines, BrightField/
// BFUpdateYSlice.cpp:147-335, in the colour-class order of the call's schedule) walks its
// classes one after another in every voxel slice, with a CTA barrier between classes.  Each
// class step of the plain scheduled sweep (run_slice in mbir_sweep.cuh) is one dependent chain:
// the voxel's A-column from its table, then the bright-field weights at that footprint, the 26
// neighbours from the volume, the prior coefficients, the theta sums, the update and the
// scatter.  Three of those loads do not depend on the classes before: the A-column (a table),
// the weights (fixed during a call) and the neighbours in the slices y-1 and y+1 (the other
// colour, fixed during the launch), and the voxel's own value (each line appears once per call).
// Here every voxel group keeps the data of its next two classes in flight:
//   class k+2: A-column table entries;
//   class k+1: weights at its footprint (its A-column arrived during class k), neighbours and
//              its own value;
//   class k:   the update itself, from registers and the staged error / selector rows.
// The neighbours in the voxel's own slice may change in class k-1 (lines of consecutive
// classes may be 3x3 neighbours); every class publishes its updated lines (a bit per line and
// the (line, value) pairs of the class) and the next class patches the neighbours it holds.
// Lines of one class are independent, so the results equal the plain scheduled sweep bit for
// bit (same arithmetic, same order per voxel).
//
// Requirements (checked by the host): FP32, bright field, ICD, one detector row per slice,
// slices staged in shared memory, every class at most as large as the CTA's voxel groups (the
// device colour schedule caps them so), 16-lane voxel groups with up to 4 views per lane.
#include "mbir_sweep.cuh"

namespace mbir {
namespace sweep {

constexpr int kSchedG = 16;   // lanes per voxel group
constexpr int kSchedVPL = 4;  // views per lane (n_theta <= 64)
constexpr int kSchedGroups = kWarps * 32 / kSchedG;

struct SchedLayout {
  size_t bar, ctl, stats, gw, upd, bits, es, sel, total;
  int bit_words;
};

__host__ __device__ inline SchedLayout sched_layout(int n_theta, int n_lines, int n_rs,
                                                    int n_sp) {
  SchedLayout L;
  size_t o = 0;
  L.bar = o;
  o += 16;
  L.ctl = o;
  o += 16;
  L.stats = o;
  o += sizeof(unsigned long long) * kSchedGroups * kStatSlots;
  L.gw = o;
  o = align_up(o + sizeof(float2) * n_theta, 16);
  L.upd = o;  // [2][groups] (line, value) of the last two classes
  o = align_up(o + 2 * sizeof(int2) * kSchedGroups, 16);
  L.bits = o;  // [2][bit_words] lines updated in the last two classes
  L.bit_words = (n_lines + 31) / 32;
  o = align_up(o + 2 * sizeof(unsigned) * static_cast<size_t>(L.bit_words), 128);
  L.es = o;
  o += sizeof(float) * static_cast<size_t>(n_theta) * n_rs;
  o = align_up(o, 16);
  L.sel = o;
  o += static_cast<size_t>(n_theta) * n_sp;
  L.total = align_up(o, 16);
  return L;
}

// The loads of one voxel group for one class: its line, A-column table entries, the weights at
// the footprint, the neighbour entries this lane holds (k = gl, gl + 16) and its own value.
template <int NB>
struct SchedItem {
  static constexpr int AW = acol_width(NB);
  int line;  // z * n_x + x, or -1 (no voxel for this group in the class)
  float4 aq[kSchedVPL][AW];
  float w[kSchedVPL][NB];
  float nb[2];
  float V;
};

template <int NB>
__device__ __forceinline__ int sched_line(const SweepArgs& A, int n_levels, int lv, int group) {
  if (lv >= n_levels) return -1;
  const int b = __ldg(A.sched_lofs + lv), e = __ldg(A.sched_lofs + lv + 1);
  return group < e - b ? __ldg(A.sched_lines + b + group) : -1;
}

template <int NB>
__device__ __forceinline__ void sched_load_acol(const SweepArgs& A, int gl, SchedItem<NB>& it) {
  constexpr int AW = acol_width(NB);
  const DevGeom& g = A.g;
  const float4* ac = A.acol + static_cast<size_t>(it.line < 0 ? 0 : it.line) * g.n_theta * AW;
#pragma unroll
  for (int i = 0; i < kSchedVPL; ++i) {
    const int v = gl + kSchedG * i;
#pragma unroll
    for (int w = 0; w < AW; ++w)
      it.aq[i][w] = (it.line >= 0 && v < g.n_theta) ? __ldg(ac + v * AW + w)
                                                    : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Weights at the footprint (the same safe-index rule as group_step), the neighbours and V.
template <int NB>
__device__ __forceinline__ void sched_load_rest(const SweepArgs& A, int gl, int y,
                                                const float* bw, SchedItem<NB>& it) {
  const DevGeom& g = A.g;
  const bool act = it.line >= 0;
  const int z = act ? it.line / g.n_x : 0, x = act ? it.line - z * g.n_x : 0;
#pragma unroll
  for (int i = 0; i < kSchedVPL; ++i) {
    const int v = gl + kSchedG * i;
    const bool vok = v < g.n_theta && act;
    const int jlo = __float_as_int(it.aq[i][0].x);
    const int widx = vok ? v * g.n_rp + jlo : 0;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const float a = f4_at(it.aq[i][(b + 1) >> 2], (b + 1) & 3);
      const bool ok = vok && a > 0.f;
      it.w[i][b] = __ldg(bw + (ok ? widx + b : 0));
    }
  }
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  const float* vol = static_cast<const float*>(A.x);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int k = gl + kSchedG * i;
    it.nb[i] = 0.f;
    if (act && k < 27 && k != 13) {
      const int dy = k / 9 - 1, dz = (k / 3) % 3 - 1, dx = k % 3 - 1;
      const int yy = y + dy, zz = z + dz, xx = x + dx;
      if (yy >= 0 && yy < g.n_y && zz >= 0 && zz < g.n_z && xx >= 0 && xx < g.n_x) {
        const float* src = vol + static_cast<size_t>(yy) * plane + static_cast<size_t>(zz) * g.n_x + xx;
        // the slices y-1, y+1 do not change during the launch; this slice's plane does
        it.nb[i] = dy != 0 ? __ldg(src) : *src;
      }
    }
  }
  it.V = act ? vol[static_cast<size_t>(y) * plane + static_cast<size_t>(it.line)] : 0.f;
}

template <int NB>
__global__ void __launch_bounds__(kWarps * 32, 1) sched_sweep_kernel(SweepArgs A) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int G = kSchedG, VPL = kSchedVPL;
  const int y = (A.y_end > 0 ? A.y_first : A.colour) + 2 * static_cast<int>(blockIdx.x);
  if (y >= (A.y_end > 0 ? A.y_end : A.g.n_y)) return;
  init_slice_barrier(smem);
  const DevGeom& g = A.g;
  const int tid = threadIdx.x, nthreads = blockDim.x;
  const int lane = tid & 31, gl = lane & (G - 1);
  const int group = (tid >> 5) * (32 / G) + (lane / G);
  const int n_sp = A.bfa.n_sp;
  const int n_lines = g.n_z * g.n_x;
  const SchedLayout L = sched_layout(g.n_theta, n_lines, A.n_rs, n_sp);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L.bar);
  unsigned long long* sstat = reinterpret_cast<unsigned long long*>(smem + L.stats);
  float2* sgw = reinterpret_cast<float2*>(smem + L.gw);
  int2* upd = reinterpret_cast<int2*>(smem + L.upd);
  unsigned* bits = reinterpret_cast<unsigned*>(smem + L.bits);
  float* es = reinterpret_cast<float*>(smem + L.es);
  uint8_t* ssel = smem + L.sel;
  const int rs = A.n_rs, srs = n_sp;
  const int tfirst = A.tab.t_first[y];

  __shared__ PriorConst<float> s_pc;
  __shared__ float s_qf[27];
  __shared__ float s_hh;
  if (tid == 0) s_pc = prior_const<float>(A.flt, A.g);
  if (tid < 27) s_qf[tid] = static_cast<float>(A.flt.f[tid]);
  if (tid == 0) s_hh = static_cast<const float*>(A.tab.hval)[y * kMaxTRows];
  const float2* ggw = static_cast<const float2*>(A.tab.gw);
  for (int v = tid; v < g.n_theta; v += nthreads) sgw[v] = ggw[v];
  for (int i = tid; i < 2 * L.bit_words; i += nthreads) bits[i] = 0u;
  __syncthreads();

  // stage the slice's error and selector rows (one detector row)
  float* const ge = static_cast<float*>(A.e);
  const size_t sino_plane = static_cast<size_t>(g.n_theta) * g.n_rp;
  const size_t sel_plane = static_cast<size_t>(g.n_theta) * n_sp;
  const uint32_t row_bytes = static_cast<uint32_t>(g.n_rp * sizeof(float));
  uint32_t phase = 0;
  {
    const uint32_t total = static_cast<uint32_t>(g.n_theta) * (row_bytes + n_sp);
    if (tid == 0) mbar_expect_tx(bar, total);
    __syncthreads();
    for (int v = tid; v < g.n_theta; v += nthreads) {
      bulk_g2s(es + v * rs, ge + static_cast<size_t>(tfirst) * sino_plane +
                                static_cast<size_t>(v) * g.n_rp, row_bytes, bar);
      bulk_g2s(ssel + v * srs, A.bfa.sel + static_cast<size_t>(tfirst) * sel_plane +
                                   static_cast<size_t>(v) * n_sp,
               static_cast<uint32_t>(n_sp), bar);
    }
    const bool ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (!__syncthreads_and(ok)) {
      if (tid == 0) atomicOr(A.err, 1);
      mbar_wait(bar, phase ^ 1u);  // give copies still in flight a second bounded chance
      return;
    }
  }

  const float* bw = static_cast<const float*>(A.bfa.w) + static_cast<size_t>(tfirst) * sino_plane;
  float* vol = static_cast<float*>(A.x);
  const size_t plane = static_cast<size_t>(g.n_z) * g.n_x;
  const PriorConst<float>& pc = s_pc;
  const float bt = static_cast<float>(A.bfa.bragg_t), bdt = static_cast<float>(A.bfa.bragg_dt);
  unsigned long long* mag_fx = A.bfa.mag_fx;
  const bool zs_on = A.zero_skipping && A.iter_nonzero;
  const int n_levels = A.sched_count != nullptr ? __ldg(A.sched_count + 1) : A.n_levels;

  GroupAcc acc;
#pragma unroll
  for (int s2 = 0; s2 < kStatSlots; ++s2) acc.v[s2] = 0ull;

  // the pipeline: cur (class lv), nx1 (lv + 1), nx2 (lv + 2, A-column only)
  SchedItem<NB> cur, nx1, nx2;
  cur.line = sched_line<NB>(A, n_levels, 0, group);
  nx1.line = sched_line<NB>(A, n_levels, 1, group);
  sched_load_acol<NB>(A, gl, cur);
  sched_load_acol<NB>(A, gl, nx1);
  sched_load_rest<NB>(A, gl, y, bw, cur);
  int old_line = -1;  // the line this group published two classes ago (its bit to clear)
  int prev_line = -1;
  for (int lv = 0; lv < n_levels; ++lv) {
    // issue the next classes' loads: class lv + 2's A-column, class lv + 1's weights,
    // neighbours and value (its A-column was requested one class ago)
    nx2.line = sched_line<NB>(A, n_levels, lv + 2, group);
    sched_load_acol<NB>(A, gl, nx2);
    sched_load_rest<NB>(A, gl, y, bw, nx1);
    const int buf = lv & 1;
    // this group's bit from class lv - 2 leaves the buffer class lv publishes into
    if (gl == 0 && old_line >= 0) atomicAnd(bits + buf * L.bit_words + (old_line >> 5),
                                            ~(1u << (old_line & 31)));
    old_line = prev_line;
    prev_line = -1;

    const bool act = cur.line >= 0;
    const int z = act ? cur.line / g.n_x : 0, x = act ? cur.line - z * g.n_x : 0;
    // neighbours in this slice updated by class lv - 1 (loaded before that class ran)
    float nbv[2];
    bool nvalid[2];
    bool pos = false;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int k = gl + G * i;
      nbv[i] = cur.nb[i];
      nvalid[i] = false;
      if (act && k < 27 && k != 13) {
        const int dy = k / 9 - 1, dz = (k / 3) % 3 - 1, dx = k % 3 - 1;
        const int yy = y + dy, zz = z + dz, xx = x + dx;
        if (yy >= 0 && yy < g.n_y && zz >= 0 && zz < g.n_z && xx >= 0 && xx < g.n_x) {
          nvalid[i] = true;
          if (dy == 0 && lv > 0) {
            const int ln = zz * g.n_x + xx;
            const unsigned* pb = bits + (buf ^ 1) * L.bit_words;
            if ((pb[ln >> 5] >> (ln & 31)) & 1u) {
              const int2* pu = upd + (buf ^ 1) * kSchedGroups;
              for (int j = 0; j < kSchedGroups; ++j)
                if (pu[j].x == ln) {
                  nbv[i] = __int_as_float(pu[j].y);
                  break;
                }
            }
          }
          pos |= nbv[i] > 0.f;
        }
      }
    }
    const float V = cur.V;
    bool live = act;
    if (zs_on) {
      const bool any_pos = group_any<G>(pos, lane);
      if (V == 0.f && !any_pos) {
        if (live && gl == 0) acc.v[2] += 1;
        live = false;
      }
    }
    if (__any_sync(kFull, live)) {
      // prior surrogate sums, theta sums, update, scatter: group_step's arithmetic in its order
      float s1 = 0.f, s2 = 0.f;
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        if (nvalid[i]) {
          const float tc = s_qf[gl + G * i] * qggmrf_coef<float>(pc, V - nbv[i]);
          s1 += tc * nbv[i];
          s2 += tc;
        }
      }
      int jlo[VPL];
      float a[VPL][NB];
#pragma unroll
      for (int i = 0; i < VPL; ++i) {
        const int v = gl + G * i;
        jlo[i] = 0;
#pragma unroll
        for (int b = 0; b < NB; ++b) a[i][b] = 0.f;
        if (v < g.n_theta && live) {
          jlo[i] = __float_as_int(cur.aq[i][0].x);
#pragma unroll
          for (int b = 0; b < NB; ++b) a[i][b] = f4_at(cur.aq[i][(b + 1) >> 2], (b + 1) & 3);
        }
      }
      const float hh = s_hh;
      // the footprint's error values are read from the staged rows where they are used (theta
      // sums, scatter): no other voxel of the class touches them in between
      unsigned svm = 0u;  // selector bits of the footprint entries (bit i * NB + b)
      int eidx[VPL];
#pragma unroll
      for (int i = 0; i < VPL; ++i) {
        const int v = gl + G * i;
        const bool vok = v < g.n_theta && live;
        eidx[i] = vok ? v * rs + jlo[i] : 0;
        const int sidx = vok ? v * srs + jlo[i] : 0;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          const bool ok = vok && a[i][b] > 0.f;
          svm |= (ssel[ok ? sidx + b : 0] != 0 ? 1u : 0u) << (i * NB + b);
        }
      }
      float t1 = 0.f, t2 = 0.f;
#pragma unroll
      for (int i = 0; i < VPL; ++i) {
        const int v = gl + G * i;
        if (v >= g.n_theta || !live) continue;
        const float2 gw = sgw[v];
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          if (a[i][b] > 0.f) {
            const float pe = gw.x * a[i][b] * hh;
            const float w = cur.w[i][b];
            const float evb = es[eidx[i] + b];
            if ((svm >> (i * NB + b)) & 1u) {
              t2 += pe * pe * w;
              t1 += evb * pe * w;
            } else {
              const float qc = bdt / (fabsf(evb) * sqrtf(w));
              t2 += qc * (pe * pe * w);
              t1 += qc * (evb * pe * w);
            }
          }
        }
      }
      const float theta1 = -group_sum<G>(t1);
      const float theta2 = group_sum<G>(t2);
      float lo = 0.f, hi = 0.f;
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        lo = nbv[i] < lo ? nbv[i] : lo;
        hi = nbv[i] > hi ? nbv[i] : hi;
      }
      lo = group_min<G>(lo);
      hi = group_max<G>(hi);
      if (theta2 != 0.f) {
        const float cand = V - theta1 / theta2;
        lo = lo > cand ? cand : lo;
        hi = hi < cand ? cand : hi;
      }
      s1 = group_sum<G>(s1);
      s2 = group_sum<G>(s2);
      const float u = (s1 + theta2 * V - theta1) / (s2 + theta2);
      float nv = V + pc.alpha * (u - V);
      nv = (nv < lo) ? lo : ((nv > hi) ? hi : nv);
      if (nv < 0.f) nv = 0.f;
      const float dlt = nv - V;
      if (live) {
#pragma unroll
        for (int i = 0; i < VPL; ++i) {
          const int v = gl + G * i;
          if (v >= g.n_theta) continue;
          const float gain = sgw[v].x;
#pragma unroll
          for (int b = 0; b < NB; ++b)
            if (a[i][b] > 0.f) {
              const float ne = es[eidx[i] + b] - gain * (a[i][b] * hh * dlt);
              es[eidx[i] + b] = ne;
              ssel[v * srs + jlo[i] + b] = bragg_selected<float>(ne, cur.w[i][b], bt);
            }
        }
        if (gl == 0) {
          vol[static_cast<size_t>(y) * plane + static_cast<size_t>(cur.line)] = nv;
          if (x >= g.roi_x0 && x <= g.roi_x1 && z >= g.roi_z0 && z <= g.roi_z1) {
            acc.v[0] += fix32<float>(dlt);
            acc.v[1] += fix32<float>(V);
          }
          acc.v[3] += 1;
          if (mag_fx != nullptr && dlt != 0.f) atomicAdd(mag_fx + cur.line, fix32<float>(dlt));
          upd[buf * kSchedGroups + group] = make_int2(cur.line, __float_as_int(nv));
          atomicOr(bits + buf * L.bit_words + (cur.line >> 5), 1u << (cur.line & 31));
          prev_line = cur.line;
        }
      }
    }
    if (gl == 0 && prev_line < 0) upd[buf * kSchedGroups + group] = make_int2(-1, 0);
    __syncthreads();
    cur = nx1;
    nx1 = nx2;
  }

  // store the rows back
  fence_proxy_async_smem();
  __syncthreads();
  for (int v = tid; v < g.n_theta; v += nthreads) {
    bulk_s2g(ge + static_cast<size_t>(tfirst) * sino_plane + static_cast<size_t>(v) * g.n_rp,
             es + v * rs, row_bytes);
    bulk_s2g(A.bfa.sel + static_cast<size_t>(tfirst) * sel_plane + static_cast<size_t>(v) * n_sp,
             ssel + v * srs, static_cast<uint32_t>(n_sp));
  }
  bulk_commit();
  bulk_wait_all();
  if (A.stats != nullptr) {
    double* stat_out = A.stats + static_cast<size_t>(blockIdx.x) * kStatSlots;
    if (gl == 0)
      for (int s = 0; s < kStatSlots; ++s) sstat[group * kStatSlots + s] = acc.v[s];
    __syncthreads();
    if (tid < kStatSlots) {
      unsigned long long t = 0;
      for (int w = 0; w < kSchedGroups; ++w) t += sstat[w * kStatSlots + tid];
      stat_out[tid] = tid < 2 ? static_cast<double>(t) / kFixScale : static_cast<double>(t);
    }
  }
}

template <int NB>
int launch_sched_t(const SweepArgs& a, cudaStream_t s) {
  auto k = sched_sweep_kernel<NB>;
  const size_t smem = sched_layout(a.g.n_theta, a.g.n_z * a.g.n_x, a.n_rs, a.bfa.n_sp).total;
  static const int lim = dyn_smem_limit(k);
  if (smem > static_cast<size_t>(lim)) return -7;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess)
    return -3;
  static int per_sm = 0;
  if (per_sm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  }
  if (per_sm > 0) {
    const int pct =
        static_cast<int>(std::min<size_t>(100, (100 * (smem + 4096) + per_sm - 1) / per_sm));
    cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
  }
  k<<<a.n_slices, kWarps * 32, smem, s>>>(a);
  return ok_or(cudaGetLastError());
}

}  // namespace sweep

size_t sched_sweep_smem(int n_theta, int n_lines, int n_rs, int n_sp) {
  return sweep::sched_layout(n_theta, n_lines, n_rs, n_sp).total;
}

// -7: this configuration is not run by the pipelined kernel (the caller uses the plain one)
int launch_sweep_sched(const SweepArgs& a, int nb, void* stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (a.fp64 || !a.bf || a.mode != kModeICD || !a.smem_rows || a.sched_lines == nullptr ||
      a.acol == nullptr || a.g.n_theta > sweep::kSchedG * sweep::kSchedVPL)
    return -7;
  if (nb == 3) return sweep::launch_sched_t<3>(a, s);  // voxel = detector pixel (fine levels)
  return -7;
}

}  // namespace mbir
