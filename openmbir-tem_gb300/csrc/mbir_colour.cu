// mbir_colour.cu -- the colour schedule of a sparse ICD call, built on the device.
//
// Same result as colour_schedule (mbir_schedule.cpp), the host definition: the call's voxel
// lines (non-empty A-column, in the call's active mask) are visited in ascending line order
// (z-major); each takes the smallest colour that no earlier conflicting line holds and whose
// class has fewer than class_cap lines.  Two lines conflict when they touch a common detector
// bin at some view or are 3x3 (z, x) neighbours.  Output: the lines colour by colour (ascending
// within a colour), the colour offsets and the counts, all in device memory, so the sweep that
// follows reads them without a host round trip.
//
// Lines are coloured 31 at a time (a block).  First, one CTA per block computes the block's
// conflict words from the lines' footprints (bit j of conf[i]: line j < i of the block
// conflicts with line i; conf_p1..conf_p4[i]: line j of the block before, of the one before
// that, and so on, kBack = 4 blocks back); this needs no colours, so every block runs in
// parallel.  Then one CTA of 1024 threads walks the blocks in order, one CTA barrier per block:
// warp 0 colours block b while warps 1-31 bring in, one line each, block b+1's taken-colour sets
// F (the colours of the conflicting lines of the blocks up to b+1-kBack-1, read from bit planes
// per detector bin and per line in global memory) and conflict words, add the colours of the
// conflicting lines of blocks b+2-kBack..b-1 (conflict words), and, once warp 0 has chosen block
// b's colours (a named barrier it arrives at), those of block b.  Warp 0 adds only the colours
// of the earlier lines of the block it colours.
//
// Warp 0's choice is the sequential greedy's, found in parallel: each lane (line) takes the
// first colour free of its set, of the full classes and of the current choices of the earlier
// lines of the block it conflicts with, and the lanes repeat that until no choice changes.
// Line i's choice depends only on lines 0..i-1, so it is final once they are, and the rounds end
// within 31 with exactly the sequential choices; the class caps are then checked in one step
// (each line joined a class below its cap exactly when no class ends above it).  A block whose
// choices leave the 128-colour window or overfill a class is coloured line by line instead.
//
// The bit planes are read and written either by the colouring CTA itself (one-CTA form: warps
// 1-31 OR block b-1's colours into the planes and read block b+1's sets, the planes holding the
// blocks up to b-2) or, the default where cooperative launch is available, by helper CTAs (the
// multi-CTA form).  Helper h takes the blocks h, h+R, h+2R, ... (R helpers): it waits until the
// blocks up to b-kBack-1 are in the planes, reads block b's sets into global memory and flags
// them ready, waits until the colouring CTA has coloured block b, ORs block b's colours into the
// planes and flags block b written.  A set may also hold colours of later blocks that a reader
// happened to see; those belong to lines that conflict with its line, which the conflict words
// add anyway, so both forms give the same schedule.  Every wait on a flag is bounded in time;
// one that runs out raises an abort flag that ends the other CTAs' waits, and the call reports
// a timed-out device wait.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mbir_internal.h"
#include "mbir_schedule.h"

namespace mbir {
namespace {

constexpr int kThreads = 1024;
constexpr int kBlock = 31;  // lines coloured per step
// blocks before a block whose colours reach it through conflict words (the planes a block's
// sets are read from hold the blocks up to b-kBack-1)
constexpr int kBack = 4;
constexpr int kRing = 8;  // colour ring slots (a power of two above kBack)
static_assert(kRing > kBack && (kRing & (kRing - 1)) == 0, "colour ring");

// int32 footprints of 3 blocks, rounded up to 16 bytes so that what follows stays aligned
__host__ __device__ constexpr size_t footprint_ints(int n_theta) {
  return (static_cast<size_t>(3 * kBlock) * n_theta + 3) & ~static_cast<size_t>(3);
}

__device__ __forceinline__ bool bins_overlap(int32_t pi, int32_t pj) {
  const unsigned mi = static_cast<unsigned>(pi) & 0xffffu, mj = static_cast<unsigned>(pj) & 0xffffu;
  if (!mi || !mj) return false;
  const int d = (pj >> 16) - (pi >> 16);  // first bins: lo_j - lo_i
  if (d >= 16 || d <= -16) return false;
  return d >= 0 ? ((mj << d) & mi) != 0u : ((mi << -d) & mj) != 0u;
}

__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += n;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int s = warp_sums[lane];
    int si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += n;
    }
    warp_sums[lane] = si - s;
    if (lane == 31) *total = si;
  }
  __syncthreads();
  return warp_sums[warp] + incl - v;
}

// conflict words of block blockIdx.x of the call's lines: within the block and against the
// kBack blocks before it
__global__ void __launch_bounds__(kThreads) colour_conflicts_kernel(ColourArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nt = A.n_theta, nx = A.n_x;
  int32_t* pk = reinterpret_cast<int32_t*>(smem);  // [(kBack+1) kBlock][nt]: b, b-1, ...
  __shared__ int vz[(kBack + 1) * kBlock], vx[(kBack + 1) * kBlock];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bk = blockIdx.x, s = bk * kBlock;
  const int m = min(kBlock, A.n - s);
  if (m <= 0) return;
  for (int r = warp; r < (kBack + 1) * kBlock; r += kThreads / 32) {
    const int d = r / kBlock, j = r - d * kBlock;  // block bk - d, line j
    if (bk < d || (d == 0 && j >= m)) continue;
    const int l = A.vis[(bk - d) * kBlock + j];
    const int32_t* pl = A.packed + static_cast<size_t>(l) * nt;
    for (int v = lane; v < nt; v += 32) pk[r * nt + v] = pl[v];
    if (lane == 0) {
      vz[r] = l / nx;
      vx[r] = l - (l / nx) * nx;
    }
  }
  __syncthreads();
  if (warp < m) {
    const int i = warp, j = lane;
    unsigned words[kBack + 1];
#pragma unroll
    for (int d = 0; d <= kBack; ++d) {
      bool c = false;
      if (d == 0 ? j < i : (bk >= d && j < kBlock)) {
        const int q = d * kBlock + j;
        c = abs(vz[i] - vz[q]) <= 1 && abs(vx[i] - vx[q]) <= 1;
        for (int v = 0; v < nt && !c; ++v) c = bins_overlap(pk[i * nt + v], pk[q * nt + v]);
      }
      words[d] = __ballot_sync(0xffffffffu, c);
    }
    if (lane == 0) {
      A.conf[s + i] = words[0];
      A.conf_p1[s + i] = words[1];
      A.conf_p2[s + i] = words[2];
      A.conf_p3[s + i] = words[3];
      A.conf_p4[s + i] = words[4];
    }
  }
}

// One warp: the colours taken at the bins (footprints pw) and neighbour lines of line l, words
// below uw, read from the bit planes into Fl[0..W).  Each lane group reads one word pair, its
// lanes over (view, bin), so that consecutive lanes read neighbouring bins and a load touches
// few cache lines; six loads in flight per lane.
__device__ __forceinline__ void load_planes(const ColourArgs& A, int W, int uw, int l,
                                            const int32_t* pw, unsigned long long* Fl) {
  const int lane = threadIdx.x & 31;
  const int nt = A.n_theta, nx = A.n_x, nb = A.nb;
  const int z = l / nx, x = l - z * nx;
  const int np = uw <= 2 ? 1 : uw <= 4 ? 2 : uw <= 8 ? 4 : 8;  // word pairs read (W 2..16)
  const int gs = 32 / np;                        // lanes per word pair
  const int kk = lane / gs, sub = lane - kk * gs;
  const int dv = gs / nb, db = gs - dv * nb;
  // the neighbour lines first, in flight with the first bin loads
  ulonglong2 un = make_ulonglong2(0ull, 0ull);
  for (int q = sub; q < 9; q += gs) {
    const int zz = z + q / 3 - 1, xx = x + q % 3 - 1;
    if (zz >= 0 && zz < A.n_z && xx >= 0 && xx < nx) {
      const size_t row = (static_cast<size_t>(zz) * nx + xx) * W;
      const ulonglong2 u = __ldcg(reinterpret_cast<const ulonglong2*>(A.line_used + row) + kk);
      un.x |= u.x;
      un.y |= u.y;
    }
  }
  unsigned long long fx = 0ull, fy = 0ull;
  int v = sub / nb, b = sub - (sub / nb) * nb;
  while (v < nt) {
    ulonglong2 q[6];
#pragma unroll
    for (int u = 0; u < 6; ++u) {
      q[u] = make_ulonglong2(0ull, 0ull);
      if (v < nt) {
        const int32_t p = pw[v];
        if ((static_cast<unsigned>(p) >> b) & 1u) {
          const size_t row = (static_cast<size_t>(v) * A.n_r + (p >> 16) + b) * W;
          q[u] = __ldcg(reinterpret_cast<const ulonglong2*>(A.bin_used + row) + kk);
        }
      }
      v += dv;
      b += db;
      if (b >= nb) {
        b -= nb;
        ++v;
      }
    }
#pragma unroll
    for (int u = 0; u < 6; ++u) {
      fx |= q[u].x;
      fy |= q[u].y;
    }
  }
  fx |= un.x;
  fy |= un.y;
  for (int o = gs >> 1; o > 0; o >>= 1) {
    fx |= __shfl_xor_sync(0xffffffffu, fx, o);
    fy |= __shfl_xor_sync(0xffffffffu, fy, o);
  }
  if (sub == 0) {
    Fl[2 * kk] = fx;
    Fl[2 * kk + 1] = fy;
  }
  if (lane == 0)  // words from 2 np on hold no colours of these planes
    for (int k = 2 * np; k < W; ++k) Fl[k] = 0ull;
}

// One warp: colour c of line l (footprints pw) ORed into the bit planes of its bins and line,
// lanes over (view, bin); not waited for.
__device__ __forceinline__ void set_line(const ColourArgs& A, int W, const int32_t* pw, int l,
                                         int c) {
  const int lane = threadIdx.x & 31;
  const int nt = A.n_theta, nb = A.nb;
  const unsigned long long bit = 1ull << (c & 63);
  const int wk = c >> 6;
  const int dv = 32 / nb, db = 32 - dv * nb;
  for (int v = lane / nb, b = lane - (lane / nb) * nb; v < nt;) {
    const int32_t p = pw[v];
    if ((static_cast<unsigned>(p) >> b) & 1u)
      atomicOr(A.bin_used + (static_cast<size_t>(v) * A.n_r + (p >> 16) + b) * W + wk, bit);
    v += dv;
    b += db;
    if (b >= nb) {
      b -= nb;
      ++v;
    }
  }
  if (lane == 0) atomicOr(A.line_used + static_cast<size_t>(l) * W + wk, bit);
}

__device__ __forceinline__ uint64_t colour_clock_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Wait (one thread) until *flag is nonzero; returns its value, or 0 when the abort flag is up or
// the wait ran out of time (which raises the abort flag and ORs 2 into the error word).
__device__ int wait_flag(const ColourArgs& A, const int* flag) {
  int v = ld_acquire(flag);
  if (v) return v;
  const uint64_t t0 = colour_clock_ns();
  unsigned ns = 32;
  for (unsigned it = 0;; ++it) {
    v = ld_acquire(flag);
    if (v) return v;
    if (ld_acquire(A.abort_flag)) return 0;
    if ((it & 15u) == 15u && colour_clock_ns() - t0 > A.wait_ns) {
      atomicExch(A.abort_flag, 1);
      atomicOr(A.err, 2);
      return 0;
    }
    __nanosleep(ns);
    if (ns < 128) ns <<= 1;
  }
}

// Helper CTA of the multi-CTA form: the taken-colour sets of its blocks (read from the planes
// once the blocks up to b-kBack-1 are in them), then its blocks' colours into the planes.
__device__ void colour_helper(const ColourArgs& A, unsigned char* smem) {
  const int W = A.words, nt = A.n_theta, n = A.n;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nblk = (n + kBlock - 1) / kBlock;
  int* ready = A.flags;
  int* coloured = A.flags + nblk;
  int* written = A.flags + 2 * nblk;
  int32_t* pk = reinterpret_cast<int32_t*>(smem);  // [kBlock][nt] footprints of the block
  __shared__ int hline[kBlock];
  __shared__ int s_ok, s_uw;
  int wm = 0;  // thread 0: blocks [0, wm) are known to be in the planes
  for (int b = blockIdx.x - 1; b < nblk; b += gridDim.x - 1) {
    const int s = b * kBlock, m = min(kBlock, n - s);
    if (warp < m) {
      const int l = A.vis[s + warp];
      const int32_t* pl = A.packed + static_cast<size_t>(l) * nt;
      for (int v = lane; v < nt; v += 32) pk[warp * nt + v] = pl[v];
      if (lane == 0) hline[warp] = l;
    }
    if (tid == 0) {
      int ok = 1;
      for (; wm <= b - kBack - 1 && ok; ++wm) ok = wait_flag(A, written + wm) != 0;
      s_ok = ok;
      // words holding the colours of the blocks up to b-kBack-1
      s_uw = (ok && b > kBack) ? min((ld_acquire(coloured + b - kBack - 1) - 1) / 64 + 1, W) : 1;
    }
    __syncthreads();
    if (!s_ok) return;
    if (warp < m)
      load_planes(A, W, s_uw, hline[warp], pk + warp * nt,
                  A.fsets + (static_cast<size_t>(s) + warp) * W);
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release(ready + b, 1);
      s_ok = wait_flag(A, coloured + b) > 0;
    }
    __syncthreads();
    if (!s_ok) return;
    if (warp < m) {
      const int c = __ldcg(A.colour + s + warp);
      set_line(A, W, pk + warp * nt, hline[warp], c);
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release(written + b, 1);
    }
  }
}

// One warp, line j of the next block: the colours of its conflicting lines in N earlier blocks
// (conflict words b[d], colours c[d] a lane each) ORed into its set Fl, one warp reduction per
// colour word that holds one of them (the colours of a few neighbouring blocks share one or two).
template <int N>
__device__ __forceinline__ void add_older(unsigned long long* Fl, int W, const unsigned* b,
                                          const int* const* c) {
  const int lane = threadIdx.x & 31;
  int q[N];
#pragma unroll
  for (int d = 0; d < N; ++d) q[d] = ((b[d] >> lane) & 1u) ? c[d][lane] : -1;
  for (;;) {
    int fw = 0x7fffffff;  // this lane's lowest word still to add
#pragma unroll
    for (int d = 0; d < N; ++d)
      if (q[d] >= 0) fw = min(fw, q[d] >> 6);
    const unsigned pend = __ballot_sync(0xffffffffu, fw != 0x7fffffff);
    if (!pend) break;
    const int w = __shfl_sync(0xffffffffu, fw, __ffs(pend) - 1);
    unsigned lo = 0u, hi = 0u;
#pragma unroll
    for (int d = 0; d < N; ++d)
      if (q[d] >= 0 && (q[d] >> 6) == w) {
        const int r = q[d] & 63;
        if (r < 32) lo |= 1u << r; else hi |= 1u << (r - 32);
        q[d] = -1;
      }
    lo = __reduce_or_sync(0xffffffffu, lo);
    hi = __reduce_or_sync(0xffffffffu, hi);
    if (lane == 0 && w < W) Fl[w] |= (static_cast<unsigned long long>(hi) << 32) | lo;
  }
  __syncwarp();
}

// One warp, line j of the next block, its set Fl complete: the lowest colour free of the set
// and of the full classes (64 W: none) into *lowest.
__device__ __forceinline__ void note_lowest_free(const unsigned long long* Fl, int W,
                                                 const unsigned long long* full, int* lowest) {
  const int lane = threadIdx.x & 31;
  const unsigned long long t = lane < W ? (Fl[lane] | full[lane]) : ~0ull;
  const unsigned words = __ballot_sync(0xffffffffu, ~t != 0ull);
  if (lane == 0) {
    int first = 64 * W;
    if (words) {
      const int k = __ffs(words) - 1;
      first = 64 * k + __ffsll(static_cast<long long>(~(Fl[k] | full[k]))) - 1;
    }
    *lowest = first;
  }
}

// Named barrier 1 of the colouring CTA, once a step: warp 0 arrives when it has chosen the
// step's colours (in shared memory), the reading warps wait there before adding them to the
// next block's sets.  A hardware barrier that every warp reaches once per step, no spin.
__device__ __forceinline__ void colours_chosen_arrive() {
  asm volatile("bar.arrive 1, %0;" ::"n"(kThreads) : "memory");
}
__device__ __forceinline__ void colours_chosen_wait() {
  asm volatile("bar.sync 1, %0;" ::"n"(kThreads) : "memory");
}

template <bool PIPE>
__global__ void __launch_bounds__(kThreads, 1) colour_kernel(ColourArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (PIPE && blockIdx.x > 0) {
    colour_helper(A, smem);
    return;
  }
  const int W = A.words;
  const int nt = A.n_theta;
  int32_t* pk = reinterpret_cast<int32_t*>(smem);  // [3][kBlock][nt] footprints, block index % 3
  // [2][kBlock][W] colours taken for each line of a block, by block parity
  unsigned long long* F = reinterpret_cast<unsigned long long*>(pk + footprint_ints(nt));
  int* csize = reinterpret_cast<int*>(F + 2 * kBlock * W);  // [64 W] class sizes
  __shared__ unsigned conf[2][32];            // in-block conflict words, by block parity
  __shared__ int col[kRing][32];              // colours (a lane each), block index % kRing
  __shared__ int choice[32];                  // warp 0: the current choices of a block's lines
  __shared__ int vline[3][32];
  __shared__ int warp_sums[32];
  __shared__ unsigned long long full_s[16];
  __shared__ int s_total, s_ncol[2], s_fail;
  __shared__ int s_first[2][32];  // each line's lowest free colour, by block parity
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int c = tid; c < 64 * W; c += kThreads) csize[c] = 0;
  if (tid < 32) s_first[0][tid] = 0;  // block 0: nothing coloured yet
  if (tid < 16) full_s[tid] = 0ull;
  if (tid == 0) {
    s_ncol[0] = 0;
    s_fail = 0;

  }
  const int n = A.n;  // the call's lines, ascending, in A.vis
  __syncthreads();

  // phase 1: colour kBlock lines per step; block 0's lines need no planes (nothing coloured)
  static_assert(kThreads / 32 - 1 == kBlock, "one reading warp per line of a block");
  const int nblk = (n + kBlock - 1) / kBlock;
  int ncol_w = 0;  // warp 0: colours so far
  if (warp < min(kBlock, n)) {
    const int l = A.vis[warp];
    const int32_t* pl = A.packed + static_cast<size_t>(l) * nt;
    for (int v = lane; v < nt; v += 32) pk[warp * nt + v] = pl[v];
    if (lane < W) F[warp * W + lane] = 0ull;
    if (lane == 0) {
      vline[0][warp] = l;
      conf[0][warp] = A.conf[warp];
    }
  }
  auto publish = [&](int b) {
    const int sb = b * kBlock, mb = min(kBlock, n - sb);
    if (lane < mb) A.colour[sb + lane] = static_cast<int16_t>(col[b & (kRing - 1)][lane]);
    if (PIPE) {
      __syncwarp();
      if (lane == 0) {
        __threadfence();
        st_release(A.flags + nblk + b, s_ncol[(b + 1) & 1] + 1);
      }
    }
    __syncwarp();
  };
  // reading warps: the line of block 1 (read a step ahead from here on)
  int l_ahead = warp >= 1 && kBlock + warp - 1 < n ? A.vis[kBlock + warp - 1] : 0;
  __syncthreads();
  for (int bk = 0; bk < nblk; ++bk) {
    const int s = bk * kBlock, m = min(kBlock, n - s);
    const int mp = bk > 0 ? kBlock : 0;                                 // lines of block bk-1
    const int mn = bk + 1 < nblk ? min(kBlock, n - s - kBlock) : 0;  // lines of block bk+1
    const int nxt = (bk + 1) % 3, prv = (bk + 2) % 3;
    const int ccur = bk & (kRing - 1);  // col ring slot of block bk
    const int fc = bk & 1, fn = fc ^ 1;
    // warp 1: block bk-1's colours to global memory and, in the multi-CTA form, to its helper
    // (value: colours so far + 1); its memory fence stays off warp 0's path
    if (warp == 1 && bk > 0) publish(bk - 1);
    if (warp == 0) {
      // The greedy choice of block bk.  Line i's taken colours: its set F (colours of the
      // conflicting lines of the blocks before bk, built by the reading warps in step bk-1),
      // those of its conflicting lines in block bk before it, and the full classes.  Fast form on a 128-colour window from base (the lowest colour
      // free for some line; lower colours are taken or full for every line): every lane takes
      // the first free colour given the current choices of the earlier lines it conflicts
      // with, repeated until no choice changes -- line i's choice is final once lines 0..i-1
      // are, so this ends within kBlock rounds with the sequential greedy's choices -- then the
      // class caps are checked (every line joined a class below its cap exactly when no class
      // ends above it).  A block whose choices leave the window or overfill a class takes the
      // sequential form below.
      const unsigned long long* Fb = F + fc * kBlock * W;
      const int cap = A.class_cap > 0 ? A.class_cap : 0x7fffffff;
      const bool act = lane < m;
      const unsigned my_conf = act ? conf[fc][lane] : 0u;
      // each line's lowest free colour was noted by its reading warp as its set was completed
      int base = act ? s_first[fc][lane] : 64 * W;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) base = min(base, __shfl_xor_sync(0xffffffffu, base, o));
      const int k0 = base >> 6, sh = base & 63;
      // 128 colours from base as two words; colours from max_colours on count as full
      auto win = [&](const unsigned long long* v, unsigned long long& w0, unsigned long long& w1) {
        const unsigned long long a = k0 < W ? v[k0] : ~0ull, b = k0 + 1 < W ? v[k0 + 1] : ~0ull,
                                 c = k0 + 2 < W ? v[k0 + 2] : ~0ull;
        w0 = sh ? (a >> sh) | (b << (64 - sh)) : a;
        w1 = sh ? (b >> sh) | (c << (64 - sh)) : b;
      };
      unsigned long long f0 = ~0ull, f1 = ~0ull, u0, u1;
      if (act) win(Fb + lane * W, f0, f1);
      win(full_s, u0, u1);
      const int lim = A.max_colours - base;
      f0 |= u0 | (lim >= 64 ? 0ull : lim <= 0 ? ~0ull : ~0ull << lim);
      f1 |= u1 | (lim >= 128 ? 0ull : lim <= 64 ? ~0ull : ~0ull << (lim - 64));
      // colour c as its bit in the window's two words (none outside the window)
      auto bit0 = [&](int c) {
        const unsigned r = static_cast<unsigned>(c - base);
        return r < 64u ? 1ull << r : 0ull;
      };
      auto bit1 = [&](int c) {
        const unsigned r = static_cast<unsigned>(c - base) - 64u;
        return r < 64u ? 1ull << r : 0ull;
      };
      // the colours of the lanes of bits b in table t, four loads in flight at a time (a bit
      // taken twice adds its colour twice, which changes nothing)
      auto add_bits = [&](unsigned long long& w0, unsigned long long& w1, unsigned b,
                          const int* t) {
        while (b) {
          const int k0 = __ffs(b) - 1;
          b &= b - 1u;
          const int k1 = b ? __ffs(b) - 1 : k0;
          b &= b - 1u;
          const int k2 = b ? __ffs(b) - 1 : k0;
          b &= b - 1u;
          const int k3 = b ? __ffs(b) - 1 : k0;
          b &= b - 1u;
          const int c0 = t[k0], c1 = t[k1], c2 = t[k2], c3 = t[k3];
          w0 |= (bit0(c0) | bit0(c1)) | (bit0(c2) | bit0(c3));
          w1 |= (bit1(c0) | bit1(c1)) | (bit1(c2) | bit1(c3));
        }
      };
      auto first_free = [](unsigned long long w0, unsigned long long w1) {
        return ~w0 ? __ffsll(static_cast<long long>(~w0)) - 1
                   : (~w1 ? 63 + __ffsll(static_cast<long long>(~w1)) : -1);
      };
      // one round: each line's first free colour given the current choices of the earlier
      // lines it conflicts with and the classes the earlier lines fill (a class is full for
      // line i once its count before the block plus the earlier lines' choices of it reach the
      // cap: the filling line is the one that takes its last place)
      const unsigned lt = (1u << lane) - 1u;
      int c = act ? first_free(f0, f1) : -1;
      int room = 0;
      bool settled = false;
      for (int r = 0; r <= kBlock; ++r) {
        const bool has = act && c >= 0;
        const unsigned grp = __match_any_sync(0xffffffffu, has ? c : -2 - lane);
        room = has ? cap - csize[base + c] : 0;
        const unsigned fills =
            __ballot_sync(0xffffffffu, has && __popc(grp & lt) + 1 == room);
        choice[lane] = c >= 0 ? base + c : -1;
        __syncwarp();
        unsigned long long x0 = f0, x1 = f1;
        add_bits(x0, x1, act ? (my_conf | (fills & lt)) : 0u, choice);
        __syncwarp();
        const int nc = act ? first_free(x0, x1) : c;
        const bool changed = __any_sync(0xffffffffu, nc != c);
        c = nc;
        if (!changed) {
          settled = true;
          break;
        }
      }
      const unsigned grp = __match_any_sync(0xffffffffu, act ? c : -2 - lane);
      const int cls = base + c;
      const int before = (act && c >= 0) ? csize[cls] : 0;
      const bool ok = !act || (c >= 0 && before + __popc(grp) <= cap);
      int mine = -1;
      bool fail = false;
      if (__all_sync(0xffffffffu, ok) && settled && !A.sequential) {
        mine = act ? cls : -1;
        if (act && lane == __ffs(grp) - 1) {
          const int nv = before + __popc(grp);
          csize[cls] = nv;
          if (nv >= cap) atomicOr(&full_s[cls >> 6], 1ull << (cls & 63));
        }
        col[ccur][lane] = mine;
        __syncwarp();
      } else {
        // sequential form: line by line on a 64-colour window
        int sbase = 64 * W;
        if (act)
          for (int k = 0; k < W; ++k) {
            const unsigned long long t = Fb[lane * W + k] | full_s[k];
            if (~t) {
              sbase = 64 * k + __ffsll(static_cast<long long>(~t)) - 1;
              break;
            }
          }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sbase = min(sbase, __shfl_xor_sync(0xffffffffu, sbase, o));
        const int sk0 = sbase >> 6, ssh = sbase & 63;
        auto window = [&](const unsigned long long* v) {
          const unsigned long long lo = sk0 < W ? v[sk0] : 0ull, hi = sk0 + 1 < W ? v[sk0 + 1] : 0ull;
          return ssh ? (lo >> ssh) | (hi << (64 - ssh)) : lo;
        };
        unsigned long long acc = act ? window(Fb + lane * W) : 0ull;
        const int slim = A.max_colours - sbase;
        unsigned long long fullw =
            window(full_s) | (slim >= 64 ? 0ull : slim <= 0 ? ~0ull : ~0ull << slim);
        const int cl = sbase + lane, ch = sbase + 32 + lane;  // this lane's two window classes
        int n_lo = cl < 64 * W ? csize[cl] : 0, n_hi = ch < 64 * W ? csize[ch] : 0;
        auto write_back = [&]() {
          col[ccur][lane] = mine;
          if (cl < 64 * W) {
            csize[cl] = n_lo;
            if (n_lo >= cap) atomicOr(&full_s[cl >> 6], 1ull << (cl & 63));
          }
          if (ch < 64 * W) {
            csize[ch] = n_hi;
            if (n_hi >= cap) atomicOr(&full_s[ch >> 6], 1ull << (ch & 63));
          }
          __syncwarp();
        };
        for (int i = 0; i < m; ++i) {
          const int first = __ffsll(static_cast<long long>(~(acc | fullw))) - 1;  // -1: none
          const int rel = __shfl_sync(0xffffffffu, first, i);
          if (rel < 0) {  // window exhausted for line i: the exact choice from the shared copies
            write_back();
            int cc = -1;
            if (lane == i)
              for (int k = 0; k < W && cc < 0; ++k) {
                unsigned long long t = Fb[i * W + k] | full_s[k];
                for (unsigned b = my_conf; b; b &= b - 1u) {
                  const int q = col[ccur][__ffs(b) - 1];
                  if ((q >> 6) == k) t |= 1ull << (q & 63);
                }
                if (~t) cc = 64 * k + __ffsll(static_cast<long long>(~t)) - 1;
              }
            const int cw = __shfl_sync(0xffffffffu, cc, i);
            if (cw < 0 || cw >= A.max_colours) {
              fail = true;
              break;
            }
            mine = lane == i ? cw : mine;  // beyond the window: counted in shared memory
            if (lane == 0 && ++csize[cw] >= cap) full_s[cw >> 6] |= 1ull << (cw & 63);
            __syncwarp();
            continue;
          }
          mine = lane == i ? sbase + rel : mine;
          acc |= ((my_conf >> i) & 1u) ? 1ull << rel : 0ull;
          n_lo += rel == lane;
          n_hi += rel == lane + 32;
          fullw |= (static_cast<unsigned long long>(__ballot_sync(0xffffffffu, n_hi >= cap)) << 32) |
                   __ballot_sync(0xffffffffu, n_lo >= cap);
        }
        write_back();
      }
      int top = mine;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(0xffffffffu, top, o));
      ncol_w = max(ncol_w, top + 1);
      if (lane == 0) {
        if (fail) atomicOr(&s_fail, 1);  // 1: colours exhausted, 2: a wait failed
        if (PIPE && fail) atomicExch(A.abort_flag, 1);
        s_ncol[fn] = ncol_w;
      }
      __syncwarp();
      colours_chosen_arrive();  // block bk's colours are in col: the reading warps add them
    } else if (PIPE) {
      // warps 1-31, one line j each: block bk+1's taken-colour sets, from its helper
      const int j = warp - 1;
      unsigned long long* Fl = F + (fn * kBlock + j) * W;
      unsigned b1 = 0u;  // conflicts with block bk, added once warp 0 has chosen its colours
      bool have = false;
      if (j < mn) {
        const int ok = lane == 0 ? wait_flag(A, A.flags + bk + 1) : 0;
        if (__shfl_sync(0xffffffffu, ok, 0) == 0) {
          if (lane == 0) atomicOr(&s_fail, 2);
        } else {
          const int q = s + kBlock + j;
          if (lane < W) Fl[lane] = __ldcg(A.fsets + static_cast<size_t>(q) * W + lane);
          const unsigned bo[kBack - 1] = {A.conf_p2[q], A.conf_p3[q], A.conf_p4[q]};
          const int* co[kBack - 1] = {col[(bk + kRing - 1) & (kRing - 1)],
                                      col[(bk + kRing - 2) & (kRing - 1)],
                                      col[(bk + kRing - 3) & (kRing - 1)]};
          __syncwarp();
          add_older<kBack - 1>(Fl, W, bo, co);
          if (lane == 0) {
            vline[nxt][j] = A.vis[q];
            conf[fn][j] = A.conf[q];
          }
          b1 = A.conf_p1[q];
          have = true;
        }
      }
      colours_chosen_wait();
      if (b1) {
        const int* co[1] = {col[ccur]};
        add_older<1>(Fl, W, &b1, co);
      }
      if (have) note_lowest_free(Fl, W, full_s, &s_first[fn][j]);
    } else {
      // warps 1-31, one line j each: the footprints of block bk+1's line (its line read a step
      // ahead) requested first, block bk-1's colours into the planes meanwhile, then block
      // bk+1's colour sets (the planes hold the blocks up to bk-2)
      const int j = warp - 1;
      const int uw = min(s_ncol[fc] / 64 + 1, W);  // words holding colours of blocks before bk
      const int l = l_ahead;
      const int32_t* pl = A.packed + static_cast<size_t>(l) * nt;
      int32_t f0 = 0, f1 = 0;
      unsigned cw = 0u, cw1 = 0u, cw2 = 0u, cw3 = 0u, cw4 = 0u;
      if (j < mn) {
        if (lane < nt) f0 = pl[lane];
        if (lane + 32 < nt) f1 = pl[lane + 32];
        cw = A.conf[s + kBlock + j];
        cw1 = A.conf_p1[s + kBlock + j];
        cw2 = A.conf_p2[s + kBlock + j];
        cw3 = A.conf_p3[s + kBlock + j];
        cw4 = A.conf_p4[s + kBlock + j];
      }
      l_ahead = s + 2 * kBlock + j < n ? A.vis[s + 2 * kBlock + j] : 0;
      if (j < mp)
        set_line(A, W, pk + (prv * kBlock + j) * nt, vline[prv][j],
                 col[(bk + kRing - 1) & (kRing - 1)][j]);
      if (j < mn) {
        int32_t* pw = pk + (nxt * kBlock + j) * nt;
        if (lane < nt) pw[lane] = f0;
        if (lane + 32 < nt) pw[lane + 32] = f1;
        for (int v = lane + 64; v < nt; v += 32) pw[v] = pl[v];
        __syncwarp();
        load_planes(A, W, uw, l, pw, F + (fn * kBlock + j) * W);
        __syncwarp();
        const unsigned bo[kBack - 1] = {cw2, cw3, cw4};
        const int* co[kBack - 1] = {col[(bk + kRing - 1) & (kRing - 1)],
                                    col[(bk + kRing - 2) & (kRing - 1)],
                                    col[(bk + kRing - 3) & (kRing - 1)]};
        add_older<kBack - 1>(F + (fn * kBlock + j) * W, W, bo, co);
        if (lane == 0) {
          vline[nxt][j] = l;
          conf[fn][j] = cw;
        }
      }
      colours_chosen_wait();  // cw1: conflicts with block bk (zero without a line j)
      if (cw1) {
        const int* co[1] = {col[ccur]};
        add_older<1>(F + (fn * kBlock + j) * W, W, &cw1, co);
      }
      if (j < mn) note_lowest_free(F + (fn * kBlock + j) * W, W, full_s, &s_first[fn][j]);
    }
    __threadfence_block();  // this step's plane updates land before the next step reads
    __syncthreads();
    if (s_fail) break;
  }
  if (warp == 1 && !s_fail && nblk > 0) publish(nblk - 1);
  if (s_fail) {
    if (tid == 0) {
      A.count[0] = 0;
      A.count[1] = 0;
      if (s_fail & 1) atomicOr(A.err, 4);
      if (PIPE) atomicExch(A.abort_flag, 1);
    }
    return;
  }
  // phase 2: colour offsets, lines colour by colour, ascending within a colour
  const int ncol = s_ncol[nblk & 1];
  int cs = 0;
  const int cper = (ncol + kThreads - 1) / kThreads;
  const int c0 = min(tid * cper, ncol), c1 = min(c0 + cper, ncol);
  for (int c = c0; c < c1; ++c) cs += csize[c];
  int off = block_exclusive_scan(cs, warp_sums, &s_total);
  for (int c = c0; c < c1; ++c) {
    A.lofs[c] = off;
    const int sz = csize[c];
    csize[c] = off;  // cursor
    off += sz;
  }
  if (tid == 0) {
    A.lofs[ncol] = n;
    A.count[0] = n;
    A.count[1] = ncol;
  }
  __syncthreads();
  for (int i = tid; i < n; i += kThreads) {
    const int p = atomicAdd(&csize[A.colour[i]], 1);
    A.lines[p] = A.vis[i];
  }
  __syncthreads();
  __threadfence_block();
  // sort each class ascending (classes hold at most 32 lines): one warp per class
  for (int c = warp; c < ncol; c += kThreads / 32) {
    const int b = A.lofs[c], e = (c + 1 < ncol) ? A.lofs[c + 1] : n;
    int v = (lane < e - b) ? A.lines[b + lane] : 0x7fffffff;
    // bitonic sort across the warp
    for (int k = 2; k <= 32; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        const int o = __shfl_xor_sync(0xffffffffu, v, j);
        const bool up = ((lane & k) == 0);
        const bool lower = (lane & j) == 0;
        v = (lower == up) ? min(v, o) : max(v, o);
      }
    if (lane < e - b) A.lines[b + lane] = v;
  }
}

// packed[i] = packed_footprint of table entry i (wf floats each), i < n
__global__ void pack_footprints_kernel(const float* __restrict__ table, size_t n, int wf, int nb,
                                       int32_t* __restrict__ packed) {
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    packed[i] = packed_footprint(table + i * wf, nb);
}

}  // namespace

int launch_pack_footprints(const float4* table, size_t n, int nb, int32_t* packed, void* stream) {
  if (nb < 1 || nb > 16) return -7;
  if (n == 0) return 0;
  constexpr int kPackThreads = 256;
  const size_t blocks = std::min<size_t>((n + kPackThreads - 1) / kPackThreads, 152 * 16);
  pack_footprints_kernel<<<static_cast<unsigned>(blocks), kPackThreads, 0,
                           static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float*>(table), n, 4 * acol_width(nb), nb, packed);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t colour_smem_bytes(int n_theta, int words) {
  return sizeof(int32_t) * footprint_ints(n_theta) +
         sizeof(unsigned long long) * 2 * kBlock * words +
         sizeof(int) * 64 * words;
}

bool colour_schedule_fits(int n_theta, int words) {
  static const int lim_c = dyn_smem_limit(colour_conflicts_kernel);
  static const int lim_k = dyn_smem_limit(colour_kernel<false>);
  return sizeof(int32_t) * (kBack + 1) * kBlock * n_theta <= static_cast<size_t>(lim_c) &&
         colour_smem_bytes(n_theta, words) <= static_cast<size_t>(lim_k);
}

int launch_colour_schedule(const ColourArgs& a, void* stream) {
  if ((a.words != 2 && a.words != 4 && a.words != 8 && a.words != 16) ||
      a.max_colours > 64 * a.words ||
      a.class_cap < 1 || a.class_cap > 32 || a.nb > 16)
    return -7;
  // an error left pending by an earlier call on this thread is reported as such
  const cudaError_t pending = cudaGetLastError();
  if (pending != cudaSuccess) return -1000 - static_cast<int>(pending);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t bins = static_cast<size_t>(a.n_theta) * a.n_r * a.words;
  const size_t lines = static_cast<size_t>(a.n_z) * a.n_x * a.words;
  cudaMemsetAsync(a.bin_used, 0, bins * sizeof(unsigned long long), s);
  cudaMemsetAsync(a.line_used, 0, lines * sizeof(unsigned long long), s);
  if (a.n > 0) {
    const size_t csm = sizeof(int32_t) * (kBack + 1) * kBlock * a.n_theta;
    static const int lim = dyn_smem_limit(colour_conflicts_kernel);
    if (csm > static_cast<size_t>(lim)) return -7;
    cudaError_t e = cudaFuncSetAttribute(colour_conflicts_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return -2000 - static_cast<int>(e);
    colour_conflicts_kernel<<<(a.n + kBlock - 1) / kBlock, kThreads, csm, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return -3000 - static_cast<int>(e);
  }
  const size_t smem = colour_smem_bytes(a.n_theta, a.words);
  static const int lim = dyn_smem_limit(colour_kernel<false>);
  if (smem > static_cast<size_t>(lim)) return -7;
  const int nblk = (a.n + kBlock - 1) / kBlock;
  static const bool coop = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrCooperativeLaunch, dev);
    return v != 0;
  }();
  if (a.helpers > 0 && a.fsets != nullptr && a.flags != nullptr && a.abort_flag != nullptr &&
      coop && nblk > 1) {
    const int helpers = std::min(a.helpers, nblk);
    cudaMemsetAsync(a.flags, 0, sizeof(int) * 3 * static_cast<size_t>(nblk), s);
    cudaMemsetAsync(a.abort_flag, 0, sizeof(int), s);
    cudaError_t e = cudaFuncSetAttribute(colour_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return -4000 - static_cast<int>(e);
    ColourArgs arg = a;
    void* params[] = {&arg};
    e = cudaLaunchCooperativeKernel(reinterpret_cast<void*>(colour_kernel<true>),
                                    dim3(1 + helpers), dim3(kThreads), params, smem, s);
    return e == cudaSuccess ? 0 : -5000 - static_cast<int>(e);
  }
  cudaError_t e = cudaFuncSetAttribute(colour_kernel<false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  if (e != cudaSuccess) return -4000 - static_cast<int>(e);
  colour_kernel<false><<<1, kThreads, smem, s>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : -5000 - static_cast<int>(e);
}

}  // namespace mbir
