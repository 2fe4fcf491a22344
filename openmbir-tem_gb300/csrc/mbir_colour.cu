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
// Lines are coloured 31 at a time (a block: warp 0 colours one block while the other 31 warps
// read for the next, one line each).  First, one CTA per block computes the block's
// conflict words from the lines' footprints (bit j of conf[i]: line j < i of the block
// conflicts with line i; conf_p1[i], conf_p2[i]: line j of the block before, of the one before
// that); this needs no colours, so every block runs in parallel.  Then one CTA of 1024 threads
// walks the blocks in order.  While warp 0 assigns the colours of block b in order (the
// sequential greedy choice, because each line also sees the colours of the earlier lines of its
// block that it conflicts with), warps 1-31 OR the colours of block b-1 into the bit planes of
// its bins and lines (global memory, L2-resident) and read, for block b+1, the planes of each
// line's bins and neighbours.  Those hold every block before b-1; the colours of blocks b-1 and
// b that a line must see (those of the lines it conflicts with) are added from conf_p2 and
// conf_p1 once block b is coloured, so the planes being updated meanwhile change nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mbir_internal.h"
#include "mbir_schedule.h"

namespace mbir {
namespace {

constexpr int kThreads = 1024;
constexpr int kBlock = 31;  // lines coloured per step

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

// conflict words of block blockIdx.x of the call's lines: within the block and against the two
// blocks before it
__global__ void __launch_bounds__(kThreads) colour_conflicts_kernel(ColourArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nt = A.n_theta, nx = A.n_x;
  int32_t* pk = reinterpret_cast<int32_t*>(smem);  // [3 kBlock][nt]: this block, b-1, b-2
  __shared__ int vz[3 * kBlock], vx[3 * kBlock];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bk = blockIdx.x, s = bk * kBlock;
  const int m = min(kBlock, A.n - s);
  if (m <= 0) return;
  for (int r = warp; r < 3 * kBlock; r += kThreads / 32) {
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
    unsigned words[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
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
  const int np = uw <= 2 ? 1 : uw <= 4 ? 2 : 4;  // word pairs read (W is 2, 4 or 8)
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

__global__ void __launch_bounds__(kThreads, 1) colour_kernel(ColourArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int W = A.words;
  const int nt = A.n_theta;
  int32_t* pk = reinterpret_cast<int32_t*>(smem);  // [3][kBlock][nt] footprints, block index % 3
  // [2][kBlock][W] colours taken for each line of a block, by block parity
  unsigned long long* F = reinterpret_cast<unsigned long long*>(pk + footprint_ints(nt));
  int* csize = reinterpret_cast<int*>(F + 2 * kBlock * W);  // [64 W] class sizes
  __shared__ unsigned conf[2][32];  // in-block conflict words, by block parity
  __shared__ unsigned cprev[2][32];  // the next block's words against blocks b and b-1
  __shared__ int col[3][32];        // colours (a lane each), block index % 3
  __shared__ int vline[3][32];
  __shared__ int warp_sums[32];
  __shared__ unsigned long long full_s[8];
  __shared__ int s_total, s_ncol, s_fail;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int c = tid; c < 64 * W; c += kThreads) csize[c] = 0;
  if (tid < 8) full_s[tid] = 0ull;
  if (tid == 0) {
    s_ncol = 0;
    s_fail = 0;
  }
  const int n = A.n;  // the call's lines, ascending, in A.vis
  __syncthreads();

  // phase 1: colour kBlock lines per step; block 0's lines need no planes (nothing coloured)
  static_assert(kThreads / 32 - 1 == kBlock, "one reading warp per line of a block");
  const int nblk = (n + kBlock - 1) / kBlock;
  int ncol_w = 0;  // warp 0: colours so far, published in s_ncol between steps
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
  // reading warps: the line of block 1 (read a step ahead from here on)
  int l_ahead = warp >= 1 && kBlock + warp - 1 < n ? A.vis[kBlock + warp - 1] : 0;
  __syncthreads();
  for (int bk = 0; bk < nblk; ++bk) {
    const int s = bk * kBlock, m = min(kBlock, n - s);
    const int mp = bk > 0 ? kBlock : 0;                                 // lines of block bk-1
    const int mn = bk + 1 < nblk ? min(kBlock, n - s - kBlock) : 0;  // lines of block bk+1
    const int cur = bk % 3, nxt = (bk + 1) % 3, prv = (bk + 2) % 3;
    const int fc = bk & 1, fn = fc ^ 1;
    // warp 0: the greedy choice, line by line, on a window of 64 colours from base, the lowest
    // colour free for some line of the block (colours below it are full or taken for every
    // line, and stay so).  Every lane keeps in
    // registers its line's taken colours of the window, the window's full classes and the sizes
    // of two of its classes, and finds its first free colour; line i takes lane i's.  A line
    // with no free colour in the window takes the first free colour found from the shared
    // copies (written back for it); classes beyond the window are counted in shared memory.
    if (warp == 0) {
      const unsigned long long* Fb = F + fc * kBlock * W;
      int base = 64 * W;
      if (lane < m)
        for (int k = 0; k < W; ++k) {
          const unsigned long long t = Fb[lane * W + k] | full_s[k];
          if (~t) {
            base = 64 * k + __ffsll(static_cast<long long>(~t)) - 1;
            break;
          }
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) base = min(base, __shfl_xor_sync(0xffffffffu, base, o));
      const int k0 = base >> 6, sh = base & 63;
      auto window = [&](const unsigned long long* v) {
        const unsigned long long lo = k0 < W ? v[k0] : 0ull, hi = k0 + 1 < W ? v[k0 + 1] : 0ull;
        return sh ? (lo >> sh) | (hi << (64 - sh)) : lo;
      };
      unsigned long long acc = lane < m ? window(Fb + lane * W) : 0ull;
      // colours from max_colours on count as full, so a free window colour is a valid one
      const int lim = A.max_colours - base;
      unsigned long long fullw =
          window(full_s) | (lim >= 64 ? 0ull : lim <= 0 ? ~0ull : ~0ull << lim);
      const int cap = A.class_cap > 0 ? A.class_cap : 0x7fffffff;
      const int cl = base + lane, ch = base + 32 + lane;  // this lane's two window classes
      int n_lo = cl < 64 * W ? csize[cl] : 0, n_hi = ch < 64 * W ? csize[ch] : 0;
      const unsigned my_conf = lane < m ? conf[fc][lane] : 0u;
      int mine = -1;
      bool fail = false;
      auto write_back = [&]() {
        col[cur][lane] = mine;
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
                const int q = col[cur][__ffs(b) - 1];
                if ((q >> 6) == k) t |= 1ull << (q & 63);
              }
              if (~t) cc = 64 * k + __ffsll(static_cast<long long>(~t)) - 1;
            }
          const int c = __shfl_sync(0xffffffffu, cc, i);
          if (c < 0 || c >= A.max_colours) {
            fail = true;
            break;
          }
          mine = lane == i ? c : mine;  // beyond the window: counted in shared memory
          if (lane == 0 && ++csize[c] >= cap) full_s[c >> 6] |= 1ull << (c & 63);
          __syncwarp();
          continue;
        }
        mine = lane == i ? base + rel : mine;
        acc |= ((my_conf >> i) & 1u) ? 1ull << rel : 0ull;
        n_lo += rel == lane;
        n_hi += rel == lane + 32;
        fullw |= (static_cast<unsigned long long>(__ballot_sync(0xffffffffu, n_hi >= cap)) << 32) |
                 __ballot_sync(0xffffffffu, n_lo >= cap);
      }
      write_back();
      if (lane < m && !fail) A.colour[s + lane] = static_cast<int16_t>(mine);
      int top = mine;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(0xffffffffu, top, o));
      ncol_w = max(ncol_w, top + 1);
      if (lane == 0 && fail) s_fail = 1;
    } else {
      // warps 1-31, one line j each: the footprints of block bk+1's line (its line read a step
      // ahead) requested first, block bk-1's colours into the planes meanwhile, then block
      // bk+1's colour sets
      const int j = warp - 1;
      const int uw = min(s_ncol / 64 + 1, W);  // words holding colours of blocks before bk
      const int l = l_ahead;
      const int32_t* pl = A.packed + static_cast<size_t>(l) * nt;
      int32_t f0 = 0, f1 = 0;
      unsigned cw = 0u, cw1 = 0u, cw2 = 0u;
      if (j < mn) {
        if (lane < nt) f0 = pl[lane];
        if (lane + 32 < nt) f1 = pl[lane + 32];
        cw = A.conf[s + kBlock + j];
        cw1 = A.conf_p1[s + kBlock + j];
        cw2 = A.conf_p2[s + kBlock + j];
      }
      l_ahead = s + 2 * kBlock + j < n ? A.vis[s + 2 * kBlock + j] : 0;
      if (j < mp) set_line(A, W, pk + (prv * kBlock + j) * nt, vline[prv][j], col[prv][j]);
      if (j < mn) {
        int32_t* pw = pk + (nxt * kBlock + j) * nt;
        if (lane < nt) pw[lane] = f0;
        if (lane + 32 < nt) pw[lane + 32] = f1;
        for (int v = lane + 64; v < nt; v += 32) pw[v] = pl[v];
        __syncwarp();
        load_planes(A, W, uw, l, pw, F + (fn * kBlock + j) * W);
        if (lane == 0) {
          vline[nxt][j] = l;
          conf[fn][j] = cw;
          cprev[0][j] = cw1;
          cprev[1][j] = cw2;
        }
      }
    }
    __threadfence_block();  // this step's plane updates land before the next step reads
    __syncthreads();
    if (s_fail) break;
    // the colours of blocks bk-1 and bk that the lines of block bk+1 conflict with
    if (warp < mn) {
      const unsigned c1 = cprev[0][warp], c2 = cprev[1][warp];
      unsigned long long* Fl = F + (fn * kBlock + warp) * W;
      if ((c1 >> lane) & 1u) {
        const int c = col[cur][lane];
        atomicOr(&Fl[c >> 6], 1ull << (c & 63));
      }
      if ((c2 >> lane) & 1u) {
        const int c = col[prv][lane];
        atomicOr(&Fl[c >> 6], 1ull << (c & 63));
      }
    }
    if (tid == 0) s_ncol = ncol_w;
    __syncthreads();
  }
  if (s_fail) {
    if (tid == 0) {
      A.count[0] = 0;
      A.count[1] = 0;
      atomicOr(A.err, 4);
    }
    return;
  }
  // phase 2: colour offsets, lines colour by colour, ascending within a colour
  const int ncol = s_ncol;
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
  static const int lim_k = dyn_smem_limit(colour_kernel);
  return sizeof(int32_t) * 3 * kBlock * n_theta <= static_cast<size_t>(lim_c) &&
         colour_smem_bytes(n_theta, words) <= static_cast<size_t>(lim_k);
}

int launch_colour_schedule(const ColourArgs& a, void* stream) {
  if ((a.words != 2 && a.words != 4 && a.words != 8) || a.max_colours > 64 * a.words ||
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
    const size_t csm = sizeof(int32_t) * 3 * kBlock * a.n_theta;
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
  static const int lim = dyn_smem_limit(colour_kernel);
  if (smem > static_cast<size_t>(lim)) return -7;
  cudaError_t e = cudaFuncSetAttribute(colour_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       lim);
  if (e != cudaSuccess) return -4000 - static_cast<int>(e);
  colour_kernel<<<1, kThreads, smem, s>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : -5000 - static_cast<int>(e);
}

}  // namespace mbir
