// k_list.cu — cell-grid sort, blocks, tile list, exclusion masks and the
// per-evaluation position pack.  Replaces NeighbourList::calcNewList
// (PD src/mmlib/workspace/neighbourlist.cpp:222-439): PD scans all j < i at
// minimum image; here atoms are binned on a 32^3 grid ordered along a Hilbert
// curve, grouped into 32-atom blocks, and block pairs whose bounding boxes come
// within max(cutoffs)+Padding form the tile list, found through a grid over the
// block centres (work and memory follow the tiles, not the square of the block
// count).  The bond order PD packs into
// each list entry (neighbourlist.cpp:398-422, 179-220) becomes a per-tile
// exclusion / 1-4 bit mask.
#include <cstdio>

#include "pdgpu_tile.cuh"

namespace pdgpu {

// ---------------------------------------------------------------------------
// 3-D Hilbert index of a cell (J. Skilling, "Programming the Hilbert curve",
// AIP Conf. Proc. 707, 2004: axes -> transposed form, then bit interleave).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int hilbert3(unsigned x0, unsigned x1, unsigned x2) {
  unsigned X[3] = {x0, x1, x2};
  const unsigned M = 1u << (kHilbertBits - 1);
  for (unsigned Q = M; Q > 1; Q >>= 1) {
    unsigned P = Q - 1;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        unsigned t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  X[2] ^= X[1];
  unsigned t = 0;
  for (unsigned Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  X[0] ^= t; X[1] ^= t; X[2] ^= t;
  int h = 0;
  for (int b = kHilbertBits - 1; b >= 0; b--) {
    h = (h << 3) | (((X[0] >> b) & 1) << 2) | (((X[1] >> b) & 1) << 1) | ((X[2] >> b) & 1);
  }
  return h;
}

// order-preserving float <-> int for atomic min / max
__device__ __forceinline__ int f2ord(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void k_bbox_init(int* lo, int* hi, int* hmax, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    lo[i] = f2ord(3.0e38f);
    hi[i] = f2ord(-3.0e38f);
    hmax[i] = f2ord(0.f);
  }
}

// bounding box of each open-space system (periodic systems key on the box);
// a warp whose atoms share one system reduces first and adds one atomic per
// coordinate (a whole system's atoms otherwise meet on the same six words)
__global__ void k_bbox(DevView v, const int* atom_sys, int* lo, int* hi) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int s = a < v.natom ? atom_sys[a] : -1;
  const bool use = s >= 0 && !v.sys[s].periodic;
  const unsigned act = __ballot_sync(0xffffffffu, use);
  if (!act) return;
  const int s0 = __shfl_sync(0xffffffffu, s, __ffs(act) - 1);
  const bool uniform = __all_sync(0xffffffffu, !use || s == s0);
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const int x = use ? f2ord((float)v.pos[3 * a + c]) : 0;
    if (uniform) {
      int mn = use ? x : f2ord(3.0e38f), mx = use ? x : f2ord(-3.0e38f);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      }
      if (lane == __ffs(act) - 1) {
        atomicMin(&lo[3 * s0 + c], mn);
        atomicMax(&hi[3 * s0 + c], mx);
      }
    } else if (use) {
      atomicMin(&lo[3 * s + c], x);
      atomicMax(&hi[3 * s + c], x);
    }
  }
}

__device__ __forceinline__ double wrap_coord(double x, double L, double iL) { return x - L * floor(x * iL); }

__global__ void k_keys(DevView v, const int* atom_sys, const int* lo, const int* hi, int* bucket, int* count) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= v.natom) return;
  int s = atom_sys[a];
  const SystemInfo& S = v.sys[s];
  unsigned q[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double x = v.pos[3 * a + c];
    double f;
    if (S.periodic) {
      f = wrap_coord(x, S.box[c], S.ibox[c]) * S.ibox[c];
    } else {
      double l = ord2f(lo[3 * s + c]), h = ord2f(hi[3 * s + c]);
      f = (x - l) / (h - l + 1e-3);
    }
    int qi = (int)(f * (1 << kHilbertBits));
    qi = qi < 0 ? 0 : (qi > (1 << kHilbertBits) - 1 ? (1 << kHilbertBits) - 1 : qi);
    q[c] = (unsigned)qi;
  }
  int b = s * kCellsPerSystem + hilbert3(q[0], q[1], q[2]);
  bucket[a] = b;
  atomicAdd(&count[b], 1);
}

// --- exclusive scans --------------------------------------------------------
__device__ __forceinline__ int warp_inclusive_scan(int x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// 1024 threads: the exclusive prefix of each thread's value within the CTA
// (warp scans, then a scan of the 32 warp totals); *total gets the CTA's sum
__device__ __forceinline__ int cta_exclusive_scan(int x, int* wsum, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_inclusive_scan(x, lane);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int t = wsum[lane];
    const int ti = warp_inclusive_scan(t, lane);
    wsum[lane] = ti - t;
    if (lane == 31) wsum[32] = ti;
  }
  __syncthreads();
  *total = wsum[32];
  return wsum[wid] + inc - x;
}

// three-phase scan, 1024 elements per CTA
__global__ void __launch_bounds__(1024) k_scan_block(const int* in, int* out, int* block_sums, int n) {
  __shared__ int wsum[33];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int x = i < n ? in[i] : 0;
  int total;
  const int e = cta_exclusive_scan(x, wsum, &total);
  if (i < n) out[i] = e;
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int* sums, int nb) {
  // single CTA: 1024-element chunks in order, carrying the running total
  __shared__ int wsum[33];
  int carry = 0;
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const int x = i < nb ? sums[i] : 0;
    int total;
    const int e = cta_exclusive_scan(x, wsum, &total);
    if (i < nb) sums[i] = e + carry;
    carry += total;
    __syncthreads();
  }
}

// one CTA for n <= kScanOne: 8 consecutive elements per thread
constexpr int kScanOne = 8192;
__global__ void __launch_bounds__(1024) k_scan_one(const int* in, int* out, int n) {
  __shared__ int wsum[33];
  const int base = threadIdx.x * 8;
  int x[8], s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    x[k] = base + k < n ? in[base + k] : 0;
    s += x[k];
  }
  int total;
  int run = cta_exclusive_scan(s, wsum, &total);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (base + k < n) out[base + k] = run;
    run += x[k];
  }
}

__global__ void k_scan_add(int* out, const int* sums, int n) {
  int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

__global__ void k_scatter(int natom, const int* bucket, const int* offset, int* cursor, int* tmp) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= natom) return;
  int b = bucket[a];
  tmp[offset[b] + atomicAdd(&cursor[b], 1)] = a;
}

// insertion sort inside each non-empty cell so the order is deterministic
__global__ void k_cell_sort(int ncells, const int* offset, const int* count, int* tmp) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= ncells) return;
  int n = count[b];
  if (n < 2) return;
  int* p = tmp + offset[b];
  for (int i = 1; i < n; i++) {
    int x = p[i];
    int j = i - 1;
    while (j >= 0 && p[j] > x) {
      p[j + 1] = p[j];
      j--;
    }
    p[j + 1] = x;
  }
}

__global__ void k_to_slots(DevView v, const int* atom_sys, const int* tmp, int* sorted_atom, int* slot_of) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.natom) return;
  int a = tmp[k];
  int s = atom_sys[a];
  const SystemInfo& S = v.sys[s];
  int slot = S.pad_start + (k - S.atom_start);
  sorted_atom[slot] = a;
  slot_of[a] = slot;
}

// block bounding boxes, and each system's largest half-extent; one warp per block
__global__ void k_blocks(DevView v, int* hmax) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= v.nblocks) return;
  int slot = warp * 32 + lane;
  int a = v.sorted_atom[slot];
  const SystemInfo& S = v.sys[v.slot_sys[warp]];
  double lo[3], hi[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double x = 0;
    if (a >= 0) {
      x = v.pos[3 * a + c];
      if (S.periodic) x = wrap_coord(x, S.box[c], S.ibox[c]);
    }
    lo[c] = a >= 0 ? x : 1e300;
    hi[c] = a >= 0 ? x : -1e300;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  }
  if (lane == 0) {
    float4 h;
    for (int c = 0; c < 3; c++) v.center[3 * warp + c] = 0.5 * (lo[c] + hi[c]);
    h.x = (float)(0.5 * (hi[0] - lo[0])) + 1e-4f;
    h.y = (float)(0.5 * (hi[1] - lo[1])) + 1e-4f;
    h.z = (float)(0.5 * (hi[2] - lo[2])) + 1e-4f;
    h.w = 0.f;
    v.half[warp] = h;
    const int s3 = 3 * v.slot_sys[warp];
    atomicMax(&hmax[s3], f2ord(h.x));
    atomicMax(&hmax[s3 + 1], f2ord(h.y));
    atomicMax(&hmax[s3 + 2], f2ord(h.z));
  }
}

// static per-slot parameters (LJ radius, sqrt eps, GB radius, Vj)
__global__ void k_slot_params(DevView v, const double* radius, const double* sqeps, const double* gbR,
                              const double* gbVj, const double* lcR, const int* lcUse, float4* lc_par) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 l = make_float4(0.f, 0.f, 0.f, 0.f);
  if (a >= 0) {
    p.x = (float)radius[a];
    p.y = (float)sqeps[a];
    if (gbR) {
      p.z = (float)gbR[a];
      p.w = (float)gbVj[a];
    }
    if (lcR) {
      l.x = (float)lcR[a];
      l.y = lcUse[a] ? 1.f : 0.f;
    }
  }
  v.par[s] = p;
  if (lc_par) lc_par[s] = l;
}

// ---------------------------------------------------------------------------
// Tile list.  Block pair (bi, bj), bi <= bj of one system, is a tile when the
// two blocks' bounding boxes come within R (periodic: at the minimum image of
// their centres).  Each build bins every system's block centres on a grid of
// at most one cell per block; row bi visits only the cells within
// R + h_i + hmax of its centre along each axis (h: half-extents, hmax the
// system's largest), marks its hits in a per-warp bitmap over its columns
// bj >= bi, takes its place in the list with one atomic on the tile total and
// writes its tiles there in ascending bj.  Rows land in any order, each
// contiguous with ascending columns (what the binary searches, the GB tile
// pairs and the NB groups rely on); every sum over tiles is in fixed point,
// so the results do not depend on the rows' order.  A row whose cell range
// spans the whole grid (all pairs within reach) walks its columns directly.
// ---------------------------------------------------------------------------
// box test of one block pair; flags as Tile::flags.  FP32 geometry (the FP64
// pipe is narrow on this GPU), every decision taken 1e-3 A on the safe side:
// include, per-pair image, not all-inside
__device__ __forceinline__ bool tile_test(const DevView& v, const SystemInfo& S, int gi, int gj, float R,
                                          float margin, float full_R, float full_margin, int& flags) {
  const float4 hi4 = v.half[gi], hj4 = v.half[gj];
  const float hs[3] = {hi4.x + hj4.x, hi4.y + hj4.y, hi4.z + hj4.z};
  constexpr float kSafe = 1e-3f;
  float dist2 = 0.f, dmax2 = 0.f;
  bool need_mi = false;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float d = (float)(v.center[3 * gj + c] - v.center[3 * gi + c]);
    if (S.periodic) {
      const float L = (float)S.box[c];
      d -= L * rintf(d * (float)S.ibox[c]);
      // a pair of the two blocks inside the cutoff in some other image would
      // sit at least L - R apart along this axis in the tile's image: below
      // that every pair inside the cutoff takes the tile's image, and pairs
      // whose images differ lie beyond the cutoff in both
      if (fabsf(d) + hs[c] + margin >= L - R - kSafe) need_mi = true;
    }
    const float g = fabsf(d) - hs[c];
    if (g > 0.f) dist2 += g * g;
    const float m = fabsf(d) + hs[c];
    dmax2 += m * m;
  }
  // full: the farthest pair of the two boxes, grown by the displacement margin,
  // stays inside every cutoff and switch radius
  const bool full = full_R > 0.f && !need_mi && sqrtf(dmax2) + full_margin + kSafe < full_R;
  flags = (need_mi ? 1 : 0) | (gi == gj ? 2 : 0) | (full ? 4 : 0);
  const float Rs = R + kSafe;
  return dist2 <= Rs * Rs;
}

// the tile record at position t (centre offset formed in FP64, rounded once)
__device__ __forceinline__ void write_tile(const DevView& v, const SystemInfo& S, int gi, int gj, int flags,
                                           long long t, long long cap) {
  if (t >= cap) return;
  Tile T;
  T.bi = gi;
  T.bj = gj;
  T.mask = -1;
  T.flags = flags;
  double o[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    o[c] = v.center[3 * gj + c] - v.center[3 * gi + c];
    if (S.periodic) o[c] -= S.box[c] * rint(o[c] * S.ibox[c]);
  }
  T.ox = (float)o[0];
  T.oy = (float)o[1];
  T.oz = (float)o[2];
  T.pad = 0.f;
  v.tiles[t] = T;
}

// one thread per system: the grid of its block centres for this build
__global__ void k_grid_setup(DevView v, const int* lo, const int* hi, const int* hmax, BlockGrid* grid) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nsys) return;
  const SystemInfo& S = v.sys[s];
  BlockGrid G;
  double ext[3];
  for (int c = 0; c < 3; c++) {
    if (S.periodic) {
      G.origin[c] = 0.0;
      ext[c] = S.box[c];
    } else {
      const double l = ord2f(lo[3 * s + c]), h = ord2f(hi[3 * s + c]);
      G.origin[c] = l;
      ext[c] = fmax(h - l, 1e-3);
    }
    G.hmax[c] = ord2f(hmax[3 * s + c]);
  }
  // cells of about equal edge, at most grid_cells of them
  const double edge = cbrt(ext[0] * ext[1] * ext[2] / (double)S.grid_cells);
  for (int c = 0; c < 3; c++) G.dims[c] = (int)fmax(1.0, fmin(floor(ext[c] / edge), 4096.0));
  while ((long long)G.dims[0] * G.dims[1] * G.dims[2] > S.grid_cells) {
    const int m = G.dims[0] >= G.dims[1] ? (G.dims[0] >= G.dims[2] ? 0 : 2) : (G.dims[1] >= G.dims[2] ? 1 : 2);
    G.dims[m]--;
  }
  for (int c = 0; c < 3; c++) G.cell[c] = ext[c] / G.dims[c];
  G.start = S.grid_start;
  G.pad = 0.f;
  grid[s] = G;
}

// cell coordinate of x along axis c (clamped into the grid)
__device__ __forceinline__ int grid_axis(const BlockGrid& G, int c, double x) {
  const double q = floor((x - G.origin[c]) / G.cell[c]);
  return (int)fmin(fmax(q, 0.0), (double)(G.dims[c] - 1));
}

__global__ void k_bgrid_count(DevView v, const BlockGrid* grid, int* bcell, int* count) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= v.nblocks) return;
  const BlockGrid& G = grid[v.slot_sys[b]];
  const double* x = v.center + 3 * b;
  const int cell = G.start + (grid_axis(G, 2, x[2]) * G.dims[1] + grid_axis(G, 1, x[1])) * G.dims[0] +
                   grid_axis(G, 0, x[0]);
  bcell[b] = cell;
  atomicAdd(&count[cell], 1);
}

// blocks in cell order (the order inside a cell does not matter: rows collect
// their hits in a bitmap)
__global__ void k_bgrid_scatter(int nblocks, const int* bcell, const int* offset, int* cursor, int* blocks) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  const int cell = bcell[b];
  blocks[offset[cell] + atomicAdd(&cursor[cell], 1)] = b;
}

// position of the n-th (from 0) set bit of m (m holds more than n set bits)
__device__ __forceinline__ int nth_set_bit(unsigned m, int n) {
  int pos = 0;
#pragma unroll
  for (int b = 16; b > 0; b >>= 1) {
    const int c = __popc(m & ((1u << b) - 1u));
    if (n >= c) {
      n -= c;
      m >>= b;
      pos += b;
    }
  }
  return pos;
}

// the tiles that get an exclusion mask whatever their pairs hold (diagonal, and
// those with a system's padded last block) and the ones k_mask_mark finds with
// a bonded pair: each tile once (need: one bit per tile), in the mask list
__device__ __forceinline__ void mask_list_add(unsigned* need, int* mlist, int* nml, int mask_cap, int t) {
  const unsigned bit = 1u << (t & 31);
  // (a plain read first: most marks repeat a tile already in the list)
  if ((need[t >> 5] & bit) || (atomicOr(&need[t >> 5], bit) & bit)) return;
  const int k = atomicAdd(nml, 1);
  if (k < mask_cap) mlist[k] = t;
}

// one warp per row bi, 4 warps per CTA, `words` bitmap words per warp in
// dynamic shared memory: the row's tiles are found (hits marked in the bitmap),
// counted, given a place in the list by an atomic on the tile total (rows land
// in any order, each contiguous with ascending columns) and written there;
// positions past `cap` are dropped (k_tile_total flags the overflow)
__global__ void __launch_bounds__(128) k_tile_rows(DevView v, const BlockGrid* grid, const int* cell_off,
                                                   const int* cell_count, const int* cell_blocks, float R,
                                                   float margin, float full_R, float full_margin, int* row_cnt,
                                                   int* row_start, long long cap, int words, int* total,
                                                   unsigned* need, int* mlist, int* nml) {
  extern __shared__ unsigned s_bits[];
  const int lane = threadIdx.x & 31;
  const int bi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (bi >= v.nblocks) return;
  unsigned* bits = s_bits + (threadIdx.x >> 5) * words;
  const SystemInfo& S = v.sys[v.slot_sys[bi]];
  const BlockGrid& G = grid[v.slot_sys[bi]];
  const int end = S.block_start + S.nblocks;
  const float4 h4 = v.half[bi];
  const float h[3] = {h4.x, h4.y, h4.z};
  int lo[3], hi[3];
  bool all = true;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double x = v.center[3 * bi + c] - G.origin[c];
    // reach along the axis: list radius, both half-extents, and a slack far
    // above the rounding of the centres and cell edges
    const double r = (double)R + (double)h[c] + (double)G.hmax[c] + 0.01;
    const int D = G.dims[c];
    int a = (int)fmax(floor((x - r) / G.cell[c]), -1.0e9);
    int b = (int)fmin(floor((x + r) / G.cell[c]), 1.0e9);
    if (S.periodic) {
      if (b - a + 1 >= D) {
        a = 0;
        b = D - 1;
      } else {
        all = false;
      }
    } else {
      a = max(a, 0);
      b = min(b, D - 1);
      if (a > 0 || b < D - 1) all = false;
    }
    lo[c] = a;
    hi[c] = b;
  }
  const unsigned lt = (1u << lane) - 1u;
  long long n = 0;   // tiles of the row
  long long base = 0;
  if (all) {
    // count, take the row's place, then write (the test is cheap: no cell walk)
#pragma unroll 2
    for (int j0 = bi; j0 < end; j0 += 32) {
      const int bj = j0 + lane;
      int fl = 0;
      n += __popc(__ballot_sync(0xffffffffu, bj < end && tile_test(v, S, bi, bj, R, margin, 0.f, 0.f, fl)));
    }
    if (lane == 0) base = atomicAdd(total, (int)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    long long w = 0;
#pragma unroll 2
    for (int j0 = bi; j0 < end; j0 += 32) {
      const int bj = j0 + lane;
      int fl = 0;
      const bool hit = bj < end && tile_test(v, S, bi, bj, R, margin, full_R, full_margin, fl);
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (hit) write_tile(v, S, bi, bj, fl, base + w + __popc(m & lt), cap);
      w += __popc(m);
    }
  } else {
    const int nw = (end - bi + 31) >> 5;
    for (int w = lane; w < nw; w += 32) bits[w] = 0u;
    __syncwarp();
    // the cell runs to visit: one per (y, z) cell row of the range, two where
    // a periodic x range wraps.  Each lane reads one run's block range, then
    // the warp deals the runs' blocks over its lanes (the reads of a row are
    // independent of one another, not a chain of dependent loads)
    const int Dx = G.dims[0], Dy = G.dims[1], Dz = G.dims[2];
    const int nyr = hi[1] - lo[1] + 1, nzr = hi[2] - lo[2] + 1;
    const bool wrapx = lo[0] < 0 || hi[0] >= Dx;
    const int nxr = wrapx ? 2 : 1;
    const int nrun = nyr * nzr * nxr;
    for (int q0 = 0; q0 < nrun; q0 += 32) {
      const int q = q0 + lane;
      int p0 = 0, len = 0;
      if (q < nrun) {
        const int xr = q % nxr, yz = q / nxr;
        const int cy = ((lo[1] + yz % nyr) % Dy + Dy) % Dy, cz = ((lo[2] + yz / nyr) % Dz + Dz) % Dz;
        const int row0 = G.start + (cz * Dy + cy) * Dx;
        int c0 = lo[0], c1 = hi[0];
        if (lo[0] < 0) {
          c0 = xr ? 0 : lo[0] + Dx;
          c1 = xr ? hi[0] : Dx - 1;
        } else if (hi[0] >= Dx) {
          c0 = xr ? 0 : lo[0];
          c1 = xr ? hi[0] - Dx : Dx - 1;
        }
        p0 = cell_off[row0 + c0];
        len = cell_off[row0 + c1] + cell_count[row0 + c1] - p0;
      }
      int inc = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
      }
      const int cnt = __shfl_sync(0xffffffffu, inc, 31);
      const int excl = inc - len;
      for (int t0 = 0; t0 < cnt; t0 += 32) {
        const int t = t0 + lane;
        // the run holding entry t: the last lane whose runs start at or before t
        int L = 0;
#pragma unroll
        for (int b = 16; b > 0; b >>= 1)
          if (__shfl_sync(0xffffffffu, excl, L + b) <= t) L += b;
        const int p = __shfl_sync(0xffffffffu, p0, L) + t - __shfl_sync(0xffffffffu, excl, L);
        if (t < cnt) {
          const int bj = cell_blocks[p];
          int fl;
          if (bj >= bi && tile_test(v, S, bi, bj, R, margin, 0.f, 0.f, fl))
            atomicOr(&bits[(bj - bi) >> 5], 1u << ((bj - bi) & 31));
        }
      }
    }
    __syncwarp();
    int k = 0;
    for (int w = lane; w < nw; w += 32) k += __popc(bits[w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    n = k;
    if (lane == 0) base = atomicAdd(total, (int)n);
    base = __shfl_sync(0xffffffffu, base, 0);
    long long done = 0;
    for (int w0 = 0; w0 < nw; w0 += 32) {
      const int w = w0 + lane;
      const unsigned word = w < nw ? bits[w] : 0u;
      const int kw = __popc(word);
      int inc = kw;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
      }
      const int tot = __shfl_sync(0xffffffffu, inc, 31);
      // the hits of these 32 words dealt over the lanes, in column order
      const int excl = inc - kw;
      for (int t0 = 0; t0 < tot; t0 += 32) {
        const int t = t0 + lane;
        int L = 0;
#pragma unroll
        for (int b = 16; b > 0; b >>= 1)
          if (__shfl_sync(0xffffffffu, excl, L + b) <= t) L += b;
        const unsigned wl = __shfl_sync(0xffffffffu, word, L);
        const int nth = t - __shfl_sync(0xffffffffu, excl, L);
        if (t < tot) {
          const int bj = bi + 32 * (w0 + L) + nth_set_bit(wl, nth);
          int fl = 0;
          tile_test(v, S, bi, bj, R, margin, full_R, full_margin, fl);
          write_tile(v, S, bi, bj, fl, base + done + t, cap);
        }
      }
      done += tot;
    }
  }
  if (lane == 0) {
    row_start[bi] = (int)base;
    row_cnt[bi] = (int)n;
    // the diagonal tile is the row's first; a tile with the system's padded
    // last block, its last
    if (base < cap) mask_list_add(need, mlist, nml, v.mask_cap, (int)base);
    const int last = end - 1;
    int fl;
    if (S.natom != S.npad && bi != last && n > 1 && base + n - 1 < cap &&
        tile_test(v, S, bi, last, R, margin, 0.f, 0.f, fl))
      mask_list_add(need, mlist, nml, v.mask_cap, (int)(base + n - 1));
  }
}

// the tile count from the rows' total, clamped to the capacity (an overflow
// leaves a short list and is flagged)
__global__ void k_tile_total(DevView v, const int* total, long long cap) {
  const long long t = *total;
  *v.ntiles = (int)(t < cap ? t : cap);
  if (t > cap) atomicOr(v.status, (unsigned)ST_TILE_OVERFLOW);
}

// index of tile (bi, bj) in the list (rows contiguous, ascending columns), -1 if absent
__device__ __forceinline__ int tile_index(const DevView& v, const int* row_start, const int* row_cnt, int bi, int bj) {
  const int nt = *v.ntiles;
  int lo = row_start[bi], hi = min(lo + row_cnt[bi], nt) - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int c = v.tiles[mid].bj;
    if (c == bj) return mid;
    if (c < bj) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

// exclusion masks in rotation order (bit k <-> j slot (lane+k)&31); one warp per tile
// tiles holding a bonded pair (bond order <= 3: excluded or 1-4), found from
// each atom's partners (band words, far list) and added to the mask list
__global__ void k_mask_mark(DevView v, const int* slot_of, const int* row_start, const int* row_cnt,
                            unsigned* need, int* mlist, int* nml) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= v.natom) return;
  const unsigned long long w = v.band_excl[a] | v.band_14[a];
  const int fs = v.far_start[a], fe = v.far_start[a + 1];
  if (!w && fs == fe) return;
  const int ga = slot_of[a] >> 5;
  int last = ga;
  auto mark = [&](int b) {
    const int gb = slot_of[b] >> 5;
    // (diagonal tiles are in the list already; partners of one block come in runs)
    if (gb == last || gb == ga) return;
    last = gb;
    const int t = tile_index(v, row_start, row_cnt, ga < gb ? ga : gb, ga < gb ? gb : ga);
    if (t >= 0) mask_list_add(need, mlist, nml, v.mask_cap, t);
  };
  for (unsigned long long m = w; m; m &= m - 1) mark(a + __ffsll((long long)m));
  for (int q = fs; q < fe; q++)
    if (v.far_bo[q] <= 3) mark(v.far_idx[q]);
}

// one warp per tile of the mask list (grid-stride): the tile's exclusion and
// 1-4 bits, a mask table entry when any is set
__global__ void k_masks(DevView v, const int* mlist, const int* nml) {
  const int lane = threadIdx.x & 31;
  const int n = min(*nml, v.mask_cap);
  if (*nml > v.mask_cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(v.status, (unsigned)ST_TILE_OVERFLOW);
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n; e += nwarps) {
    const int warp = mlist[e];
    Tile T = v.tiles[warp];
    int ai = v.sorted_atom[T.bi * 32 + lane];
    int aj0 = v.sorted_atom[T.bj * 32 + lane];
    // each atom's band words and far-partner range, loaded once per lane (the
    // lower index of a pair holds them, as in pair_bondorder); j's are shuffled in
    unsigned long long exi = 0ull, b14i = 0ull, exj0 = 0ull, b14j0 = 0ull;
    int fsi = 0, fei = 0, fsj0 = 0, fej0 = 0;
    if (ai >= 0) {
      exi = v.band_excl[ai];
      b14i = v.band_14[ai];
      fsi = v.far_start[ai];
      fei = v.far_start[ai + 1];
    }
    if (aj0 >= 0) {
      exj0 = v.band_excl[aj0];
      b14j0 = v.band_14[aj0];
      fsj0 = v.far_start[aj0];
      fej0 = v.far_start[aj0 + 1];
    }
    unsigned ex = 0, m14 = 0;
    for (int k = 0; k < 32; k++) {
      const int src = (lane + k) & 31;
      const int aj = __shfl_sync(0xffffffffu, aj0, src);
      const unsigned long long exj = __shfl_sync(0xffffffffu, exj0, src);
      const unsigned long long b14j = __shfl_sync(0xffffffffu, b14j0, src);
      const int fsj = __shfl_sync(0xffffffffu, fsj0, src);
      const int fej = __shfl_sync(0xffffffffu, fej0, src);
      if (ai < 0 || aj < 0 || ai == aj) {
        ex |= 1u << k;
        continue;
      }
      const bool lo_i = ai < aj;
      const int hi = lo_i ? aj : ai;
      const int d = lo_i ? aj - ai : ai - aj;
      int bo = 7;
      if (d <= kBandWidth) {
        const unsigned long long bit = 1ull << (d - 1);
        if ((lo_i ? exi : exj) & bit) bo = 2;
        else if ((lo_i ? b14i : b14j) & bit) bo = 3;
      } else {
        for (int q = lo_i ? fsi : fsj, e = lo_i ? fei : fej; q < e; q++)
          if (v.far_idx[q] == hi && v.far_bo[q] < bo) bo = v.far_bo[q];
      }
      if (bo <= 2) ex |= 1u << k;
      else if (bo == 3) m14 |= 1u << k;
    }
    bool any = __any_sync(0xffffffffu, (ex | m14) != 0);
    if (!any) continue;
    int idx = 0;
    if (lane == 0) idx = atomicAdd(v.nmasks, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= v.mask_cap) {
      // (the capacity bounds the diagonal, padded and bonded tiles: not reached)
      if (lane == 0) atomicOr(v.status, (unsigned)ST_TILE_OVERFLOW);
      continue;
    }
    v.masks[idx * 32 + lane] = make_uint2(ex, m14);
    if (lane == 0) v.tiles[warp].mask = idx;
  }
}

// per-evaluation pack: FP64 positions -> float offsets from the block centre
// check2: squared skin limit (0 = no skin check); full2: squared limit that keeps
// tiles flagged full valid (0 = none flagged), checked where the skin check is not
// cull: the NB j-atom groups are in use (the displacement check always runs)
__global__ void k_pack(DevView v, const double* charge, float check2, float full2, int store_ref,
                       long long npairs_all, int cull) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  int b = s >> 5;
  float4 o;
  if (a < 0) {
    // padding slot: zero parameters, parked far away from everything and each other
    o = make_float4(1.0e6f * (float)(1 + (s & 31)), 1.0e6f * (float)(1 + (s >> 5)), -1.0e6f, 0.f);
  } else {
    const SystemInfo& S = v.sys[v.slot_sys[b]];
    double r[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double d = v.pos[3 * a + c] - v.center[3 * b + c];
      if (S.periodic) d -= S.box[c] * rint(d * S.ibox[c]);
      r[c] = d;
    }
    o = make_float4((float)r[0], (float)r[1], (float)r[2], (float)charge[a]);
    if (store_ref) {
      v.rel0[s] = o;
    } else {
      // (in open space, when every block pair of every system is a tile, no pair
      // can leave the list; in a periodic box the tile images still depend on it)
      const bool skin = check2 > 0.f && (S.periodic || (long long)*v.ntiles < npairs_all || cull);
      const float lim = skin ? check2 : full2;
      if (lim > 0.f) {
        float4 q = v.rel0[s];
        float dx = o.x - q.x, dy = o.y - q.y, dz = o.z - q.z;
        if (dx * dx + dy * dy + dz * dz > lim) atomicOr(v.status, (unsigned)ST_STALE_LIST);
      }
    }
  }
  v.xq[s] = o;
}

// GB work items: tiles t and t + 1 go together when they share the row, sit in
// adjacent columns with bj - bi odd for the first (a fixed pairing that does not
// depend on the other systems of a batch), are both unmasked and off-diagonal,
// need no per-pair image and agree on the all-inside flag
__device__ __forceinline__ bool tile_pairable(const DevView& v, int t, int nt) {
  if (t < 0 || t + 1 >= nt) return false;
  const Tile A = v.tiles[t], B = v.tiles[t + 1];
  return A.bi == B.bi && B.bj == A.bj + 1 && ((A.bj - A.bi) & 1) && !tile_masked(A) && !tile_masked(B) &&
         tile_full(A) == tile_full(B) && !((A.flags | B.flags) & 1);
}

// pairs: 0 makes every item a single tile
__global__ void k_item_flags(DevView v, long long cap, int pairs, int* flag) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cap) return;
  const int nt = *v.ntiles;
  flag[t] = (t < nt && !(pairs && tile_pairable(v, (int)t - 1, nt))) ? 1 : 0;
}

__global__ void k_item_write(DevView v, long long cap, int pairs, const int* flag, const int* pos) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cap) return;
  if (t == cap - 1) *v.nitems = pos[t] + flag[t];
  if (!flag[t]) return;
  v.items[pos[t]] = (unsigned)t | ((pairs && tile_pairable(v, (int)t, *v.ntiles)) ? 0x80000000u : 0u);
}

// ---------------------------------------------------------------------------
// NB j-atom groups.  A 32x32 tile at list radius R holds ~12 % pairs inside a
// 12 A cutoff (dense solvent, 7.5 A blocks); most of its j atoms lie beyond R
// of the whole i block.  Per i-block row, the j atoms of the row's plain tiles
// (no exclusion mask, off-diagonal, one periodic image) that lie within R of the
// i block's box are packed into groups of 32; the pair kernel rotates a group
// like a tile's j block.  Valid while every atom stays within half the skin of
// its build position (the per-step displacement check, forced on with groups):
// a pair inside the cutoff then had its j atom within R of the i box at build.
// row: [0, nb) kept j atoms, [nb, 2nb) first tile, [2nb, 3nb) groups,
// [3nb, 4nb) first group (exclusive scan).
// ---------------------------------------------------------------------------
// cnt: zeroed beforehand over the tile capacity (the scan runs over it)
__global__ void k_cull_mask(DevView v, float R2, unsigned* jmask, int* cnt, int* row) {
  const int lane = threadIdx.x & 31;
  const int nt = *v.ntiles;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const bool plain = T.mask < 0 && !(T.flags & 3);
    unsigned m = 0u;
    if (plain) {
      const int sj = T.bj * 32 + lane;
      const float4 x = v.xq[sj];
      const float4 h = v.half[T.bi];
      const float gx = fmaxf(fabsf(x.x + T.ox) - h.x, 0.f);
      const float gy = fmaxf(fabsf(x.y + T.oy) - h.y, 0.f);
      const float gz = fmaxf(fabsf(x.z + T.oz) - h.z, 0.f);
      m = __ballot_sync(0xffffffffu, v.sorted_atom[sj] >= 0 && gx * gx + gy * gy + gz * gz <= R2);
    }
    if (lane == 0) {
      jmask[t] = m;
      cnt[t] = __popc(m);
      const int nb = v.nblocks;
      if (m) atomicAdd(&row[T.bi], __popc(m));
      atomicMin(&row[nb + T.bi], t);
      if (!plain) v.cull_rest[atomicAdd(&v.cull_n[0], 1)] = t;
    }
  }
}

__global__ void k_cull_groups(int nb, int* row) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) row[2 * nb + b] = (row[b] + 31) >> 5;
}

// pos: exclusive scan of the kept counts over the tile list (a row's tiles are
// contiguous, so its entries keep tile order, then lane order)
__global__ void k_cull_write(DevView v, const unsigned* jmask, const int* pos, const int* row) {
  const int lane = threadIdx.x & 31;
  const int nt = *v.ntiles;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nb = v.nblocks;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const unsigned m = jmask[t];
    if (!((m >> lane) & 1u)) continue;
    const Tile T = v.tiles[t];
    const long long e = (long long)row[3 * nb + T.bi] * 32 + (pos[t] - pos[row[nb + T.bi]]) +
                        __popc(m & ((1u << lane) - 1u));
    if (e < v.cull_cap) v.cull_ent[e] = make_float4(T.ox, T.oy, T.oz, __int_as_float(T.bj * 32 + lane));
  }
}

// one warp per row: group -> row, empty entries closing the row's last group,
// and (last row) the group count and whether it fits the capacity
__global__ void k_cull_rows(DevView v, const int* row) {
  const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nb = v.nblocks;
  if (b >= nb) return;
  const int n = row[b], G = row[2 * nb + b], base = row[3 * nb + b];
  const long long gcap = v.cull_cap / 32;
  for (int g = lane; g < G; g += 32)
    if (base + g < gcap) v.cull_bi[base + g] = b;
  for (int i = n + lane; i < G * 32; i += 32) {
    const long long e = (long long)base * 32 + i;
    if (e < v.cull_cap) v.cull_ent[e] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
  }
  if (b == nb - 1 && lane == 0) {
    v.cull_n[1] = base + G;
    v.cull_n[2] = (long long)(base + G) * 32 <= v.cull_cap ? 1 : 0;
  }
}

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// grid of the warp-per-tile list kernels (grid-stride; 16 CTAs of 8 warps per SM)
static int list_tile_grid(const Context& c) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
  const long long want = (c.tile_cap + 7) / 8, g = 16LL * (sms > 0 ? sms : 1);
  return (int)(want < g ? (want > 0 ? want : 1) : g);
}

// exclusive scan of n ints (n <= 2^20): one CTA up to kScanOne, else three phases
static void scan_ints(Context& c, const int* in, int* out, int* tmp, long long n, cudaStream_t st) {
  c.kernel_launches += n <= kScanOne ? 1 : 3;
  if (n <= kScanOne) {
    k_scan_one<<<1, 1024, 0, st>>>(in, out, (int)n);
    return;
  }
  const int nb = nblk(n, 1024);
  k_scan_block<<<nb, 1024, 0, st>>>(in, out, tmp, (int)n);
  k_scan_sums<<<1, 1024, 0, st>>>(tmp, nb);
  k_scan_add<<<nb, 1024, 0, st>>>(out, tmp, (int)n);
}

static void launch_cull(Context& c, float list_radius) {
  c.kernel_launches += 4;   // and two scans
  DevView v = c.view();
  cudaStream_t st = c.stream;
  const int nb = c.nblocks;
  int* row = c.d_cull_row.p;
  cudaMemsetAsync(row, 0, sizeof(int) * nb, st);
  cudaMemsetAsync(row + nb, 0x7f, sizeof(int) * nb, st);
  const float R = list_radius + 1e-3f;
  // the kept counts and their scan reuse the tile-compaction arrays
  cudaMemsetAsync(c.d_tile_flag.p, 0, sizeof(int) * c.tile_cap, st);
  k_cull_mask<<<list_tile_grid(c), 256, 0, st>>>(v, R * R, c.d_cull_mask.p, c.d_tile_flag.p, row);
  scan_ints(c, c.d_tile_flag.p, c.d_tile_pos.p, c.d_scan_tmp2.p, c.tile_cap, st);
  k_cull_groups<<<nblk(nb, 256), 256, 0, st>>>(nb, row);
  scan_ints(c, row + 2 * nb, row + 3 * nb, c.d_cull_scan_tmp.p, nb, st);
  k_cull_write<<<list_tile_grid(c), 256, 0, st>>>(v, c.d_cull_mask.p, c.d_tile_pos.p, row);
  k_cull_rows<<<nblk((long long)nb * 32, 256), 256, 0, st>>>(v, row);
}

// rows of the tile-list build: 4 warps per CTA, a bitmap over each warp's row
// (the row total, the mask list and the need bits zeroed beforehand)
static void launch_rows(Context& c, float R, float full_radius) {
  const int words = (c.max_sys_blocks + 31) / 32 + 1;
  const size_t smem = (size_t)4 * words * sizeof(unsigned);
  DevView v = c.view();
  const int g = nblk((long long)c.nblocks * 32, 128);
  int* cnt = c.d_counters.p;
  cudaMemsetAsync(cnt + 6, 0, 2 * sizeof(int), c.stream);
  cudaMemsetAsync(c.d_tile_need.p, 0, sizeof(unsigned) * c.d_tile_need.n, c.stream);
  k_tile_rows<<<g, 128, smem, c.stream>>>(v, c.d_bgrid.p, c.d_bcell_off.p, c.d_bcell_count.p, c.d_bcell_blocks.p, R,
                                          (float)c.lp.Padding, full_radius, c.full_margin(), c.d_row_cnt.p,
                                          c.d_row_start.p, c.tile_cap, words, cnt + 6, c.d_tile_need.p,
                                          c.d_mlist.p, cnt + 7);
}

int launch_list_build(Context& c, float list_radius, float full_radius, ListSizing sizing) {
  c.kernel_launches += 16;   // and two scans
  DevView v = c.view();
  cudaStream_t st = c.stream;
  int ncells = c.nsys * kCellsPerSystem;
  int* lo = reinterpret_cast<int*>(c.d_sys_lo.p);
  int* hi = reinterpret_cast<int*>(c.d_sys_hi.p);
  int* hmax = reinterpret_cast<int*>(c.d_sys_hmax.p);
  k_bbox_init<<<nblk(3 * c.nsys, 128), 128, 0, st>>>(lo, hi, hmax, 3 * c.nsys);
  k_bbox<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_atom_sys.p, lo, hi);
  cudaMemsetAsync(c.d_count.p, 0, sizeof(int) * ncells, st);
  cudaMemsetAsync(c.d_cursor.p, 0, sizeof(int) * ncells, st);
  k_keys<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_atom_sys.p, lo, hi, c.d_bucket.p, c.d_count.p);
  scan_ints(c, c.d_count.p, c.d_offset.p, c.d_scan_tmp.p, ncells, st);
  k_scatter<<<nblk(c.natom, 256), 256, 0, st>>>(c.natom, c.d_bucket.p, c.d_offset.p, c.d_cursor.p,
                                                 c.d_tmp_sorted.p);
  k_cell_sort<<<nblk(ncells, 256), 256, 0, st>>>(ncells, c.d_offset.p, c.d_count.p, c.d_tmp_sorted.p);
  cudaMemsetAsync(c.d_sorted_atom.p, 0xff, sizeof(int) * c.nslots, st);
  k_to_slots<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_atom_sys.p, c.d_tmp_sorted.p, c.d_sorted_atom.p,
                                                  c.d_slot_of.p);
  k_blocks<<<nblk((long long)c.nblocks * 32, 256), 256, 0, st>>>(v, hmax);
  k_slot_params<<<nblk(c.nslots, 256), 256, 0, st>>>(v, c.d_radius.p, c.d_sqeps.p, c.has_gb ? c.d_gbR.p : nullptr,
                                                      c.has_gb ? c.d_gbVj.p : nullptr,
                                                      c.has_sa ? c.d_lcpoR.p : nullptr,
                                                      c.has_sa ? c.d_lcpoUse.p : nullptr,
                                                      c.has_sa ? c.d_lc_par.p : nullptr);
  // block grid and the row counts of the tile list
  k_grid_setup<<<nblk(c.nsys, 64), 64, 0, st>>>(v, lo, hi, hmax, c.d_bgrid.p);
  cudaMemsetAsync(c.d_bcell_count.p, 0, sizeof(int) * c.nblocks, st);
  cudaMemsetAsync(c.d_bcell_cursor.p, 0, sizeof(int) * c.nblocks, st);
  k_bgrid_count<<<nblk(c.nblocks, 256), 256, 0, st>>>(v, c.d_bgrid.p, c.d_bcell.p, c.d_bcell_count.p);
  scan_ints(c, c.d_bcell_count.p, c.d_bcell_off.p, c.d_bcell_scan_tmp.p, c.nblocks, st);
  k_bgrid_scatter<<<nblk(c.nblocks, 256), 256, 0, st>>>(c.nblocks, c.d_bcell.p, c.d_bcell_off.p,
                                                         c.d_bcell_cursor.p, c.d_bcell_blocks.p);
  launch_rows(c, list_radius, full_radius);
  if (sizing != kListDevice) {
    // the tile count against the capacity: a list that outgrew the arrays is
    // rebuilt into grown ones
    int total = 0;
    if (cudaMemcpyAsync(&total, c.d_counters.p + 6, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return PDGPU_ERR_CUDA;
    if (total > c.tile_cap) {
      if (sizing == kListCheck) return PDGPU_ERR_CAPACITY;
      const int e = alloc_tiles(c, total);
      if (e != PDGPU_OK) return e;
      v = c.view();
      c.kernel_launches += 1;
      launch_rows(c, list_radius, full_radius);
    }
  }
  cudaMemsetAsync(c.d_counters.p, 0, sizeof(int) * 6, st);
  k_tile_total<<<1, 1, 0, st>>>(v, c.d_counters.p + 6, c.tile_cap);
  k_mask_mark<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_slot_of.p, c.d_row_start.p, c.d_row_cnt.p,
                                                   c.d_tile_need.p, c.d_mlist.p, c.d_counters.p + 7);
  k_masks<<<nblk((long long)c.mask_cap * 32, 256) < list_tile_grid(c) ? nblk((long long)c.mask_cap * 32, 256)
                                                                       : list_tile_grid(c),
            256, 0, st>>>(v, c.d_mlist.p, c.d_counters.p + 7);
  if (c.has_gb) {
    c.kernel_launches += 2;   // and a scan
    const int pairs = c.gb_item_tiles == 2 ? 1 : 0;
    k_item_flags<<<nblk(c.tile_cap, 256), 256, 0, st>>>(v, c.tile_cap, pairs, c.d_tile_flag.p);
    scan_ints(c, c.d_tile_flag.p, c.d_tile_pos.p, c.d_scan_tmp2.p, c.tile_cap, st);
    k_item_write<<<nblk(c.tile_cap, 256), 256, 0, st>>>(v, c.tile_cap, pairs, c.d_tile_flag.p, c.d_tile_pos.p);
  }
  k_pack<<<nblk(c.nslots, 256), 256, 0, st>>>(v, c.d_charge.p, 0.f, 0.f, 1, c.npairs_all, 0);
  // NB j-atom groups: only where the per-step displacement check runs
  c.cull_built = c.nb_set && c.nb_cull && c.lp.check_skin && c.cull_cap > 0;
  if (c.cull_built) launch_cull(c, list_radius);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_slot_params(Context& c) {
  c.kernel_launches += 1;
  DevView v = c.view();
  k_slot_params<<<nblk(c.nslots, 256), 256, 0, c.stream>>>(v, c.d_radius.p, c.d_sqeps.p,
                                                            c.has_gb ? c.d_gbR.p : nullptr,
                                                            c.has_gb ? c.d_gbVj.p : nullptr,
                                                            c.has_sa ? c.d_lcpoR.p : nullptr,
                                                            c.has_sa ? c.d_lcpoUse.p : nullptr,
                                                            c.has_sa ? c.d_lc_par.p : nullptr);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_pack(Context& c, float check_disp) {
  c.kernel_launches += 1;
  DevView v = c.view();
  float c2 = check_disp > 0 ? check_disp * check_disp : 0.f;
  float f2 = 0.f;
  if (c.full_radius_built > 0.f) {
    const float h = 0.5f * c.full_margin();
    f2 = h * h;
  }
  k_pack<<<nblk(c.nslots, 256), 256, 0, c.stream>>>(v, c.d_charge.p, c2, f2, 0, c.npairs_all,
                                                     c.cull_built ? 1 : 0);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
