// k_list.cu — cell-grid sort, blocks, tile list, exclusion masks and the
// per-evaluation position pack.  Replaces NeighbourList::calcNewList
// (PD src/mmlib/workspace/neighbourlist.cpp:222-439): PD scans all j < i at
// minimum image; here atoms are binned on a 32^3 grid ordered along a Hilbert
// curve, grouped into 32-atom blocks, and block pairs whose bounding boxes come
// within max(cutoffs)+Padding form the tile list.  The bond order PD packs into
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

__global__ void k_bbox_init(int* lo, int* hi, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    lo[i] = f2ord(3.0e38f);
    hi[i] = f2ord(-3.0e38f);
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

// --- exclusive scan (three-phase, 1024 elements per block) -----------------
__global__ void k_scan_block(const int* in, int* out, int* block_sums, int n) {
  __shared__ int sh[1024];
  int tid = threadIdx.x;
  int i = blockIdx.x * 1024 + tid;
  int x = i < n ? in[i] : 0;
  sh[tid] = x;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int y = tid >= o ? sh[tid - o] : 0;
    __syncthreads();
    sh[tid] += y;
    __syncthreads();
  }
  if (i < n) out[i] = sh[tid] - x;
  if (tid == 1023) block_sums[blockIdx.x] = sh[1023];
}

__global__ void k_scan_sums(int* sums, int nb) {
  // single block: sequential chunks, inclusive -> exclusive
  __shared__ int sh[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    int i = base + threadIdx.x;
    int x = i < nb ? sums[i] : 0;
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += y;
      __syncthreads();
    }
    if (i < nb) sums[i] = sh[threadIdx.x] - x + carry;
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
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

// block bounding boxes; one warp per block
__global__ void k_blocks(DevView v) {
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

// candidate block pairs -> include flags, in candidate order (row-major: bi, then bj >= bi)
__device__ __forceinline__ bool candidate_pair(const DevView& v, long long t, int& gi, int& gj, int& flags, float R,
                                               float margin, float full_R, float full_margin) {
  // system by binary search over cand_start
  int lo = 0, hi = v.nsys - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (v.sys[mid].cand_start <= t) lo = mid;
    else hi = mid - 1;
  }
  const SystemInfo& S = v.sys[lo];
  long long l = t - S.cand_start;
  long long nb = S.nblocks;
  // row bi starts at bi*nb - bi*(bi-1)/2 and holds nb-bi entries (FP32 estimate,
  // corrected by the integer tests below)
  const float q = 2.f * (float)nb + 1.f;
  float fb = (q - sqrtf(fmaxf(q * q - 8.f * (float)l, 0.f))) * 0.5f;
  long long bi = (long long)fb;
  if (bi < 0) bi = 0;
  if (bi > nb - 1) bi = nb - 1;
  while (bi > 0 && bi * nb - bi * (bi - 1) / 2 > l) bi--;
  while (bi + 1 < nb && (bi + 1) * nb - (bi + 1) * bi / 2 <= l) bi++;
  long long bj = bi + (l - (bi * nb - bi * (bi - 1) / 2));
  gi = S.block_start + (int)bi;
  gj = S.block_start + (int)bj;
  float4 hi4 = v.half[gi], hj4 = v.half[gj];
  float hs[3] = {hi4.x + hj4.x, hi4.y + hj4.y, hi4.z + hj4.z};
  // FP32 geometry (the FP64 pipe is narrow on this GPU), every decision taken
  // 1e-3 A on the safe side: include, per-pair image, not all-inside
  constexpr float kSafe = 1e-3f;
  float dist2 = 0.f, dmax2 = 0.f;
  bool need_mi = false;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float d = (float)(v.center[3 * gj + c] - v.center[3 * gi + c]);
    if (S.periodic) {
      const float L = (float)S.box[c];
      d -= L * rintf(d * (float)S.ibox[c]);
      if (fabsf(d) + hs[c] + margin >= 0.5f * L - kSafe) need_mi = true;
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

__global__ void k_tile_flags(DevView v, long long ncand, float R, float margin, int* flag) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncand) return;
  int gi, gj, fl;
  flag[t] = candidate_pair(v, t, gi, gj, fl, R, margin, 0.f, 0.f) ? 1 : 0;
}

// write the included pairs at their scanned positions: the tile list is in
// row-major order, so every run of tiles with one i-block is contiguous and
// its order is the same on every build
__global__ void k_tile_write(DevView v, long long ncand, float R, float margin, float full_R, float full_margin,
                             const int* flag, const int* pos) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncand) return;
  if (t == ncand - 1) *v.ntiles = pos[t] + flag[t];
  if (!flag[t]) return;
  int gi, gj, fl;
  candidate_pair(v, t, gi, gj, fl, R, margin, full_R, full_margin);
  Tile T;
  T.bi = gi;
  T.bj = gj;
  T.mask = -1;
  T.flags = fl;
  {
    const SystemInfo& S = v.sys[v.slot_sys[gi]];
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
  }
  v.tiles[pos[t]] = T;
}

// exclusion masks in rotation order (bit k <-> j slot (lane+k)&31); one warp per tile
// tiles holding a bonded pair (bond order <= 3: excluded or 1-4), marked from
// each atom's partners (band words, far list) through the candidate index of its
// block pair: need[tile] = 1.  flag / pos: the tile-compaction scan (candidate ->
// tile).  Diagonal tiles and tiles with padding slots are recognised in k_masks.
__global__ void k_mask_mark(DevView v, const int* slot_of, const int* flag, const int* pos, unsigned char* need) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= v.natom) return;
  const unsigned long long w = v.band_excl[a] | v.band_14[a];
  const int fs = v.far_start[a], fe = v.far_start[a + 1];
  if (!w && fs == fe) return;
  const int sa = slot_of[a];
  const int ga = sa >> 5;
  const SystemInfo& S = v.sys[v.slot_sys[ga]];
  auto mark = [&](int b) {
    const int gb = slot_of[b] >> 5;
    const long long bi = (ga < gb ? ga : gb) - S.block_start, bj = (ga < gb ? gb : ga) - S.block_start;
    const long long nb = S.nblocks;
    const long long l = S.cand_start + bi * nb - bi * (bi - 1) / 2 + (bj - bi);
    if (flag[l]) need[pos[l]] = 1;
  };
  for (unsigned long long m = w; m; m &= m - 1) mark(a + __ffsll((long long)m));
  for (int q = fs; q < fe; q++)
    if (v.far_bo[q] <= 3) mark(v.far_idx[q]);
}

// grid-stride over the tiles, one warp per tile; tiles without a bonded pair,
// padding slot or diagonal get no mask and skip the pair loop
__global__ void k_masks(DevView v, const unsigned char* need) {
  const int lane = threadIdx.x & 31;
  const int nt = *v.ntiles;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp < nt; warp += nwarps) {
    Tile T = v.tiles[warp];
    int ai = v.sorted_atom[T.bi * 32 + lane];
    int aj0 = v.sorted_atom[T.bj * 32 + lane];
    bool diag = T.flags & 2;
    if (!need[warp] && !diag && __all_sync(0xffffffffu, ai >= 0 && aj0 >= 0)) continue;
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
    v.masks[idx * 32 + lane] = make_uint2(ex, m14);
    if (lane == 0) v.tiles[warp].mask = idx;
  }
}

// per-evaluation pack: FP64 positions -> float offsets from the block centre
// check2: squared skin limit (0 = no skin check); full2: squared limit that keeps
// tiles flagged full valid (0 = none flagged), checked where the skin check is not
// cull: the NB j-atom groups are in use (the displacement check always runs)
__global__ void k_pack(DevView v, const double* charge, float check2, float full2, int store_ref, long long ncand,
                       int cull) {
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
      const bool skin = check2 > 0.f && (S.periodic || (long long)*v.ntiles < ncand || cull);
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
__global__ void k_item_flags(DevView v, long long ncand, int pairs, int* flag) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncand) return;
  const int nt = *v.ntiles;
  flag[t] = (t < nt && !(pairs && tile_pairable(v, (int)t - 1, nt))) ? 1 : 0;
}

__global__ void k_item_write(DevView v, long long ncand, int pairs, const int* flag, const int* pos) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncand) return;
  if (t == ncand - 1) *v.nitems = pos[t] + flag[t];
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
// cnt: zeroed beforehand over all candidates (the scan runs over them)
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

// pos: exclusive scan of the kept counts over the tile list (row-major, so a
// row's entries keep tile order, then lane order)
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
  const long long want = (c.ncand + 7) / 8, g = 16LL * (sms > 0 ? sms : 1);
  return (int)(want < g ? (want > 0 ? want : 1) : g);
}

static void launch_cull(Context& c, float list_radius) {
  c.kernel_launches += 10;
  DevView v = c.view();
  cudaStream_t st = c.stream;
  const int nb = c.nblocks;
  int* row = c.d_cull_row.p;
  cudaMemsetAsync(row, 0, sizeof(int) * nb, st);
  cudaMemsetAsync(row + nb, 0x7f, sizeof(int) * nb, st);
  const float R = list_radius + 1e-3f;
  // the kept counts and their scan reuse the tile-compaction arrays
  cudaMemsetAsync(c.d_tile_flag.p, 0, sizeof(int) * c.ncand, st);
  k_cull_mask<<<list_tile_grid(c), 256, 0, st>>>(v, R * R, c.d_cull_mask.p, c.d_tile_flag.p, row);
  const int nb2 = nblk(c.ncand, 1024);
  k_scan_block<<<nb2, 1024, 0, st>>>(c.d_tile_flag.p, c.d_tile_pos.p, c.d_scan_tmp2.p, (int)c.ncand);
  k_scan_sums<<<1, 1024, 0, st>>>(c.d_scan_tmp2.p, nb2);
  k_scan_add<<<nb2, 1024, 0, st>>>(c.d_tile_pos.p, c.d_scan_tmp2.p, (int)c.ncand);
  k_cull_groups<<<nblk(nb, 256), 256, 0, st>>>(nb, row);
  const int nb3 = nblk(nb, 1024);
  k_scan_block<<<nb3, 1024, 0, st>>>(row + 2 * nb, row + 3 * nb, c.d_cull_scan_tmp.p, nb);
  k_scan_sums<<<1, 1024, 0, st>>>(c.d_cull_scan_tmp.p, nb3);
  k_scan_add<<<nb3, 1024, 0, st>>>(row + 3 * nb, c.d_cull_scan_tmp.p, nb);
  k_cull_write<<<list_tile_grid(c), 256, 0, st>>>(v, c.d_cull_mask.p, c.d_tile_pos.p, row);
  k_cull_rows<<<nblk((long long)nb * 32, 256), 256, 0, st>>>(v, row);
}

int launch_list_build(Context& c, float list_radius, float full_radius) {
  c.kernel_launches += 19;
  DevView v = c.view();
  cudaStream_t st = c.stream;
  int ncells = c.nsys * kCellsPerSystem;
  int* lo = reinterpret_cast<int*>(c.d_sys_lo.p);
  int* hi = reinterpret_cast<int*>(c.d_sys_hi.p);
  k_bbox_init<<<nblk(3 * c.nsys, 128), 128, 0, st>>>(lo, hi, 3 * c.nsys);
  k_bbox<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_atom_sys.p, lo, hi);
  cudaMemsetAsync(c.d_count.p, 0, sizeof(int) * ncells, st);
  cudaMemsetAsync(c.d_cursor.p, 0, sizeof(int) * ncells, st);
  k_keys<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_atom_sys.p, lo, hi, c.d_bucket.p, c.d_count.p);
  int nsb = nblk(ncells, 1024);
  k_scan_block<<<nsb, 1024, 0, st>>>(c.d_count.p, c.d_offset.p, c.d_scan_tmp.p, ncells);
  k_scan_sums<<<1, 1024, 0, st>>>(c.d_scan_tmp.p, nsb);
  k_scan_add<<<nsb, 1024, 0, st>>>(c.d_offset.p, c.d_scan_tmp.p, ncells);
  k_scatter<<<nblk(c.natom, 256), 256, 0, st>>>(c.natom, c.d_bucket.p, c.d_offset.p, c.d_cursor.p,
                                                 c.d_tmp_sorted.p);
  k_cell_sort<<<nblk(ncells, 256), 256, 0, st>>>(ncells, c.d_offset.p, c.d_count.p, c.d_tmp_sorted.p);
  cudaMemsetAsync(c.d_sorted_atom.p, 0xff, sizeof(int) * c.nslots, st);
  k_to_slots<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_atom_sys.p, c.d_tmp_sorted.p, c.d_sorted_atom.p,
                                                  c.d_slot_of.p);
  k_blocks<<<nblk((long long)c.nblocks * 32, 256), 256, 0, st>>>(v);
  k_slot_params<<<nblk(c.nslots, 256), 256, 0, st>>>(v, c.d_radius.p, c.d_sqeps.p, c.has_gb ? c.d_gbR.p : nullptr,
                                                      c.has_gb ? c.d_gbVj.p : nullptr,
                                                      c.has_sa ? c.d_lcpoR.p : nullptr,
                                                      c.has_sa ? c.d_lcpoUse.p : nullptr,
                                                      c.has_sa ? c.d_lc_par.p : nullptr);
  cudaMemsetAsync(c.d_counters.p, 0, sizeof(int) * 6, st);
  k_tile_flags<<<nblk(c.ncand, 256), 256, 0, st>>>(v, c.ncand, list_radius, (float)c.lp.Padding, c.d_tile_flag.p);
  {
    int nb2 = nblk(c.ncand, 1024);
    k_scan_block<<<nb2, 1024, 0, st>>>(c.d_tile_flag.p, c.d_tile_pos.p, c.d_scan_tmp2.p, (int)c.ncand);
    k_scan_sums<<<1, 1024, 0, st>>>(c.d_scan_tmp2.p, nb2);
    k_scan_add<<<nb2, 1024, 0, st>>>(c.d_tile_pos.p, c.d_scan_tmp2.p, (int)c.ncand);
  }
  k_tile_write<<<nblk(c.ncand, 256), 256, 0, st>>>(v, c.ncand, list_radius, (float)c.lp.Padding, full_radius,
                                                    c.full_margin(), c.d_tile_flag.p, c.d_tile_pos.p);
  cudaMemsetAsync(c.d_tile_need.p, 0, c.ncand, st);
  k_mask_mark<<<nblk(c.natom, 256), 256, 0, st>>>(v, c.d_slot_of.p, c.d_tile_flag.p, c.d_tile_pos.p,
                                                   c.d_tile_need.p);
  k_masks<<<list_tile_grid(c), 256, 0, st>>>(v, c.d_tile_need.p);
  if (c.has_gb) {
    c.kernel_launches += 5;
    int nb2 = nblk(c.ncand, 1024);
    const int pairs = c.gb_item_tiles == 2 ? 1 : 0;
    k_item_flags<<<nblk(c.ncand, 256), 256, 0, st>>>(v, c.ncand, pairs, c.d_tile_flag.p);
    k_scan_block<<<nb2, 1024, 0, st>>>(c.d_tile_flag.p, c.d_tile_pos.p, c.d_scan_tmp2.p, (int)c.ncand);
    k_scan_sums<<<1, 1024, 0, st>>>(c.d_scan_tmp2.p, nb2);
    k_scan_add<<<nb2, 1024, 0, st>>>(c.d_tile_pos.p, c.d_scan_tmp2.p, (int)c.ncand);
    k_item_write<<<nblk(c.ncand, 256), 256, 0, st>>>(v, c.ncand, pairs, c.d_tile_flag.p, c.d_tile_pos.p);
  }
  k_pack<<<nblk(c.nslots, 256), 256, 0, st>>>(v, c.d_charge.p, 0.f, 0.f, 1, c.ncand, 0);
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
  k_pack<<<nblk(c.nslots, 256), 256, 0, c.stream>>>(v, c.d_charge.p, c2, f2, 0, c.ncand, c.cull_built ? 1 : 0);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
