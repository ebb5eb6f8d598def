// pdgpu_tile.cuh — pieces shared by the tile kernels: lane rotation of the j
// block, diagonal-tile exclusion, FP64 distance rechecks, tile masks and the
// FF_NonBonded pair law.
#pragma once
#include "pdgpu_context.cuh"

namespace pdgpu {

__device__ __forceinline__ unsigned diag_exclusion(int lane) {
  return ~((lane == 0) ? 0xffffffffu : ((1u << (32 - lane)) - 1u)) | 1u;
}

#define ROT(x) x = __shfl_sync(0xffffffffu, x, (lane + 1) & 31)

// FP64 squared distance of two sorted slots from the original positions
static __device__ __noinline__ double r2_slots_fp64(const DevView& v, int sa, int sb) {
  int a = v.sorted_atom[sa], b = v.sorted_atom[sb];
  if (a < 0 || b < 0) return 1e300;
  double dx = v.pos[3 * b] - v.pos[3 * a], dy = v.pos[3 * b + 1] - v.pos[3 * a + 1],
         dz = v.pos[3 * b + 2] - v.pos[3 * a + 2];
  return dx * dx + dy * dy + dz * dz;
}

// j block of a tile moved into the i block's frame (centre offset in FP64)
__device__ __forceinline__ float4 j_in_i_frame(const DevView& v, const Tile& T, int lane) {
  float4 xj = v.xq[T.bj * 32 + lane];
  xj.x += T.ox;
  xj.y += T.oy;
  xj.z += T.oz;
  return xj;
}

// Whether a tile takes the masked body (bonded pairs or the diagonal).  The
// choice must be the same for all 32 lanes: the tile bodies rotate the j block
// with full-warp shuffles, which need every lane on the same path.
__device__ __forceinline__ bool tile_masked(const Tile& T) { return T.mask >= 0 || (T.flags & 2); }

// Whether every pair of the tile lies inside all cutoffs and switch radii of
// the list's components, with the list's displacement margin (set at build).
__device__ __forceinline__ bool tile_full(const Tile& T) { return (T.flags & 4) != 0; }

__device__ __forceinline__ void tile_masks(const DevView& v, const Tile& T, int lane, unsigned& ex, unsigned& m14) {
  ex = 0u;
  m14 = 0u;
  if (T.mask >= 0) {
    uint2 m = v.masks[T.mask * 32 + lane];
    ex = m.x;
    m14 = m.y;
  }
}

// bond order of an atom pair as PD's list stores it; 7 when not bonded
__device__ __forceinline__ int pair_bondorder(const DevView& v, int a, int b) {
  int lo = a < b ? a : b, hi = a < b ? b : a;
  int d = hi - lo;
  if (d == 0) return 0;
  if (d <= kBandWidth) {
    unsigned long long bit = 1ull << (d - 1);
    if (v.band_excl[lo] & bit) return 2;  // 1-1/1-2/1-3: all treated alike (excluded)
    if (v.band_14[lo] & bit) return 3;
    return 7;
  }
  int best = 7;
  for (int k = v.far_start[lo]; k < v.far_start[lo + 1]; k++)
    if (v.far_idx[k] == hi && v.far_bo[k] < best) best = v.far_bo[k];
  return best;
}

// Pair law in arithmetic type T (float for forces, double for energies).
template <typename T, int ELEC>
__device__ __forceinline__ void nb_pair(const NBConst& k, T r2, T rsum, T eps, T qq, T& ev, T& ee, T& dEdr_over_r,
                                        T& r_dEdr) {
  T invr, r;
  if (sizeof(T) == 4) {
    invr = rsqrtf((float)r2);
    r = r2 * invr;
  } else {
    r = sqrt((double)r2);
    invr = (T)1 / r;
  }
  T dv = 0, de = 0, Ev = 0, Ee = 0;
  if (k.dovdw && r < (T)k.vdwcut_d) {
    T t = rsum * invr;
    T B = t * t;
    B = B * B * B;
    T A = B * B;
    Ev = eps * (A - (T)2 * B);
    dv = (T)-12 * eps * invr * (A - B);
    if (r > (T)k.vdwinner_d) {
      T u = r - (T)k.vdwinner_d;
      T sw = (T)1 - u * u * (T)k.vdwinvw2_d;
      T dS = (T)-4 * (T)k.vdwinvw2_d * u * sw;
      T S = sw * sw;
      dv = S * dv + Ev * dS;
      Ev *= S;
    }
  }
  if (ELEC == 1) {
    Ee = qq * invr;
    de = -Ee * invr;
  } else if (ELEC == 3) {
    Ee = qq * invr;
    de = -Ee * invr;
    if (r > (T)k.inner_d) {
      T u = r - (T)k.inner_d;
      T sw = (T)1 - u * u * (T)k.invw2_d;
      T dS = (T)-4 * (T)k.invw2_d * u * sw;
      T S = sw * sw;
      de = S * de + Ee * dS;
      Ee *= S;
    }
  } else if (ELEC == 4) {
    // Steinbach & Brooks force switch, nonbonded.cpp:798-819
    if (r > (T)k.inner_d) {
      T c2mr2 = (T)k.cut2_d - r2;
      de = -qq * (T)k.sA * invr * invr * c2mr2 * c2mr2 * ((T)k.cut2_d - (T)3 * (T)k.inner2_d + (T)2 * r2);
      Ee = -qq * ((T)k.sA * r * ((T)k.sB * invr * invr + (T)k.sC + (T)k.sD * r2 + (T)k.sE * r2 * r2) - (T)k.fsw_cutV);
    } else {
      de = -qq * invr * invr;
      Ee = qq * (invr - (T)k.eshift);
    }
  }
  ev += Ev;
  ee += Ee;
  T d = dv + de;
  dEdr_over_r = d * invr;
  r_dEdr = r * d;
}

// FP64 squared distance of two sorted slots from the original positions
// (minimum image in a periodic box); used for energies and for pairs whose
// FP32 distance lies within 2e-6 of a hard cutoff.
__device__ __forceinline__ double r2_fp64(const DevView& v, const SystemInfo& S, int sa, int sb) {
  int a = v.sorted_atom[sa], b = v.sorted_atom[sb];
  if (a < 0 || b < 0) return 1e300;
  double r2 = 0;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double d = v.pos[3 * b + c] - v.pos[3 * a + c];
    if (S.periodic) d -= S.box[c] * rint(d * S.ibox[c]);
    r2 += d * d;
  }
  return r2;
}

}  // namespace pdgpu
