// k_adjoint.cu — gradients of the nonbonded / GB energy with respect to the
// per-atom force-field parameters (charge, LJ radius, sqrt epsilon, GB radius,
// GB volume Vj, GB fixed term terms123).
//
// PD has no adjoint; its parameter derivatives are finite differences of
// Forcefield::calcEnergies after re-running setup() (nonbonded.cpp:1078-1084
// explains why setup must be repeated: calcCheckSum does not see parameter
// edits).  The energy being differentiated is PD's:
//   FF_NonBonded   nonbonded.cpp:687-833
//   GB (FastMode)  gbff.cpp:1546-1746 (pair + self terms), Born radii
//                  gbff.cpp:432-483 with a = -halfeconv / Gpol + BornRadiusOffset
// The derivative is the exact one of that energy (dE/dGpol = dE/da *
// halfeconv / Gpol^2), not PD's force-path shortcut a^2/166 (gbff.cpp:1790),
// which differs from it by the Born offset and by 166 vs halfeconv.
//
// Layout: the same tiles and slots as the force kernels.  Pair distances and
// most pair terms are FP32; for FF_NonBonded the Coulomb energy per unit charge
// product is formed in FP64 (the force-switch form cancels badly in FP32).  A
// charge gradient is a potential: a sum of many terms of both signs, which plain
// FP32 sums do not resolve to the 1e-4 a parameter fit checks against.  The GB
// kernels therefore sum per tile in compensated FP32 (value plus running
// rounding error, about 48 significant bits, on the FP32 pipe: GB300's FP64 rate
// is a small fraction of its FP32 rate), fed by plain FP32 sums over 8 rotation
// steps; the NB kernel sums in FP64.  Per-tile sums
// enter 64-bit fixed point (2^32 per kcal/mol per parameter unit), so the result
// does not depend on scheduling.
#include "pdgpu_tile.cuh"

namespace pdgpu {

enum { G_Q = 0, G_R, G_EPS, G_GBR, G_VJ, G_NACC };

struct Acc3 {
  double a, b, c;
};

__device__ __forceinline__ long long fix_sum_d(double x) { return __double2ll_rn(x * kSumScale); }

// Compensated FP32 sum: hi carries the running sum and lo the rounding errors
// of its additions, each recovered exactly by Knuth's TwoSum (the _rn
// intrinsics keep the compiler from contracting or reordering the steps).
struct CSum {
  float hi, lo;
};

__device__ __forceinline__ void csum_add(CSum& c, float x) {
  const float s = __fadd_rn(c.hi, x);
  const float bb = __fsub_rn(s, c.hi);
  const float e = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  c.lo = __fadd_rn(c.lo, e);
  c.hi = s;
}

__device__ __forceinline__ double csum_value(const CSum& c) { return (double)c.hi + (double)c.lo; }

struct CAcc3 {
  CSum a, b, c;
};

__device__ __forceinline__ Acc3 cacc_value(const CAcc3& x) {
  return Acc3{csum_value(x.a), csum_value(x.b), csum_value(x.c)};
}

#define ROT_CSUM(x) \
  ROT(x.hi);        \
  ROT(x.lo)

// plain FP32 sums over 8 rotation steps, entered into the compensated sums at
// the end of each run of 8 (a short FP32 run adds only a few roundings of its
// own terms; the compensated sum then carries the long total)
struct Chunk3 {
  float a, b, c;
};

__device__ __forceinline__ void chunk_into(CAcc3& A, Chunk3& C) {
  csum_add(A.a, C.a);
  csum_add(A.b, C.b);
  csum_add(A.c, C.c);
  C.a = C.b = C.c = 0.f;
}

__device__ __forceinline__ void chunk_into2(CAcc3& A, Chunk3& C) {  // components a and b only
  csum_add(A.a, C.a);
  csum_add(A.b, C.b);
  C.a = C.b = 0.f;
}

__device__ __forceinline__ void acc_flush(const DevView& v, long long* g0, long long* g1, long long* g2, int s,
                                          const Acc3& x) {
  const double m = fabs(x.a) + fabs(x.b) + fabs(x.c);
  if (!(m < 1.0e9)) atomicOr(v.status, (unsigned)(m >= 1.0e9 ? ST_FIXED_OVERFLOW : ST_NAN));
  if (g0) atomic_add_ll(&g0[s], fix_sum_d(x.a));
  if (g1) atomic_add_ll(&g1[s], fix_sum_d(x.b));
  if (g2) atomic_add_ll(&g2[s], fix_sum_d(x.c));
}

// dE/dRmin of the LJ term eps (A - 2B) S(r), A = (R/r)^12, B = (R/r)^6, written
// without dividing by R (two zero-radius hydrogens give 0, not 0/0)
__device__ __forceinline__ float lj_dR(float R, float invr) {
  const float R2 = R * R, ir2 = invr * invr;
  const float b5 = R2 * R2 * R * (ir2 * ir2 * ir2);  // B / R
  const float t = R * invr, t2 = t * t;
  const float B = t2 * t2 * t2;
  return 12.f * b5 * (B - 1.f);                      // 12 (A - B) / R
}

// ---------------------------------------------------------------------------
// GB + vacuum pair terms: dE/dq, dE/dRmin, dE/dsqrt(eps) (Born radii held fixed;
// their dependence on the GB parameters goes through dE/da in k_adj_born)
// ---------------------------------------------------------------------------
template <bool MASKED>
__device__ __forceinline__ void adj_gb_tile(const DevView& v, const GBConst& k, const Tile& T, int lane, int si,
                                            const float4& xi, const float4& pi, float ai, unsigned ex, unsigned m14,
                                            unsigned dmask, const float* born, CAcc3& I, CAcc3& J) {
  float4 xj = j_in_i_frame(v, T, lane);
  float4 pj = v.par[T.bj * 32 + lane];
  float aj = born[T.bj * 32 + lane];
  Chunk3 IC = {0.f, 0.f, 0.f}, JC = {0.f, 0.f, 0.f};  // JC rotates with its j atom
#pragma unroll 2
  for (int kk = 0; kk < 32; kk++) {
    const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    bool pair = true, excl = false, is14 = false;
    if (MASKED) {
      pair = !((dmask >> kk) & 1u);
      excl = (ex >> kk) & 1u;
      is14 = (m14 >> kk) & 1u;
    }
    // the GB term's code runs only when some lane may lie above the exp
    // threshold (warp vote, FP64 tie-break band included)
    const bool in = r2 <= k.cut2 && pair;
    const float u = -0.25f * __fdividef(r2, ai * aj);
    const bool any_gb = __any_sync(0xffffffffu, in && u >= k.thresh - 4e-6f * fabsf(k.thresh));
    if (in) {
      const float invr = rsqrtf(r2);
      const float r = r2 * invr;
      bool gbon = false;
      if (any_gb) {
        gbon = u > k.thresh;
        if (fabsf(u - k.thresh) <= 2e-6f * fabsf(k.thresh)) {
          const int a = v.sorted_atom[si], b = v.sorted_atom[T.bj * 32 + ((lane + kk) & 31)];
          gbon = a >= 0 && b >= 0 && -0.25 * r2_slots_fp64(v, si, T.bj * 32 + ((lane + kk) & 31)) /
                                             (v.born[a] * v.born[b]) > k.thresh_d;
        }
      }
      float S = 1.f;
      if (r >= k.inner) {
        const float w = r - k.inner;
        const float sw = 1.f - w * w * k.invw2;
        S = sw * sw;
      }
      const float s14 = is14 ? k.elec14 : 1.f;
      float phi = 0.f;  // energy per unit q_i q_j
      if (any_gb && gbon) {
        const float fgb = rsqrtf(r2 + __expf(u) * ai * aj);
        phi = 2.f * k.premul * fgb * S;
        if (!excl) phi += k.econv_in * s14 * invr * S;
      } else if (!excl) {
        phi = k.econv_out * s14 * invr * S;
      }
      IC.a += phi * xj.w;
      JC.a += phi * xi.w;
      if (!excl && r < k.vdwcut) {
        const float R = pi.x + pj.x;
        const float t = R * invr;
        float B = t * t;
        B = B * B * B;
        float Sv = is14 ? k.vdw14 : 1.f;
        if (r > k.vdwinner) {
          const float w = r - k.vdwinner;
          const float sw = 1.f - w * w * k.vdwinvw2;
          Sv *= sw * sw;
        }
        const float e1 = (B * B - 2.f * B) * Sv;  // energy per unit sqrt(eps_i) sqrt(eps_j)
        const float dR = lj_dR(R, invr) * Sv * pi.y * pj.y;
        IC.b += dR;
        JC.b += dR;
        IC.c += e1 * pj.y;
        JC.c += e1 * pi.y;
      }
    }
    if ((kk & 7) == 7) {
      chunk_into(I, IC);
      chunk_into(J, JC);
    }
    ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(xj.w); ROT(pj.x); ROT(pj.y); ROT(aj);
    ROT_CSUM(J.a); ROT_CSUM(J.b); ROT_CSUM(J.c);
    ROT(JC.a); ROT(JC.b); ROT(JC.c);
  }
}

__global__ void __launch_bounds__(256) k_adj_gb_pair(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* born, long long* gq,
                                                      long long* gr, long long* ge) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    const float ai = born[si];
    unsigned ex, m14;
    tile_masks(v, T, lane, ex, m14);
    const unsigned dmask = (T.flags & 2) ? diag_exclusion(lane) : 0u;
    CAcc3 I = {}, J = {};
    if (tile_masked(T)) adj_gb_tile<true>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J);
    else adj_gb_tile<false>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J);
    acc_flush(v, gq, gr, ge, si, cacc_value(I));
    acc_flush(v, gq, gr, ge, T.bj * 32 + lane, cacc_value(J));
  }
}

// ---------------------------------------------------------------------------
// Born-radius sums Gpol_i += P4 Vj CCF(r^2/(Ri+Rj)^2) / r^4 (bond order > 2,
// r <= GbsaStillCutoff): dE/dVj and dE/dR through w = dE/dGpol per slot
// ---------------------------------------------------------------------------
template <bool MASKED>
__device__ __forceinline__ void adj_born_tile(const DevView& v, const GBConst& k, const Tile& T, int lane, int si,
                                              const float4& xi, const float4& pi, float wi, unsigned ex,
                                              const float* w, CAcc3& I, CAcc3& J) {
  float4 xj = j_in_i_frame(v, T, lane);
  float4 pj = v.par[T.bj * 32 + lane];
  float wj = w[T.bj * 32 + lane];
  Chunk3 IC = {0.f, 0.f, 0.f}, JC = {0.f, 0.f, 0.f};  // (a, b used) JC rotates with its j atom
#pragma unroll 4
  for (int kk = 0; kk < 32; kk++) {
    const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    bool in = r2 <= k.still2;
    if (fabsf(r2 - k.still2) <= 2e-6f * k.still2)
      in = r2_slots_fp64(v, si, T.bj * 32 + ((lane + kk) & 31)) <= k.still2_d;
    if (MASKED) in = in && !((ex >> kk) & 1u);
    // close contact (r^2 <= rs^2 / P5, where the CCF switches on) is rare: its
    // branch runs on a warp vote
    const float rs = pi.z + pj.z, rs2 = rs * rs;
    const bool anyc = __any_sync(0xffffffffu, in && r2 <= rs2 * k.invP5);
    if (in) {
      float ccf = 1.f, gx = 0.f;  // CCF, and dCCF/dx * dx/dR (0 outside contact)
      if (anyc) {
        if (r2 <= rs2 * k.invP5) {
          const float x = __fdividef(r2, rs2);
          float sn, cs;
          sincospif(x * k.P5, &sn, &cs);
          const float h = 0.5f - 0.5f * cs;
          ccf = h * h;
          gx = h * sn * (k.P5 * 3.14159265358979f) * (-2.f * __fdividef(x, rs));
        }
      }
      const float ir2 = __fdividef(1.f, r2);
      const float h4 = k.P4 * ir2 * ir2;
      IC.b += wj * h4 * ccf;  // dE/dV_i from Gpol_j
      JC.b += wi * h4 * ccf;  // dE/dV_j from Gpol_i
      const float gR = (wi * pj.w + wj * pi.w) * h4 * gx;
      IC.a += gR;
      JC.a += gR;
    }
    if ((kk & 7) == 7) {
      chunk_into2(I, IC);
      chunk_into2(J, JC);
    }
    ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(pj.z); ROT(pj.w); ROT(wj); ROT_CSUM(J.a); ROT_CSUM(J.b);
    ROT(JC.a); ROT(JC.b);
  }
}

__global__ void __launch_bounds__(256) k_adj_born(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* w, long long* gR,
                                                   long long* gV) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    const float wi = w[si];
    unsigned ex, m14;
    tile_masks(v, T, lane, ex, m14);
    if (T.flags & 2) ex |= diag_exclusion(lane);
    CAcc3 I = {}, J = {};
    if (tile_masked(T)) adj_born_tile<true>(v, k, T, lane, si, xi, pi, wi, ex, w, I, J);
    else adj_born_tile<false>(v, k, T, lane, si, xi, pi, wi, ex, w, I, J);
    acc_flush(v, gR, gV, nullptr, si, cacc_value(I));
    acc_flush(v, gR, gV, nullptr, T.bj * 32 + lane, cacc_value(J));
  }
}

// dE/dGpol per slot: (dE/da from the pair pass - E_self / a) * halfeconv / Gpol^2
__device__ __forceinline__ double dE_dGpol(const DevView& v, const double* terms123, const long long* gpol,
                                           const long long* deda, double premul, double halfeconv, int s, int a) {
  const double G = terms123[a] + (double)gpol[s] * (1.0 / kSumScale);
  const double ai = v.born[a], q = v.charge[a];
  const double da = (double)deda[s] * (1.0 / kSumScale) - premul * q * q / (ai * ai);
  return da * halfeconv / (G * G);
}

__global__ void k_adj_w(DevView v, const double* terms123, const long long* gpol, const long long* deda,
                        double premul, double halfeconv, float* w) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  w[s] = a < 0 ? 0.f : (float)dE_dGpol(v, terms123, gpol, deda, premul, halfeconv, s, a);
}

// ---------------------------------------------------------------------------
// NB (FF_NonBonded) pair terms: dE/dq, dE/dRmin, dE/dsqrt(eps)
// ---------------------------------------------------------------------------
template <int ELEC, bool MASKED>
__device__ __forceinline__ void adj_nb_tile(const DevView& v, const NBConst& k, const Tile& T, const SystemInfo& S,
                                            int lane, int si, const float4& xi, const float4& pi, unsigned ex,
                                            unsigned m14, Acc3& I, Acc3& J) {
  float4 xj = v.xq[T.bj * 32 + lane];
  float4 pj = v.par[T.bj * 32 + lane];
  float Lx = 1.f, Ly = 1.f, Lz = 1.f;
  if (S.periodic) {
    Lx = (float)S.box[0]; Ly = (float)S.box[1]; Lz = (float)S.box[2];
  }
  xj.x += T.ox;
  xj.y += T.oy;
  xj.z += T.oz;
  const bool mi = T.flags & 1;
  const float iLx = 1.f / Lx, iLy = 1.f / Ly, iLz = 1.f / Lz;
#pragma unroll 2
  for (int kk = 0; kk < 32; kk++) {
    float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    if (mi) {
      dx -= Lx * rintf(dx * iLx);
      dy -= Ly * rintf(dy * iLy);
      dz -= Lz * rintf(dz * iLz);
    }
    float r2 = dx * dx + dy * dy + dz * dz;
    bool listed = true;
    if (MASKED) listed = !((ex >> kk) & 1u);
    bool in = r2 <= k.cut2;
    if (listed && (fabsf(r2 - k.cut2) <= 2e-6f * k.cut2 || fabsf(r2 - k.vdwcut2) <= 2e-6f * k.vdwcut2)) {
      const double r2d = r2_fp64(v, S, si, T.bj * 32 + ((lane + kk) & 31));
      in = r2d <= k.cut2_dd;
      r2 = (float)r2d;
    }
    if (listed && in) {
      const bool is14 = MASKED && ((m14 >> kk) & 1u);
      const float sv = is14 ? k.vdw14 : 1.f;
      float ev = 0.f, ee = 0.f, fs, rd;
      // unit sqrt(eps_i) sqrt(eps_j) and unit q_i q_j: both terms are linear in them
      nb_pair<float, ELEC>(k, r2, pi.x + pj.x, sv, 0.f, ev, ee, fs, rd);
      double evd = 0.0, eed = 0.0, fsd, rdd;
      nb_pair<double, ELEC>(k, (double)r2, 0.0, 0.0, (is14 ? k.elec14_d : 1.0) * k.econv_diel_d, evd, eed, fsd, rdd);
      I.a += eed * (double)xj.w;
      J.a += eed * (double)xi.w;
      I.c += (double)(ev * pj.y);
      J.c += (double)(ev * pi.y);
      const float invr = rsqrtf(r2), r = r2 * invr;
      if (k.dovdw && r < (float)k.vdwcut_d) {
        float Sv = sv;
        if (r > (float)k.vdwinner_d) {
          const float u = r - (float)k.vdwinner_d;
          const float sw = 1.f - u * u * (float)k.vdwinvw2_d;
          Sv *= sw * sw;
        }
        const float dR = lj_dR(pi.x + pj.x, invr) * Sv * pi.y * pj.y;
        I.b += (double)dR;
        J.b += (double)dR;
      }
    }
    ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(xj.w); ROT(pj.x); ROT(pj.y);
    ROT(J.a); ROT(J.b); ROT(J.c);
  }
}

template <int ELEC>
__global__ void __launch_bounds__(256) k_adj_nb(const __grid_constant__ DevView v, const __grid_constant__ NBConst k, long long* gq, long long* gr, long long* ge) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    const SystemInfo& S = v.sys[v.slot_sys[T.bi]];
    unsigned ex = 0u, m14 = 0u;
    if (T.mask >= 0) {
      uint2 m = v.masks[T.mask * 32 + lane];
      ex = m.x;
      m14 = m.y;
    }
    if (T.flags & 2) ex |= diag_exclusion(lane);
    Acc3 I = {0.0, 0.0, 0.0}, J = {0.0, 0.0, 0.0};
    if (tile_masked(T)) adj_nb_tile<ELEC, true>(v, k, T, S, lane, si, xi, pi, ex, m14, I, J);
    else adj_nb_tile<ELEC, false>(v, k, T, S, lane, si, xi, pi, ex, m14, I, J);
    acc_flush(v, gq, gr, ge, si, I);
    acc_flush(v, gq, gr, ge, T.bj * 32 + lane, J);
  }
}

// ---------------------------------------------------------------------------
// fixed point per slot -> J per parameter unit, original atom order
// ---------------------------------------------------------------------------
struct AdjOut {
  double *q, *r, *e, *R, *V, *T;
};

__global__ void k_adj_out(DevView v, const long long* g, int nslots, bool gb, const double* terms123,
                          const long long* gpol, const long long* deda, double premul, double halfeconv,
                          double eps_unit, AdjOut o) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  if (a < 0) return;
  const double f = 1.0 / kSumScale;
  double gq = (double)g[G_Q * (size_t)nslots + s] * f;
  if (gb) {
    const double ai = v.born[a];
    gq += 2.0 * premul * v.charge[a] / ai;  // self energy premul q^2 / a
  }
  if (o.q) o.q[a] = gq * kKcalMolToJ;
  if (o.r) o.r[a] = (double)g[G_R * (size_t)nslots + s] * f * kKcalMolToJ;
  if (o.e) o.e[a] = (double)g[G_EPS * (size_t)nslots + s] * f * eps_unit * kKcalMolToJ;
  if (o.R) o.R[a] = gb ? (double)g[G_GBR * (size_t)nslots + s] * f * kKcalMolToJ : 0.0;
  if (o.V) o.V[a] = gb ? (double)g[G_VJ * (size_t)nslots + s] * f * kKcalMolToJ : 0.0;
  if (o.T) o.T[a] = gb ? dE_dGpol(v, terms123, gpol, deda, premul, halfeconv, s, a) * kKcalMolToJ : 0.0;
}


// Runs after an energy evaluation of the same component (its Born radii, Gpol
// sums and dE/da are read from the context).  g: G_NACC * nslots fixed-point
// accumulators (cleared here), w: nslots floats (written in full here).
static int launch_adjoint_into(Context& c, unsigned what, long long* g, float* w, double* d_q, double* d_r,
                               double* d_e, double* d_R, double* d_V, double* d_T) {
  DevView v = c.view();
  cudaStream_t st = c.stream;
  const int ns = c.nslots;
  const int grid = tile_grid(c), nb = (ns + 255) / 256;
  const bool gb = (what & PDGPU_GB) != 0;
  const double ec = econv_kcal();
  const double halfeconv = 0.5 * ec;
  const double premul = gb ? -0.5 * ec * (1.0 / c.gb.DielectricSolute - 1.0 / c.gb.DielectricSolvent) : 0.0;
  if (cudaMemsetAsync(g, 0, sizeof(long long) * G_NACC * (size_t)ns, st) != cudaSuccess) return PDGPU_ERR_CUDA;
  long long *gq = g + G_Q * (size_t)ns, *gr = g + G_R * (size_t)ns, *ge = g + G_EPS * (size_t)ns;
  if (gb) {
    GBConst k = make_gb_const(c.gb, c.list_radius_built);
    c.kernel_launches += 3;
    k_adj_gb_pair<<<grid, 256, 0, st>>>(v, k, c.d_born_f.p, gq, gr, ge);
    k_adj_w<<<nb, 256, 0, st>>>(v, c.d_gbT.p, c.d_gpol.p, c.d_deda.p, premul, halfeconv, w);
    k_adj_born<<<grid, 256, 0, st>>>(v, k, w, g + G_GBR * (size_t)ns, g + G_VJ * (size_t)ns);
  } else {
    NBConst k = make_nb_const(c.nb);
    c.kernel_launches += 1;
    switch (k.elecmode) {
      case 0: k_adj_nb<0><<<grid, 256, 0, st>>>(v, k, gq, gr, ge); break;
      case 1: k_adj_nb<1><<<grid, 256, 0, st>>>(v, k, gq, gr, ge); break;
      case 3: k_adj_nb<3><<<grid, 256, 0, st>>>(v, k, gq, gr, ge); break;
      default: k_adj_nb<4><<<grid, 256, 0, st>>>(v, k, gq, gr, ge); break;
    }
  }
  AdjOut o = {d_q, d_r, d_e, d_R, d_V, d_T};
  c.kernel_launches += 1;
  k_adj_out<<<nb, 256, 0, st>>>(v, g, ns, gb, c.d_gbT.p, c.d_gpol.p, c.d_deda.p, premul, halfeconv,
                                std::sqrt(kNa / kKcal2J), o);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_adjoint(Context& c, unsigned what, double* d_q, double* d_r, double* d_e, double* d_R, double* d_V,
                   double* d_T) {
  if (c.d_adj.n < (size_t)G_NACC * c.nslots) {
    if (c.d_adj.alloc((size_t)G_NACC * c.nslots) != cudaSuccess) return PDGPU_ERR_CUDA;
    if (c.d_adj_w.alloc((size_t)c.nslots) != cudaSuccess) return PDGPU_ERR_CUDA;
  }
  return launch_adjoint_into(c, what, c.d_adj.p, c.d_adj_w.p, d_q, d_r, d_e, d_R, d_V, d_T);
}

// ---------------------------------------------------------------------------
// Fixed scratch for the gradient call of hosts that must not allocate device
// memory inside a call.  cudaMalloc and cudaFree synchronise the whole device,
// so a host that keeps other streams busy (a fitting loop beside dynamics of
// other replicas), or whose own pool allocator holds the free memory, cannot
// let pdgpu_param_grad_device allocate its scratch on first use.  This array
// sits in the library's static device data instead: kNoAllocMaxSlots sorted
// slots, G_NACC int64 accumulators and one float each (2.75 MiB), held by every
// GPU that loads the library until the process exits.  All contexts on a
// device share it, so calls whose GPU work overlaps race.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_adj_scratch[(size_t)kNoAllocMaxSlots *
                                                             (G_NACC * sizeof(long long) + sizeof(float))];

int launch_adjoint_static(Context& c, unsigned what, double* d_q, double* d_r, double* d_e, double* d_R, double* d_V,
                          double* d_T) {
  if (c.nslots > kNoAllocMaxSlots) return PDGPU_ERR_CAPACITY;
  // The array's device address on the current device (the caller made the
  // context's device current).  In host code the array's name only stands in
  // for the symbol.  Looked up on every call: the lookup is cheap once the
  // module is loaded, keeps no host-side cache (nothing to go stale after a
  // device reset, nothing shared between host threads), and the first call on
  // a device may load the library's device code there.
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_adj_scratch) != cudaSuccess || !p) return PDGPU_ERR_CUDA;
  unsigned char* base = static_cast<unsigned char*>(p);
  long long* g = reinterpret_cast<long long*>(base);
  float* w = reinterpret_cast<float*>(base + (size_t)kNoAllocMaxSlots * G_NACC * sizeof(long long));
  return launch_adjoint_into(c, what, g, w, d_q, d_r, d_e, d_R, d_V, d_T);
}

}  // namespace pdgpu
