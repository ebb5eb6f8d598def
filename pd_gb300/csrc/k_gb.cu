// k_gb.cu — Still Generalised Born (FastMode).
//
// PD src/mmlib/forcefields/gbff.cpp:
//   Born radii            calcBornRadii_PairwiseApprox   :432-483
//   fused GB+LJ+Coulomb   calcForcesIncludingVacuo loop1 :1546-1746 (+ self term :1740-1745)
//   Born-radius chain     calcForcesIncludingVacuo loop2 :1768-1825
// GB uses plain Euclidean distances, as PD does.
//
// Work decomposition: one warp per GB work item (grid-stride over the item list
// the list build writes): a single 32x32 tile, or a tile pair (bi, bj),
// (bi, bj + 1) of one row.  In a single tile lane l holds i atom l and the j
// block rotates through the warp by shuffles; in a tile pair each lane holds
// one atom of each j block and the shared bi block rotates, so one rotation
// serves two pairs (the Born and chain bodies also run the two pairs on packed
// f32x2 arithmetic).  Every FP32 sum is converted to 64-bit fixed point and
// added atomically once per item (so a slot's total does not depend on the
// order in which items run).  Tiles without bonded pairs take a path without
// mask tests.  Registers decide the occupancy of these kernels.
#include "pdgpu_tile.cuh"

namespace pdgpu {

// 1 / x by the special-function unit alone (rcp.approx.ftz, ~1 ulp): the pair
// terms' reciprocals of r^2 (no multiply by the numerator 1 as __fdividef has)
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ---------------------------------------------------------------------------
// pass 1: Born-radius pair sums  Gpol_i += P4 Vj CCF / r^4  (bond order > 2)
// ---------------------------------------------------------------------------
// inside GbsaStillCutoff (FULL: the whole tile is); pairs within FP32 rounding of
// the cutoff are decided in FP64
template <bool FULL>
__device__ __forceinline__ bool still_in(const DevView& v, const GBConst& k, float r2, int sa, int sb) {
  if (FULL) return true;
  bool in = r2 <= k.still2;
  if (fabsf(r2 - k.still2) <= 2e-6f * k.still2) in = r2_slots_fp64(v, sa, sb) <= k.still2_d;
  return in;
}

// Close contact, r^2 / (R_i + R_j)^2 <= 1 / P5, where the CCF switches on.  Tested
// as r^2 <= rs^2 / P5 (no division); the CCF is continuous there (h = 1), so
// the rounding of the test does not matter.  Rare in a tile: the bodies take
// the branch only when some lane of the warp needs it (a warp vote), so the
// trigonometric code is skipped, not predicated, on nearly every step.
__device__ __forceinline__ bool gb_contact(const GBConst& k, float r2, float rs2) { return r2 <= rs2 * k.invP5; }

// P4 CCF / r^4 of one pair (rs = R_i + R_j, raw type radii); any_contact: the
// warp vote over gb_contact
__device__ __forceinline__ float born_w(const GBConst& k, float r2, float rs, bool any_contact) {
  const float rs2 = rs * rs;
  float ccf = 1.f;
  if (any_contact) {
    if (gb_contact(k, r2, rs2)) {
      const float h = 0.5f - 0.5f * cospif(__fdividef(r2, rs2) * k.P5);
      ccf = h * h;
    }
  }
  const float ir2 = rcp_ftz(r2);
  return k.P4 * ccf * ir2 * ir2;
}

template <bool MASKED, bool FULL>
__device__ __forceinline__ void born_tile(const DevView& v, const GBConst& k, const Tile& T, int lane, int si,
                                          const float4& xi, const float4& pi, unsigned ex, float& gi, float& gj) {
  float4 xj = j_in_i_frame(v, T, lane);
  float4 pj = v.par[T.bj * 32 + lane];
#pragma unroll 4
  for (int kk = 0; kk < 32; kk++) {
    const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    bool in = still_in<FULL>(v, k, r2, si, T.bj * 32 + ((lane + kk) & 31));
    if (MASKED) in = in && !((ex >> kk) & 1u);
    const float rs = pi.z + pj.z;
    const bool anyc = __any_sync(0xffffffffu, in && gb_contact(k, r2, rs * rs));
    if (in) {
      const float w = born_w(k, r2, rs, anyc);
      gi += w * pj.w;
      gj += w * pi.w;
    }
    ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(pj.z); ROT(pj.w); ROT(gj);
  }
}

// Tile pairs: two unmasked, off-diagonal tiles (bi, bj) and (bi, bj + 1) of one
// row at once.  The shared bi block rotates through the warp and each lane keeps
// one atom of each j block (moved into bi's frame), so one rotation of the bi
// atom (its data and its running sums) serves two pairs instead of one.  The two
// pairs' arithmetic runs on packed FP32x2 instructions (.x: the atom of bj,
// .y: the atom of bj + 1), which halves the instructions issued for it.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

template <bool FULL>
__device__ __forceinline__ void born_tile2(const DevView& v, const GBConst& k, const Tile& A, const Tile& B, int lane,
                                           long long* gpol) {
  const int sa = A.bj * 32 + lane, sb = B.bj * 32 + lane, r0 = A.bi * 32;
  const float4 xa = j_in_i_frame(v, A, lane), xb = j_in_i_frame(v, B, lane);
  const float4 pa = v.par[sa], pb = v.par[sb];
  const float2 nx = make_float2(-xa.x, -xb.x), ny = make_float2(-xa.y, -xb.y), nz = make_float2(-xa.z, -xb.z);
  const float2 RS = make_float2(pa.z, pb.z), P4 = f2(k.P4);
  float4 xr = v.xq[r0 + lane], pr = v.par[r0 + lane];
  float2 G = f2(0.f);
  float gr = 0.f;
#pragma unroll 4
  for (int kk = 0; kk < 32; kk++) {
    const int sr = r0 + ((lane + kk) & 31);
    const float2 dx = __fadd2_rn(f2(xr.x), nx), dy = __fadd2_rn(f2(xr.y), ny), dz = __fadd2_rn(f2(xr.z), nz);
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 rs = __fadd2_rn(RS, f2(pr.z));
    const float2 rs2 = __fmul2_rn(rs, rs);
    const float2 lim = __fmul2_rn(rs2, f2(k.invP5));
    const bool ca = r2.x <= lim.x, cb = r2.y <= lim.y;
    float2 ccf = f2(1.f);
    if (__any_sync(0xffffffffu, ca || cb)) {
      if (ca) {
        const float h = 0.5f - 0.5f * cospif(__fdividef(r2.x, rs2.x) * k.P5);
        ccf.x = h * h;
      }
      if (cb) {
        const float h = 0.5f - 0.5f * cospif(__fdividef(r2.y, rs2.y) * k.P5);
        ccf.y = h * h;
      }
    }
    const float2 ir2 = make_float2(rcp_ftz(r2.x), rcp_ftz(r2.y));
    float2 w = __fmul2_rn(__fmul2_rn(P4, ccf), __fmul2_rn(ir2, ir2));
    if (!FULL) {
      if (!still_in<false>(v, k, r2.x, sa, sr)) w.x = 0.f;
      if (!still_in<false>(v, k, r2.y, sb, sr)) w.y = 0.f;
    }
    G = __ffma2_rn(w, f2(pr.w), G);
    gr = fmaf(w.x, pa.w, gr);
    gr = fmaf(w.y, pb.w, gr);
    ROT(xr.x); ROT(xr.y); ROT(xr.z); ROT(pr.z); ROT(pr.w); ROT(gr);
  }
  fix_range(v.status, fabsf(G.x) + fabsf(G.y) + fabsf(gr));
  atomic_add_ll(&gpol[sa], fx32(G.x));
  atomic_add_ll(&gpol[sb], fx32(G.y));
  atomic_add_ll(&gpol[r0 + lane], fx32(gr));
}

// ---------------------------------------------------------------------------
// All-inside tile pairs (every pair inside every cutoff, no exclusions: the
// all-pairs case) take lean Born and chain-rule bodies: per-atom factors are
// folded into the values loaded once per item, and the close-contact (CCF)
// branch is entered on a warp vote over a coarse bound of the item,
// (max R_i + max R_j)^2 / P5, instead of each pair's own limit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_max(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// an upper bound of (R_i + R_j)^2 / P5 over the pairs of a tile pair: held raw
// GB radii RS, the rotating block's Rr
__device__ __forceinline__ float pair_contact2(const GBConst& k, float2 RS, float Rr) {
  const float m = warp_max(fmaxf(RS.x, RS.y)) + warp_max(Rr);
  return m * m * k.invP5 * 1.0001f;
}

// Step-packed lean bodies (Born, chain rule): lane l takes the rotating
// block's atoms l + kk and l + kk + 1 as one FP32x2 register pair, so a packed
// instruction covers two rotation steps of one held atom, whose values are
// broadcast into both halves once per item.  The rotating block is staged once
// per item in the warp's own shared-memory rows as step pairs (x_l, x_l+1,
// y_l, y_l+1) ..., read with one 16-byte load per four values; only its running
// sums rotate through the warp by shuffles, two lanes per step, so that after
// 16 rotations lane l's pair holds the sums of atoms l and l + 1.
#define ROT2(p) p.x = __shfl_sync(0xffffffffu, p.x, (lane + 2) & 31); p.y = __shfl_sync(0xffffffffu, p.y, (lane + 2) & 31)

// the CCF of one pair: 1 outside close contact
__device__ __forceinline__ float born_ccf(const GBConst& k, float r2, float rs) {
  const float rs2 = rs * rs;
  if (!gb_contact(k, r2, rs2)) return 1.f;
  const float h = 0.5f - 0.5f * cospif(__fdividef(r2, rs2) * k.P5);
  return h * h;
}

constexpr int kBornThreads = 256;
constexpr int kBornWarps = kBornThreads / 32;

__device__ __forceinline__ void born_full2(const DevView& v, const GBConst& k, const Tile& A, const Tile& B, int lane,
                                           long long* gpol) {
  __shared__ float4 rot_sh[kBornWarps][2][32];   // (x, x', y, y'), (z, z', P4 V, P4 V')
  float4 (*rs)[32] = rot_sh[threadIdx.x >> 5];
  const int sa = A.bj * 32 + lane, sb = B.bj * 32 + lane, r0 = A.bi * 32;
  const int l1 = (lane + 1) & 31;
  const float4 xa = j_in_i_frame(v, A, lane), xb = j_in_i_frame(v, B, lane);
  const float4 pa = v.par[sa], pb = v.par[sb];
  const float2 AX = f2(-xa.x), AY = f2(-xa.y), AZ = f2(-xa.z), BX = f2(-xb.x), BY = f2(-xb.y), BZ = f2(-xb.z);
  const float2 VA = f2(k.P4 * pa.w), VB = f2(k.P4 * pb.w);
  const float4 x0 = v.xq[r0 + lane], x1 = v.xq[r0 + l1];
  const float4 p0 = v.par[r0 + lane], p1 = v.par[r0 + l1];
  __syncwarp();
  rs[0][lane] = make_float4(x0.x, x1.x, x0.y, x1.y);
  rs[1][lane] = make_float4(x0.z, x1.z, k.P4 * p0.w, k.P4 * p1.w);
  __syncwarp();
  const float c2 = pair_contact2(k, make_float2(pa.z, pb.z), p0.z);
  float2 GA = f2(0.f), GB = f2(0.f), GR = f2(0.f);
#pragma unroll 4
  for (int kk = 0; kk < 32; kk += 2) {
    const int j = (lane + kk) & 31;
    const float4 P = rs[0][j], Q = rs[1][j];
    const float2 X = make_float2(P.x, P.y), Y = make_float2(P.z, P.w), Z = make_float2(Q.x, Q.y);
    const float2 VR = make_float2(Q.z, Q.w);
    const float2 ax = __fadd2_rn(X, AX), ay = __fadd2_rn(Y, AY), az = __fadd2_rn(Z, AZ);
    const float2 bx = __fadd2_rn(X, BX), by = __fadd2_rn(Y, BY), bz = __fadd2_rn(Z, BZ);
    const float2 ra = __ffma2_rn(az, az, __ffma2_rn(ay, ay, __fmul2_rn(ax, ax)));
    const float2 rb = __ffma2_rn(bz, bz, __ffma2_rn(by, by, __fmul2_rn(bx, bx)));
    const float2 ia = make_float2(rcp_ftz(ra.x), rcp_ftz(ra.y));
    const float2 ib = make_float2(rcp_ftz(rb.x), rcp_ftz(rb.y));
    float2 wa = __fmul2_rn(ia, ia), wb = __fmul2_rn(ib, ib);
    if (__any_sync(0xffffffffu, fminf(fminf(ra.x, ra.y), fminf(rb.x, rb.y)) <= c2)) {
      // rare: the rotating atoms' radii are read here, not staged
      const float R0 = v.par[r0 + j].z, R1 = v.par[r0 + ((j + 1) & 31)].z;
      wa.x *= born_ccf(k, ra.x, pa.z + R0);
      wa.y *= born_ccf(k, ra.y, pa.z + R1);
      wb.x *= born_ccf(k, rb.x, pb.z + R0);
      wb.y *= born_ccf(k, rb.y, pb.z + R1);
    }
    GA = __ffma2_rn(wa, VR, GA);
    GB = __ffma2_rn(wb, VR, GB);
    GR = __ffma2_rn(wa, VA, GR);
    GR = __ffma2_rn(wb, VB, GR);
    ROT2(GR);
  }
  // GR.x holds the sum of the rotating atom of this lane, GR.y that of lane + 1
  const float gr = GR.x + __shfl_sync(0xffffffffu, GR.y, (lane + 31) & 31);
  const float ga = GA.x + GA.y, gb = GB.x + GB.y;
  fix_range(v.status, fabsf(ga) + fabsf(gb) + fabsf(gr));
  atomic_add_ll(&gpol[sa], fx32(ga));
  atomic_add_ll(&gpol[sb], fx32(gb));
  atomic_add_ll(&gpol[r0 + lane], fx32(gr));
}

// the warp's next work item: a tile (t) or a tile pair (t, t + 1)
__device__ __forceinline__ int item_tile(const DevView& v, int it, bool& two) {
  const unsigned code = v.items[it];
  two = (code >> 31) != 0u;
  return (int)(code & 0x7fffffffu);
}

__global__ void __launch_bounds__(kBornThreads) k_gb_born(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, long long* gpol) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int ni = *v.nitems;
  for (int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < ni; it += nwarps) {
    bool two;
    const int t = item_tile(v, it, two);
    const Tile T = v.tiles[t];
    if (two) {
      const Tile U = v.tiles[t + 1];
      if (tile_full(T)) born_full2(v, k, T, U, lane, gpol);
      else born_tile2<false>(v, k, T, U, lane, gpol);
      continue;
    }
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    unsigned ex, m14;
    tile_masks(v, T, lane, ex, m14);
    if (T.flags & 2) ex |= diag_exclusion(lane);
    float gi = 0.f, gj = 0.f;
    const bool full = tile_full(T);
    if (tile_masked(T)) {
      if (full) born_tile<true, true>(v, k, T, lane, si, xi, pi, ex, gi, gj);
      else born_tile<true, false>(v, k, T, lane, si, xi, pi, ex, gi, gj);
    } else {
      if (full) born_tile<false, true>(v, k, T, lane, si, xi, pi, ex, gi, gj);
      else born_tile<false, false>(v, k, T, lane, si, xi, pi, ex, gi, gj);
    }
    fix_range(v.status, fabsf(gi) + fabsf(gj));
    atomic_add_ll(&gpol[si], fx32(gi));
    atomic_add_ll(&gpol[T.bj * 32 + lane], fx32(gj));
  }
}

// Born radii a = -halfeconv / (terms123 + sum) + BornRadiusOffset  (FP64)
__global__ void k_gb_radii(DevView v, const double* terms123, const long long* gpol, double halfeconv,
                           double offset, float* born_f, double* born_d) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  if (a < 0) {
    born_f[s] = 1.f;
    return;
  }
  double G = terms123[a] + (double)gpol[s] * (1.0 / kSumScale);
  double r = -halfeconv / G + offset;
  born_f[s] = (float)r;
  born_d[a] = r;
}

// the exp-approximation switch is discontinuous: pairs within FP32 rounding of
// the threshold are decided in FP64
__device__ __noinline__ bool gb_on_fp64(const DevView& v, int si, int sj, double thresh) {
  int a = v.sorted_atom[si], b = v.sorted_atom[sj];
  if (a < 0 || b < 0) return false;
  return -0.25 * r2_slots_fp64(v, si, sj) / (v.born[a] * v.born[b]) > thresh;
}

// ---------------------------------------------------------------------------
// pass 2: GB cross term fused with vacuum LJ + Coulomb, i > j pairs within Cutoff
// (forces, dE/da and, with ENERGY, the pair energies).  With ENERGY every pair
// closer than sqrt(GBConst::e64_r2) (4.5 A: the close contacts that carry the
// large repulsive terms) takes its displacement from FP64 slot records (rounded
// once to FP32 for the force) and its energies in FP64 from FP64 per-atom
// parameters; the other pairs' energies are FP32, in partial sums moved to FP64
// every 8 rotation steps; a work item's sums then go over the warp in FP64 and
// enter fixed point once.  The vdW total is a small difference of large
// repulsive and attractive sums: FP32 positions (rounded relative to their
// block centres) on the close contacts, or FP32 sums, leave ~1e-6 of it.
// Energy evaluations are rare (an exchange attempt, an explicit energy call),
// so this FP64 work stays off the force-only step; the energy pass of a
// parameter-gradient call sets e64_r2 = 0 (its energies only weight the loss).
// ---------------------------------------------------------------------------
struct PairAcc {
  float fx, fy, fz, da;
};

// FP64 records of every sorted slot for the energy pass (DevView::epos, epar)
__global__ void k_energy_records(DevView v, double4* epos, double2* epar) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  const int a = v.sorted_atom[s];
  if (a < 0) {
    epos[s] = make_double4(1e6, 1e6, 1e6, 0.0);
    epar[s] = make_double2(-1.0, 0.0);
    return;
  }
  epos[s] = make_double4(v.pos[3 * a], v.pos[3 * a + 1], v.pos[3 * a + 2], v.charge[a]);
  epar[s] = make_double2(v.radius[a], v.sqeps[a]);
}

// (ENERGY) pair energies of a work item: close pairs in FP64, the others in
// FP32 partial sums moved to FP64 every 8 rotation steps
struct EAcc {
  double v = 0.0, e = 0.0, p = 0.0;
  float fv = 0.f, fe = 0.f, fp = 0.f;
  __device__ __forceinline__ void flush() {
    v += (double)fv;
    e += (double)fe;
    p += (double)fp;
    fv = fe = fp = 0.f;
  }
};

// 1 / sqrt(x) in FP64 from the FP32 approximation and one Newton step
// (relative error ~1e-13), without the FP64 square-root sequence
__device__ __forceinline__ double rsqrt_fp64(double x) {
  const double y = (double)rsqrtf((float)x);
  return y * fma(-0.5 * x * y, y, 1.5);
}

// u = -r^2 / (4 a_i a_j) of a pair, and whether the pair may lie above the exp
// threshold (the FP64 tie-break band included): the warp votes on it, and the
// GB term's code runs only when some lane needs it (in the all-pairs case most
// warp steps have none)
__device__ __forceinline__ float gb_u(float r2, float ai, float aj) { return -0.25f * __fdividef(r2, ai * aj); }
__device__ __forceinline__ bool gb_maybe_on(const GBConst& k, float u) {
  return u >= k.thresh - 4e-6f * fabsf(k.thresh);
}

// One pair of the fused law: i = (xi.w, pix, piy, ai), j = (qj, pjx, pjy, aj),
// (dx, dy, dz) = x_j - x_i, u = gb_u.  Adds the force on i along d to I and its
// opposite to J, dE/da to both.  si, sj:
// slots for the FP64 threshold tie-break; any_gb: the warp's vote on
// gb_maybe_on (warp-uniform).  (ENERGY) pe: the pair's energies for
// add_pair_energy.
// (ENERGY) what a pair's energies need beyond r^2: its FP32 energies (vdW,
// Coulomb, GB cross term) and, for the FP64 path of a close pair, whether the
// GB term is on, fgb S, the Coulomb switch S and the vdW switch (0 beyond
// VdwCutoff)
struct PairE {
  float v, e, p, fgbS, S, vsw;
  bool gbon;
};

// FP64 energies of a close pair from the slot records (the caller enters this
// on a warp vote, so the FP64 code is not issued for warps without a close
// pair); returned, not accumulated, so the accumulators stay in registers
struct E3 {
  double v, e, p;
};
template <bool FAST>
__device__ __noinline__ E3 close_energy(const DevView& v, const GBConst& k, double r2d, double4 ei, double4 ej,
                                        double2 pi_e, int sj, bool excl, bool is14, PairE pe) {
  E3 r = {0.0, 0.0, 0.0};
  const double qq = ei.w * ej.w, ir = rsqrt_fp64(r2d);
  if (pe.gbon) r.p = 2.0 * k.premul_d * qq * (double)pe.fgbS;
  else if (!FAST) r.p = 2.0 * k.premul_d * qq * ir * (double)pe.S;
  if (FAST && !excl) {
    r.e = (pe.gbon ? k.econv_in_d : k.econv_out_d) * (is14 ? k.elec14_d : 1.0) * qq * ir * (double)pe.S;
    const double2 pj_e = v.epar[sj];
    const double sd = pi_e.x + pj_e.x, t2 = sd * sd * (ir * ir), B6 = t2 * t2 * t2;
    r.v = pi_e.y * pj_e.y * (is14 ? k.vdw14_d : 1.0) * (B6 * B6 - 2.0 * B6) * (double)pe.vsw;
  }
  return r;
}

// (ENERGY) a pair's energies into the item's sums: the FP64 path for a close
// pair (warp-voted; PRECISE passes only), the FP32 sums otherwise
template <bool FAST, bool PRECISE>
__device__ __forceinline__ void add_pair_energy(const DevView& v, const GBConst& k, bool in, bool close, double r2d,
                                                const double4& ei, const double4& ej, const double2& pi_e, int sj,
                                                bool excl, bool is14, const PairE& pe, EAcc& ea) {
  bool fp32 = in;
  if (PRECISE && __any_sync(0xffffffffu, in && close)) {
    if (in && close) {
      const E3 c = close_energy<FAST>(v, k, r2d, ei, ej, pi_e, sj, excl, is14, pe);
      ea.v += c.v;
      ea.e += c.e;
      ea.p += c.p;
      fp32 = false;
    }
  }
  if (fp32) {
    ea.fv += pe.v;
    ea.fe += pe.e;
    ea.fp += pe.p;
  }
}

template <bool ENERGY, bool FULL, bool FAST>
__device__ __forceinline__ void gb_pair_one(const DevView& v, const GBConst& k, float dx, float dy, float dz,
                                            float r2, float u, bool any_gb, float qi, float qj, float pix, float piy,
                                            float pjx, float pjy, float ai, float aj, bool excl, bool is14, int si,
                                            int sj, PairAcc& I, PairAcc& J, PairE& pe) {
    const float invr = rsqrtf(r2);
    const float r = r2 * invr;
    const float qiqj = qi * qj;
    const float aiaj = ai * aj;
    bool gbon = false;
    if (any_gb) {
      gbon = u > k.thresh;
      if (fabsf(u - k.thresh) <= 2e-6f * fabsf(k.thresh))
        gbon = gb_on_fp64(v, si, sj, k.thresh_d);
    }
    float g = 0.f;  // scalar multiplying (xj - xi) in the force on i
    float elec = 0.f, delec = 0.f;
    const float s14 = is14 ? k.elec14 : 1.f;
    // switching (FULL: the tile lies inside the inner cutoff) without a branch:
    // below the inner cutoff w = 0 gives S = 1 and dS = 0 exactly
    const bool sw_on = !FULL;
    float S = 1.f, dS = 0.f;
    if (sw_on) {
      const float w = fmaxf(r - k.inner, 0.f);
      const float sw = 1.f - w * w * k.invw2;
      dS = -4.f * k.invw2 * w * sw;
      S = sw * sw;
    }
    if (ENERGY) pe = PairE{0.f, 0.f, 0.f, 0.f, S, 0.f, any_gb && gbon};
    if (any_gb && gbon) {
      const float tg = __expf(u);
      const float fgb = rsqrtf(r2 + tg * aiaj);
      const float l = fgb * fgb;
      const float ep = k.premul * qiqj * fgb;
      float dedr = -ep * (r - 0.25f * r * tg) * l;
      float dalpha = -ep * tg * (1.f - u) * l;
      if (ENERGY) {
        pe.p = 2.f * ep * S;
        pe.fgbS = fgb * S;
      }
      if (FAST && !excl) {
        elec = k.econv_in * s14 * qiqj * invr;
        delec = -elec * invr;
      }
      if (sw_on) {
        dedr = S * dedr + dS * ep;
        dalpha *= S;
      }
      g += 2.f * dedr * invr;
      I.da += dalpha * aj;
      J.da += dalpha * ai;
    } else if (FAST && !excl) {
      elec = k.econv_out * s14 * qiqj * invr;
      delec = -elec * invr;
    } else if (!FAST) {
      // calcBornForces below the threshold (gbff.cpp:1308-1325): premul q_i q_j / r
      const float ep = k.premul * qiqj * invr;
      float dedr = -ep * invr;
      if (ENERGY) pe.p = 2.f * ep * S;
      if (sw_on) dedr = S * dedr + dS * ep;
      g += 2.f * dedr * invr;
    }
    if (FAST && !excl) {
      if (ENERGY) pe.e = elec * S;
      if (sw_on) delec = S * delec + elec * dS;
      const float t = (pix + pjx) * invr;
      float B = t * t;
      B = B * B * B;
      const float A = B * B;
      const float eps = piy * pjy * (is14 ? k.vdw14 : 1.f);
      float dvdw = -12.f * eps * invr * (A - B);
      float Ev = (ENERGY || !FULL) ? eps * (A - 2.f * B) : 0.f;
      float vsw = 1.f;
      if (!FULL) {
        const float w = fmaxf(r - k.vdwinner, 0.f);
        const float sw = 1.f - w * w * k.vdwinvw2;
        dvdw = sw * sw * dvdw + Ev * (-4.f * k.vdwinvw2 * w * sw);
        const bool vin = r < k.vdwcut;
        vsw = vin ? sw * sw : 0.f;
        dvdw = vin ? dvdw : 0.f;
      }
      if (ENERGY) {
        pe.v = Ev * vsw;
        pe.vsw = vsw;
      }
      g += (dvdw + delec) * invr;
    }
    I.fx += g * dx; I.fy += g * dy; I.fz += g * dz;
    J.fx -= g * dx; J.fy -= g * dy; J.fz -= g * dz;
}

// (ENERGY) for a pair closer than sqrt(k.e64_r2): the displacement x_b - x_a
// from the FP64 slot records (rounded once to FP32 for the force) and r^2 in
// FP64; false (nothing written) for a farther pair or a padding slot
__device__ __forceinline__ bool disp_fp64(const DevView& v, const GBConst& k, const double4& ea_, int sb, double4& eb,
                                          float& dx, float& dy, float& dz, float& r2, double& r2d) {
  if (!(r2 < k.e64_r2) || ea_.x > 1e5) return false;
  eb = v.epos[sb];
  if (eb.x > 1e5) return false;
  const double ex = eb.x - ea_.x, ey = eb.y - ea_.y, ez = eb.z - ea_.z;
  dx = (float)ex;
  dy = (float)ey;
  dz = (float)ez;
  r2d = ex * ex + ey * ey + ez * ez;
  r2 = (float)r2d;
  return true;
}

template <bool MASKED, bool ENERGY, bool FULL, bool FAST = true, bool PRECISE = true>
__device__ __forceinline__ void gb_pair_tile(const DevView& v, const GBConst& k, const Tile& T, int lane, int si,
                                             const float4& xi, const float4& pi, float ai, unsigned ex,
                                             unsigned m14, unsigned dmask, const float* born, PairAcc& I, PairAcc& J,
                                             EAcc& ea) {
  float4 xj = j_in_i_frame(v, T, lane);
  float4 pj = v.par[T.bj * 32 + lane];
  float aj = born[T.bj * 32 + lane];
  double4 e_i = make_double4(0.0, 0.0, 0.0, 0.0), e_j = e_i;
  double2 p_i = make_double2(0.0, 0.0);
  if (ENERGY && PRECISE) {
    e_i = v.epos[si];
    p_i = v.epar[si];
  }
#pragma unroll 2
  for (int kk = 0; kk < 32; kk++) {
    float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    float r2 = dx * dx + dy * dy + dz * dz;
    double r2d = 0.0;
    const bool close =
        ENERGY && PRECISE && disp_fp64(v, k, e_i, T.bj * 32 + ((lane + kk) & 31), e_j, dx, dy, dz, r2, r2d);
    bool pair = true, excl = false, is14 = false;
    if (MASKED) {
      pair = !((dmask >> kk) & 1u);
      excl = (ex >> kk) & 1u;  // bond order <= 2: GB term only
      is14 = (m14 >> kk) & 1u;
    }
    const bool in = (FULL || r2 <= k.cut2) && pair;
    const float u = gb_u(r2, ai, aj);
    const bool any_gb = __any_sync(0xffffffffu, in && gb_maybe_on(k, u));
    PairE pe;
    if (in)
      gb_pair_one<ENERGY, FULL, FAST>(v, k, dx, dy, dz, r2, u, any_gb, xi.w, xj.w, pi.x, pi.y, pj.x, pj.y, ai, aj,
                                      excl, is14, si, T.bj * 32 + ((lane + kk) & 31), I, J, pe);
    if (ENERGY)
      add_pair_energy<FAST, PRECISE>(v, k, in, close, r2d, e_i, e_j, p_i, T.bj * 32 + ((lane + kk) & 31), excl,
                                     is14, pe, ea);
    if (ENERGY && (kk & 7) == 7) ea.flush();
    ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(xj.w); ROT(pj.x); ROT(pj.y); ROT(aj);
    ROT(J.fx); ROT(J.fy); ROT(J.fz); ROT(J.da);
  }
}

// per-tile FP32 sums enter 64-bit fixed point before they are combined, so a
// slot's total does not depend on how its tiles were grouped into work items
struct FixAcc {
  long long fx, fy, fz, da;
};

__device__ __forceinline__ void fix_in(const DevView& v, FixAcc& F, const PairAcc& a) {
  fix_range(v.status, fabsf(a.fx) + fabsf(a.fy) + fabsf(a.fz) + fabsf(a.da));
  F.fx += fx32(a.fx);
  F.fy += fx32(a.fy);
  F.fz += fx32(a.fz);
  F.da += fx32(a.da);
}

__device__ __forceinline__ void flush_fix(const DevView& v, long long* deda, int s, const FixAcc& F) {
  atomic_add_ll(&v.facc[3 * s], F.fx);
  atomic_add_ll(&v.facc[3 * s + 1], F.fy);
  atomic_add_ll(&v.facc[3 * s + 2], F.fz);
  if (deda) atomic_add_ll(&deda[s], F.da);
}

__device__ __forceinline__ void flush_pair(const DevView& v, long long* deda, int s, const PairAcc& a) {
  FixAcc F = {0, 0, 0, 0};
  fix_in(v, F, a);
  flush_fix(v, deda, s, F);
}

__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// (ENERGY) a work item's pair energies: summed over the warp in FP64 (a fixed
// butterfly order), entered in fixed point once per item
__device__ __forceinline__ void flush_gb_energy(const DevView& v, int lane, int bi, EAcc& ea) {
  ea.flush();
  const double e0 = warp_sum_d(ea.v), e1 = warp_sum_d(ea.e), e2 = warp_sum_d(ea.p);
  if (lane == 0) {
    long long* E = v.eacc + (size_t)v.slot_sys[bi] * E_NSLOTS;
    atomic_add_ll(&E[E_VDW], fix_energy_d(e0));
    atomic_add_ll(&E[E_ELEC], fix_energy_d(e1));
    atomic_add_ll(&E[E_POL_CROSS], fix_energy_d(e2));
  }
}

template <bool ENERGY, bool FULL, bool PRECISE = true>
__device__ __forceinline__ void gb_pair_tile2(const DevView& v, const GBConst& k, const Tile& A, const Tile& B,
                                              int lane, const float* born, long long* deda, EAcc& ea) {
  const int sa = A.bj * 32 + lane, sb = B.bj * 32 + lane, r0 = A.bi * 32;
  const float4 xa = j_in_i_frame(v, A, lane), xb = j_in_i_frame(v, B, lane);
  const float4 pa = v.par[sa], pb = v.par[sb];
  const float aa = born[sa], ab = born[sb];
  float4 xr = v.xq[r0 + lane], pr = v.par[r0 + lane];
  float ar = born[r0 + lane];
  double4 e_a = make_double4(0.0, 0.0, 0.0, 0.0), e_b = e_a, e_r = e_a;
  double2 p_a = make_double2(0.0, 0.0), p_b = p_a;
  if (ENERGY && PRECISE) {
    e_a = v.epos[sa];
    e_b = v.epos[sb];
    p_a = v.epar[sa];
    p_b = v.epar[sb];
  }
  PairAcc IA = {0.f, 0.f, 0.f, 0.f}, IB = {0.f, 0.f, 0.f, 0.f}, R = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
  for (int kk = 0; kk < 32; kk++) {
    const int sr = r0 + ((lane + kk) & 31);
    {
      float dx = xr.x - xa.x, dy = xr.y - xa.y, dz = xr.z - xa.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      double r2d = 0.0;
      const bool close = ENERGY && PRECISE && disp_fp64(v, k, e_a, sr, e_r, dx, dy, dz, r2, r2d);
      const bool in = FULL || r2 <= k.cut2;
      const float u = gb_u(r2, aa, ar);
      const bool any_gb = __any_sync(0xffffffffu, in && gb_maybe_on(k, u));
      PairE pe;
      if (in)
        gb_pair_one<ENERGY, FULL, true>(v, k, dx, dy, dz, r2, u, any_gb, xa.w, xr.w, pa.x, pa.y, pr.x, pr.y, aa, ar,
                                        false, false, sa, sr, IA, R, pe);
      if (ENERGY) add_pair_energy<true, PRECISE>(v, k, in, close, r2d, e_a, e_r, p_a, sr, false, false, pe, ea);
    }
    {
      float dx = xr.x - xb.x, dy = xr.y - xb.y, dz = xr.z - xb.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      double r2d = 0.0;
      const bool close = ENERGY && PRECISE && disp_fp64(v, k, e_b, sr, e_r, dx, dy, dz, r2, r2d);
      const bool in = FULL || r2 <= k.cut2;
      const float u = gb_u(r2, ab, ar);
      const bool any_gb = __any_sync(0xffffffffu, in && gb_maybe_on(k, u));
      PairE pe;
      if (in)
        gb_pair_one<ENERGY, FULL, true>(v, k, dx, dy, dz, r2, u, any_gb, xb.w, xr.w, pb.x, pb.y, pr.x, pr.y, ab, ar,
                                        false, false, sb, sr, IB, R, pe);
      if (ENERGY) add_pair_energy<true, PRECISE>(v, k, in, close, r2d, e_b, e_r, p_b, sr, false, false, pe, ea);
    }
    if (ENERGY && (kk & 7) == 7) ea.flush();
    ROT(xr.x); ROT(xr.y); ROT(xr.z); ROT(xr.w); ROT(pr.x); ROT(pr.y); ROT(ar);
    ROT(R.fx); ROT(R.fy); ROT(R.fz); ROT(R.da);
  }
  flush_pair(v, deda, sa, IA);
  flush_pair(v, deda, sb, IB);
  flush_pair(v, deda, r0 + lane, R);
}

// The GB cross term of an all-inside pair the threshold test may switch on:
// the exact decision (FP64 within rounding of the threshold, as gb_pair_one)
// and, above it, the GB term (gbff.cpp:1592-1678) with Coulomb at eps_in in
// place of eps_out.  akh, akr: Born radii times sqrtK; e1: the pair's eps_out
// Coulomb energy; ir = 1/r.  Returns what the pair adds to dE/dr / r and to
// the two atoms' dE/da.  Inlined under the caller's warp vote: a call (the
// accumulators saved around it) or outputs through references (accumulators
// kept in local memory) both cost more than the registers it adds.
struct GBTerm {
  float g, dah, dar;
};
__device__ __forceinline__ GBTerm gb_full_term(const DevView& v, const GBConst& k, float r2, float ir, float e1,
                                               float akh, float akr, int sh, int sr) {
  GBTerm t = {0.f, 0.f, 0.f};
  const float ah = akh * k.inv_sqrtK, ar = akr * k.inv_sqrtK;
  const float aiaj = ah * ar;
  const float u = -0.25f * __fdividef(r2, aiaj);
  bool on = u > k.thresh;
  if (fabsf(u - k.thresh) <= 2e-6f * fabsf(k.thresh)) on = gb_on_fp64(v, sh, sr, k.thresh_d);
  if (!on) return t;
  const float r = r2 * ir;
  const float qq = e1 * r * k.inv_eout;
  const float tg = __expf(u);
  const float fgb = rsqrtf(fmaf(tg, aiaj, r2));
  const float l = fgb * fgb;
  const float ep = k.premul * qq * fgb;
  const float dedr = -ep * (r - 0.25f * r * tg) * l;
  const float dalpha = -ep * tg * (1.f - u) * l;
  t.g = 2.f * dedr * ir - k.in_over_out_m1 * e1 * ir * ir;
  t.dah = dalpha * ar;
  t.dar = dalpha * ah;
  return t;
}

// Force-only GB fused pair of an all-inside tile pair (the dynamics step's
// body), the two held atoms on packed FP32x2 arithmetic.  Common pair: vacuum
// LJ + Coulomb at eps_out,  dE/dr / r = -(12 eps (A - B) + E_out) / r^2,  with
// the held atoms' charges scaled by -sqrt(econv_out) and sqrt(eps) by
// -sqrt(12) (the rotating atom's by the positive factors), so one FFMA forms
// the bracket with its sign.  A pair with r^2 <= K a_i a_j may lie above the
// exp threshold; when any lane has one, gb_full_term runs for those pairs.
__device__ __forceinline__ void gb_pair_full2(const DevView& v, const GBConst& k, const Tile& A, const Tile& B,
                                              int lane, const float* born, long long* deda) {
  const int sa = A.bj * 32 + lane, sb = B.bj * 32 + lane, r0 = A.bi * 32;
  const float4 xa = j_in_i_frame(v, A, lane), xb = j_in_i_frame(v, B, lane);
  const float4 pa = v.par[sa], pb = v.par[sb];
  const float2 nx = make_float2(-xa.x, -xb.x), ny = make_float2(-xa.y, -xb.y), nz = make_float2(-xa.z, -xb.z);
  const float2 QN = make_float2(-k.sq_eout * xa.w, -k.sq_eout * xb.w);
  const float2 S = make_float2(pa.x, pb.x);
  const float2 EN = make_float2(-k.sqrt12 * pa.y, -k.sqrt12 * pb.y);
  const float2 AK = make_float2(k.sqrtK * born[sa], k.sqrtK * born[sb]);
  const float2 M1 = f2(-1.f);
  float4 xr = v.xq[r0 + lane];
  const float4 pr = v.par[r0 + lane];
  float qr = k.sq_eout * xr.w, sgr = pr.x, er = k.sqrt12 * pr.y, akr = k.sqrtK * born[r0 + lane];
  float2 FX = f2(0.f), FY = f2(0.f), FZ = f2(0.f), DA = f2(0.f);
  PairAcc R = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
  for (int kk = 0; kk < 32; kk++) {
    const float2 dx = __fadd2_rn(f2(xr.x), nx), dy = __fadd2_rn(f2(xr.y), ny), dz = __fadd2_rn(f2(xr.z), nz);
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 lim = __fmul2_rn(AK, f2(akr));
    const bool na = r2.x <= lim.x, nb = r2.y <= lim.y;
    const float2 ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
    const float2 ir2 = __fmul2_rn(ir, ir);
    const float2 e1n = __fmul2_rn(__fmul2_rn(QN, f2(qr)), ir);   // -E_out
    const float2 s = __fadd2_rn(S, f2(sgr));
    const float2 t2 = __fmul2_rn(__fmul2_rn(s, s), ir2);
    const float2 b6 = __fmul2_rn(__fmul2_rn(t2, t2), t2);
    const float2 amb = __ffma2_rn(b6, b6, __fmul2_rn(b6, M1));    // A - B
    float2 g = __fmul2_rn(__ffma2_rn(__fmul2_rn(EN, f2(er)), amb, e1n), ir2);
    if (__any_sync(0xffffffffu, na || nb)) {
      const int sr = r0 + ((lane + kk) & 31);
      if (na) {
        const GBTerm t = gb_full_term(v, k, r2.x, ir.x, -e1n.x, AK.x, akr, sa, sr);
        g.x += t.g;
        DA.x += t.dah;
        R.da += t.dar;
      }
      if (nb) {
        const GBTerm t = gb_full_term(v, k, r2.y, ir.y, -e1n.y, AK.y, akr, sb, sr);
        g.y += t.g;
        DA.y += t.dah;
        R.da += t.dar;
      }
    }
    FX = __ffma2_rn(g, dx, FX);
    FY = __ffma2_rn(g, dy, FY);
    FZ = __ffma2_rn(g, dz, FZ);
    R.fx = fmaf(-g.x, dx.x, R.fx); R.fx = fmaf(-g.y, dx.y, R.fx);
    R.fy = fmaf(-g.x, dy.x, R.fy); R.fy = fmaf(-g.y, dy.y, R.fy);
    R.fz = fmaf(-g.x, dz.x, R.fz); R.fz = fmaf(-g.y, dz.y, R.fz);
    ROT(xr.x); ROT(xr.y); ROT(xr.z); ROT(qr); ROT(sgr); ROT(er); ROT(akr);
    ROT(R.fx); ROT(R.fy); ROT(R.fz); ROT(R.da);
  }
  flush_pair(v, deda, sa, PairAcc{FX.x, FY.x, FZ.x, DA.x});
  flush_pair(v, deda, sb, PairAcc{FX.y, FY.y, FZ.y, DA.y});
  flush_pair(v, deda, r0 + lane, R);
}

// EMODE 0: forces and dE/da only; 1: with energies (close pairs in FP64);
// 2: with energies from FP32 pair terms (a gradient call's energy pass)
template <int EMODE>
__device__ __forceinline__ void gb_pair_items(const DevView& v, const GBConst& k, const float* born, long long* deda) {
  constexpr bool ENERGY = EMODE != 0, PRECISE = EMODE == 1;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int ni = *v.nitems;
  for (int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < ni; it += nwarps) {
    bool two;
    const int t = item_tile(v, it, two);
    const Tile T = v.tiles[t];
    if (two) {
      const Tile U = v.tiles[t + 1];
      EAcc ea;
      if (tile_full(T)) {
        if (ENERGY) gb_pair_tile2<true, true, PRECISE>(v, k, T, U, lane, born, deda, ea);
        else gb_pair_full2(v, k, T, U, lane, born, deda);
      }
      else gb_pair_tile2<ENERGY, false, PRECISE>(v, k, T, U, lane, born, deda, ea);
      if (ENERGY) flush_gb_energy(v, lane, T.bi, ea);
      continue;
    }
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    const float ai = born[si];
    unsigned ex, m14;
    tile_masks(v, T, lane, ex, m14);
    const unsigned dmask = (T.flags & 2) ? diag_exclusion(lane) : 0u;
    PairAcc I = {0.f, 0.f, 0.f, 0.f}, J = {0.f, 0.f, 0.f, 0.f};
    EAcc ea;
    const bool full = tile_full(T);
    if (tile_masked(T)) {
      if (full)
        gb_pair_tile<true, ENERGY, true, true, PRECISE>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J,
                                                         ea);
      else
        gb_pair_tile<true, ENERGY, false, true, PRECISE>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J,
                                                         ea);
    } else {
      if (full)
        gb_pair_tile<false, ENERGY, true, true, PRECISE>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J,
                                                         ea);
      else
        gb_pair_tile<false, ENERGY, false, true, PRECISE>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J,
                                                         ea);
    }
    flush_pair(v, deda, si, I);
    flush_pair(v, deda, T.bj * 32 + lane, J);
    if (ENERGY) flush_gb_energy(v, lane, T.bi, ea);
  }
}

// the force-only pass (every dynamics step) runs in CTAs of 128 threads, seven
// per SM (28 warps at 72 registers; 3 CTAs of 256 hold 24 at 80), launched as
// twice the tile kernels' CTA count; the energy pass carries FP64 records of
// its close pairs and gets more registers
__global__ void __launch_bounds__(128, 7) k_gb_pair(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* born, long long* deda) {
  gb_pair_items<0>(v, k, born, deda);
}
__global__ void __launch_bounds__(256, 2) k_gb_pair_energy(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* born,
                                                           long long* deda) {
  gb_pair_items<1>(v, k, born, deda);
}
__global__ void __launch_bounds__(256, 3) k_gb_pair_energy32(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* born,
                                                             long long* deda) {
  gb_pair_items<2>(v, k, born, deda);
}

// FastMode off (calcBornForces, gbff.cpp:1189-1340): the GB term of every pair
// within Cutoff, premul q_i q_j / r below the threshold; LJ and Coulomb come from
// the NB kernel with the GB object's own FF_NonBonded settings.  One masked body
// serves every tile: this mode exists for parity with PD, not for speed.
template <bool ENERGY>
__global__ void __launch_bounds__(256) k_gb_pair_born_only(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* born,
                                                           long long* deda) {
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
    PairAcc I = {0.f, 0.f, 0.f, 0.f}, J = {0.f, 0.f, 0.f, 0.f};
    EAcc ea;
    gb_pair_tile<true, ENERGY, false, false>(v, k, T, lane, si, xi, pi, ai, ex, m14, dmask, born, I, J, ea);
    flush_pair(v, deda, si, I);
    flush_pair(v, deda, T.bj * 32 + lane, J);
    if (ENERGY) flush_gb_energy(v, lane, T.bi, ea);
  }
}

// self term, total dE/da and the chain-rule prefactor a^2/166 * dE/da * P4
__global__ void k_gb_self(DevView v, const double* charge, GBConst k, double premul, const long long* deda,
                          const double* born_d, float* chain, int energy) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  long long e = 0;
  if (s < v.nslots) {  // nslots is a multiple of 32: warps are whole
    const int a = v.sorted_atom[s];
    if (a < 0) {
      chain[s] = 0.f;
    } else {
      const double ai = born_d[a], q = charge[a];
      const double inv = 1.0 / ai;
      const double self = premul * q * q * inv;
      const double da = (double)deda[s] * (1.0 / kSumScale) - self * inv;
      chain[s] = (float)(ai * ai * (1.0 / 166.0) * da * (double)k.P4);
      if (energy) e = fix_energy_d(self);
    }
  }
  if (energy) {  // a warp's slots are one block of one system: one atomic per warp
    e = warp_sum_ll(e);
    if ((threadIdx.x & 31) == 0 && s < v.nslots)
      atomic_add_ll(&v.eacc[(size_t)v.slot_sys[s >> 5] * E_NSLOTS + E_POL_SELF], e);
  }
}

// ---------------------------------------------------------------------------
// pass 3: dE/da chain rule through the Born radii, both directions of a pair
// ---------------------------------------------------------------------------
// (c_i V_j + c_j V_i) (4 CCF - dCCF) / r^6 of one pair: the chain-rule force per unit d
__device__ __forceinline__ float chain_w(const GBConst& k, float r2, float rs, float cv, bool any_contact) {
  const float rs2 = rs * rs;
  float ccf = 1.f, dccf = 0.f;
  if (any_contact) {
    if (gb_contact(k, r2, rs2)) {
      float sn, cs;
      const float x = __fdividef(r2, rs2) * k.P5;
      sincospif(x, &sn, &cs);
      const float h = 0.5f - 0.5f * cs;
      ccf = h * h;
      dccf = 2.f * h * sn * (x * 3.14159265358979f);
    }
  }
  const float ir2 = rcp_ftz(r2);
  return cv * (4.f * ccf - dccf) * ir2 * ir2 * ir2;
}

template <bool MASKED, bool FULL>
__device__ __forceinline__ void chain_tile(const DevView& v, const GBConst& k, const Tile& T, int lane, int si,
                                           const float4& xi, const float4& pi, float ci, unsigned ex,
                                           const float* chain, PairAcc& I, PairAcc& J) {
  float4 xj = j_in_i_frame(v, T, lane);
  float4 pj = v.par[T.bj * 32 + lane];
  float cj = chain[T.bj * 32 + lane];
#pragma unroll 4
  for (int kk = 0; kk < 32; kk++) {
    const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
    const float r2 = dx * dx + dy * dy + dz * dz;
    bool in = still_in<FULL>(v, k, r2, si, T.bj * 32 + ((lane + kk) & 31));
    if (MASKED) in = in && !((ex >> kk) & 1u);
    const float rs = pi.z + pj.z;
    const bool anyc = __any_sync(0xffffffffu, in && gb_contact(k, r2, rs * rs));
    if (in) {
      const float w = chain_w(k, r2, rs, ci * pj.w + cj * pi.w, anyc);
      I.fx -= w * dx; I.fy -= w * dy; I.fz -= w * dz;
      J.fx += w * dx; J.fy += w * dy; J.fz += w * dz;
    }
    ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(pj.z); ROT(pj.w); ROT(cj); ROT(J.fx); ROT(J.fy); ROT(J.fz);
  }
}

__device__ __forceinline__ void flush_force(const DevView& v, int s, const PairAcc& a) {
  FixAcc F = {0, 0, 0, 0};
  fix_in(v, F, a);
  flush_fix(v, nullptr, s, F);
}

template <bool FULL>
__device__ __forceinline__ void chain_tile2(const DevView& v, const GBConst& k, const Tile& A, const Tile& B, int lane,
                                            const float* chain) {
  const int sa = A.bj * 32 + lane, sb = B.bj * 32 + lane, r0 = A.bi * 32;
  const float4 xa = j_in_i_frame(v, A, lane), xb = j_in_i_frame(v, B, lane);
  const float4 pa = v.par[sa], pb = v.par[sb];
  const float2 nx = make_float2(-xa.x, -xb.x), ny = make_float2(-xa.y, -xb.y), nz = make_float2(-xa.z, -xb.z);
  const float2 RS = make_float2(pa.z, pb.z), VS = make_float2(pa.w, pb.w);
  const float2 CS = make_float2(chain[sa], chain[sb]);
  float4 xr = v.xq[r0 + lane], pr = v.par[r0 + lane];
  float cr = chain[r0 + lane];
  float2 FX = f2(0.f), FY = f2(0.f), FZ = f2(0.f);  // the two j atoms' sums
  PairAcc FR = {0.f, 0.f, 0.f, 0.f};               // the rotating atom's sums
#pragma unroll 4
  for (int kk = 0; kk < 32; kk++) {
    const int sr = r0 + ((lane + kk) & 31);
    const float2 dx = __fadd2_rn(f2(xr.x), nx), dy = __fadd2_rn(f2(xr.y), ny), dz = __fadd2_rn(f2(xr.z), nz);
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 rs = __fadd2_rn(RS, f2(pr.z));
    const float2 rs2 = __fmul2_rn(rs, rs);
    const float2 lim = __fmul2_rn(rs2, f2(k.invP5));
    const bool ca = r2.x <= lim.x, cb = r2.y <= lim.y;
    float2 fac = f2(4.f);  // 4 CCF - dCCF
    if (__any_sync(0xffffffffu, ca || cb)) {
      if (ca) {
        float sn, cs;
        const float x = __fdividef(r2.x, rs2.x) * k.P5;
        sincospif(x, &sn, &cs);
        const float h = 0.5f - 0.5f * cs;
        fac.x = 4.f * h * h - 2.f * h * sn * (x * 3.14159265358979f);
      }
      if (cb) {
        float sn, cs;
        const float x = __fdividef(r2.y, rs2.y) * k.P5;
        sincospif(x, &sn, &cs);
        const float h = 0.5f - 0.5f * cs;
        fac.y = 4.f * h * h - 2.f * h * sn * (x * 3.14159265358979f);
      }
    }
    const float2 ir2 = make_float2(rcp_ftz(r2.x), rcp_ftz(r2.y));
    const float2 cvv = __ffma2_rn(CS, f2(pr.w), __fmul2_rn(f2(cr), VS));
    float2 w = __fmul2_rn(__fmul2_rn(cvv, fac), __fmul2_rn(__fmul2_rn(ir2, ir2), ir2));
    if (!FULL) {
      if (!still_in<false>(v, k, r2.x, sa, sr)) w.x = 0.f;
      if (!still_in<false>(v, k, r2.y, sb, sr)) w.y = 0.f;
    }
    const float2 nw = __fmul2_rn(w, f2(-1.f));
    FX = __ffma2_rn(nw, dx, FX);
    FY = __ffma2_rn(nw, dy, FY);
    FZ = __ffma2_rn(nw, dz, FZ);
    FR.fx = fmaf(w.x, dx.x, FR.fx); FR.fx = fmaf(w.y, dx.y, FR.fx);
    FR.fy = fmaf(w.x, dy.x, FR.fy); FR.fy = fmaf(w.y, dy.y, FR.fy);
    FR.fz = fmaf(w.x, dz.x, FR.fz); FR.fz = fmaf(w.y, dz.y, FR.fz);
    ROT(xr.x); ROT(xr.y); ROT(xr.z); ROT(pr.z); ROT(pr.w); ROT(cr); ROT(FR.fx); ROT(FR.fy); ROT(FR.fz);
  }
  flush_force(v, sa, PairAcc{FX.x, FY.x, FZ.x, 0.f});
  flush_force(v, sb, PairAcc{FX.y, FY.y, FZ.y, 0.f});
  flush_force(v, r0 + lane, FR);
}

// 0.25 (4 CCF - dCCF) of a pair in close contact, 1 otherwise
__device__ __forceinline__ float chain_fac(const GBConst& k, float r2, float rs) {
  const float rs2 = rs * rs;
  if (!gb_contact(k, r2, rs2)) return 1.f;
  float sn, cs;
  const float x = __fdividef(r2, rs2) * k.P5;
  sincospif(x, &sn, &cs);
  const float h = 0.5f - 0.5f * cs;
  return 0.25f * (4.f * h * h - 2.f * h * sn * (x * 3.14159265358979f));
}

// CTAs of 128 threads, seven per SM (28 warps at 72 registers)
constexpr int kChainThreads = 128;
constexpr int kChainWarps = kChainThreads / 32;

// Born chain rule of an all-inside tile pair, step-packed: (c_i V_j + c_j V_i)
// (4 CCF - dCCF) / r^6 along d, with -4 folded into c (w then carries the held
// atom's sign and the factor 4 of the no-contact case); the CCF branch on the
// coarse-bound vote.
__device__ __forceinline__ void chain_full2(const DevView& v, const GBConst& k, const Tile& A, const Tile& B, int lane,
                                            const float* chain) {
  __shared__ float4 rot_sh[kChainWarps][3][32];   // (x, x', y, y'), (z, z', V, V'), (c, c')
  float4 (*rs)[32] = rot_sh[threadIdx.x >> 5];
  const int sa = A.bj * 32 + lane, sb = B.bj * 32 + lane, r0 = A.bi * 32;
  const int l1 = (lane + 1) & 31;
  const float4 xa = j_in_i_frame(v, A, lane), xb = j_in_i_frame(v, B, lane);
  const float4 pa = v.par[sa], pb = v.par[sb];
  const float2 AX = f2(-xa.x), AY = f2(-xa.y), AZ = f2(-xa.z), BX = f2(-xb.x), BY = f2(-xb.y), BZ = f2(-xb.z);
  const float2 VA = f2(pa.w), VB = f2(pb.w), CA = f2(-4.f * chain[sa]), CB = f2(-4.f * chain[sb]);
  float c2;
  {
    const float4 x0 = v.xq[r0 + lane], p0 = v.par[r0 + lane];
    const float c0 = -4.f * chain[r0 + lane];
    const float x1 = __shfl_sync(0xffffffffu, x0.x, l1), y1 = __shfl_sync(0xffffffffu, x0.y, l1);
    const float z1 = __shfl_sync(0xffffffffu, x0.z, l1), v1 = __shfl_sync(0xffffffffu, p0.w, l1);
    const float c1 = __shfl_sync(0xffffffffu, c0, l1);
    c2 = pair_contact2(k, make_float2(pa.z, pb.z), p0.z);
    __syncwarp();
    rs[0][lane] = make_float4(x0.x, x1, x0.y, y1);
    rs[1][lane] = make_float4(x0.z, z1, p0.w, v1);
    rs[2][lane] = make_float4(c0, c1, 0.f, 0.f);
    __syncwarp();
  }
  float2 FAX = f2(0.f), FAY = f2(0.f), FAZ = f2(0.f), FBX = f2(0.f), FBY = f2(0.f), FBZ = f2(0.f);
  float2 FRX = f2(0.f), FRY = f2(0.f), FRZ = f2(0.f);   // minus the rotating atoms' sums
#pragma unroll 1
  for (int kk = 0; kk < 32; kk += 2) {
    const int j = (lane + kk) & 31;
    const float4 P = rs[0][j], Q = rs[1][j];
    const float2 CR = *reinterpret_cast<const float2*>(&rs[2][j]);
    const float2 X = make_float2(P.x, P.y), Y = make_float2(P.z, P.w), Z = make_float2(Q.x, Q.y);
    const float2 VR = make_float2(Q.z, Q.w);
    const float2 ax = __fadd2_rn(X, AX), ay = __fadd2_rn(Y, AY), az = __fadd2_rn(Z, AZ);
    const float2 bx = __fadd2_rn(X, BX), by = __fadd2_rn(Y, BY), bz = __fadd2_rn(Z, BZ);
    const float2 ra = __ffma2_rn(az, az, __ffma2_rn(ay, ay, __fmul2_rn(ax, ax)));
    const float2 rb = __ffma2_rn(bz, bz, __ffma2_rn(by, by, __fmul2_rn(bx, bx)));
    const float2 ia = make_float2(rcp_ftz(ra.x), rcp_ftz(ra.y));
    const float2 ib = make_float2(rcp_ftz(rb.x), rcp_ftz(rb.y));
    // -w of the plain law: (c_held V_rot + c_rot V_held) (-4) / r^6
    float2 wa = __fmul2_rn(__ffma2_rn(CA, VR, __fmul2_rn(CR, VA)), __fmul2_rn(__fmul2_rn(ia, ia), ia));
    float2 wb = __fmul2_rn(__ffma2_rn(CB, VR, __fmul2_rn(CR, VB)), __fmul2_rn(__fmul2_rn(ib, ib), ib));
    if (__any_sync(0xffffffffu, fminf(fminf(ra.x, ra.y), fminf(rb.x, rb.y)) <= c2)) {
      // rare: the rotating atoms' radii are read here, not staged
      const float R0 = v.par[r0 + j].z, R1 = v.par[r0 + ((j + 1) & 31)].z;
      wa.x *= chain_fac(k, ra.x, pa.z + R0);
      wa.y *= chain_fac(k, ra.y, pa.z + R1);
      wb.x *= chain_fac(k, rb.x, pb.z + R0);
      wb.y *= chain_fac(k, rb.y, pb.z + R1);
    }
    FAX = __ffma2_rn(wa, ax, FAX); FAY = __ffma2_rn(wa, ay, FAY); FAZ = __ffma2_rn(wa, az, FAZ);
    FBX = __ffma2_rn(wb, bx, FBX); FBY = __ffma2_rn(wb, by, FBY); FBZ = __ffma2_rn(wb, bz, FBZ);
    FRX = __ffma2_rn(wa, ax, __ffma2_rn(wb, bx, FRX));
    FRY = __ffma2_rn(wa, ay, __ffma2_rn(wb, by, FRY));
    FRZ = __ffma2_rn(wa, az, __ffma2_rn(wb, bz, FRZ));
    ROT2(FRX); ROT2(FRY); ROT2(FRZ);
  }
  const int lm = (lane + 31) & 31;
  const float frx = FRX.x + __shfl_sync(0xffffffffu, FRX.y, lm);
  const float fry = FRY.x + __shfl_sync(0xffffffffu, FRY.y, lm);
  const float frz = FRZ.x + __shfl_sync(0xffffffffu, FRZ.y, lm);
  flush_force(v, sa, PairAcc{FAX.x + FAX.y, FAY.x + FAY.y, FAZ.x + FAZ.y, 0.f});
  flush_force(v, sb, PairAcc{FBX.x + FBX.y, FBY.x + FBY.y, FBZ.x + FBZ.y, 0.f});
  flush_force(v, r0 + lane, PairAcc{-frx, -fry, -frz, 0.f});
}

__global__ void __launch_bounds__(kChainThreads, 7) k_gb_chain(const __grid_constant__ DevView v, const __grid_constant__ GBConst k, const float* chain) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int ni = *v.nitems;
  for (int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < ni; it += nwarps) {
    bool two;
    const int t = item_tile(v, it, two);
    const Tile T = v.tiles[t];
    if (two) {
      const Tile U = v.tiles[t + 1];
      if (tile_full(T)) chain_full2(v, k, T, U, lane, chain);
      else chain_tile2<false>(v, k, T, U, lane, chain);
      continue;
    }
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    const float ci = chain[si];
    unsigned ex, m14;
    tile_masks(v, T, lane, ex, m14);
    if (T.flags & 2) ex |= diag_exclusion(lane);
    PairAcc I = {0.f, 0.f, 0.f, 0.f}, J = {0.f, 0.f, 0.f, 0.f};
    const bool full = tile_full(T);
    if (tile_masked(T)) {
      if (full) chain_tile<true, true>(v, k, T, lane, si, xi, pi, ci, ex, chain, I, J);
      else chain_tile<true, false>(v, k, T, lane, si, xi, pi, ci, ex, chain, I, J);
    } else {
      if (full) chain_tile<false, true>(v, k, T, lane, si, xi, pi, ci, ex, chain, I, J);
      else chain_tile<false, false>(v, k, T, lane, si, xi, pi, ci, ex, chain, I, J);
    }
    flush_force(v, si, I);
    flush_force(v, T.bj * 32 + lane, J);
  }
}

int tile_grid(Context& c) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
  long long want = (c.tile_cap + 7) / 8;
  long long g = (long long)sms * c.tile_ctas_per_sm;
  return (int)(want < g ? (want > 0 ? want : 1) : g);
}

int launch_gb(Context& c, const GBConst& k, double halfeconv, double born_offset, double premul, bool energy) {
  c.kernel_launches += 5;
  DevView v = c.view();
  cudaStream_t st = c.stream;
  int g = tile_grid(c);
  int nb = (c.nslots + 255) / 256;
  cudaMemsetAsync(c.d_gpol.p, 0, sizeof(long long) * c.nslots, st);
  cudaMemsetAsync(c.d_deda.p, 0, sizeof(long long) * c.nslots, st);
  k_gb_born<<<g, kBornThreads, 0, st>>>(v, k, c.d_gpol.p);
  k_gb_radii<<<nb, 256, 0, st>>>(v, c.d_gbT.p, c.d_gpol.p, halfeconv, born_offset, c.d_born_f.p, c.d_born_d.p);
  GBConst ke = k;
  if (c.gb_no_chain) ke.e64_r2 = 0.f;  // a gradient call's energy pass: FP32 pair energies
  if (energy && ke.e64_r2 > 0.f) {
    c.kernel_launches += 1;
    k_energy_records<<<nb, 256, 0, st>>>(v, c.d_epos.p, c.d_epar.p);
  }
  if (!k.fast) {
    if (energy) k_gb_pair_born_only<true><<<g, 256, 0, st>>>(v, k, c.d_born_f.p, c.d_deda.p);
    else k_gb_pair_born_only<false><<<g, 256, 0, st>>>(v, k, c.d_born_f.p, c.d_deda.p);
  } else if (energy) {
    if (ke.e64_r2 > 0.f) k_gb_pair_energy<<<g, 256, 0, st>>>(v, ke, c.d_born_f.p, c.d_deda.p);
    else k_gb_pair_energy32<<<g, 256, 0, st>>>(v, ke, c.d_born_f.p, c.d_deda.p);
  } else {
    k_gb_pair<<<2 * g, 128, 0, st>>>(v, k, c.d_born_f.p, c.d_deda.p);
  }
  k_gb_self<<<nb, 256, 0, st>>>(v, c.d_charge.p, k, premul, c.d_deda.p, c.d_born_d.p, c.d_chain_f.p,
                                energy ? 1 : 0);
  if (c.gb_no_chain) c.kernel_launches -= 1;
  else k_gb_chain<<<2 * g, kChainThreads, 0, st>>>(v, k, c.d_chain_f.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

// one GB pass on its own (timing probe): 1 Born sums, 2 fused pair (forces), 3 chain rule
int launch_gb_stage(Context& c, const GBConst& k, int stage) {
  DevView v = c.view();
  int g = tile_grid(c);
  c.kernel_launches += 1;
  if (stage == 1) k_gb_born<<<g, kBornThreads, 0, c.stream>>>(v, k, c.d_gpol.p);
  else if (stage == 2) k_gb_pair<<<2 * g, 128, 0, c.stream>>>(v, k, c.d_born_f.p, c.d_deda.p);
  else k_gb_chain<<<2 * g, kChainThreads, 0, c.stream>>>(v, k, c.d_chain_f.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
