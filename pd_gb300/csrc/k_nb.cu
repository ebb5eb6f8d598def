// k_nb.cu — LJ + Coulomb tile kernel (FF_NonBonded) and force finalisation.
//
// Pair law: PD src/mmlib/forcefields/nonbonded.cpp:687-833
//   (T_fast2 instantiation with VdwMode = EnergySwitch and ElecMode picked by
//    the dispatch at nonbonded.cpp:1222-1246).
// Every listed pair j < i inside Cutoff contributes once; bond order <= 2
// pairs are zero, 1-4 pairs are scaled by Vdw14Scaling / Elec14Scaling.
#include "pdgpu_tile.cuh"

namespace pdgpu {

// the pair decision for pairs whose FP32 distance lies at a hard cutoff
__device__ __noinline__ double nb_r2_fp64(const DevView& v, const SystemInfo& S, int sa, int sb) {
  return r2_fp64(v, S, sa, sb);
}

struct NBAcc {
  float fx, fy, fz;
};

// Force part of the pair law in FP32 (same law as nb_pair): dE/dr divided by r.
// SW (energy switch on both terms over the same radii, the common PD setting):
// one switch factor serves LJ and Coulomb, dE/dr / r = S^2 (gv + ge) +
// (Ev + Ee) S' / r with S' = -4 u S / w^2.
template <int ELEC, bool SW = false>
__device__ __forceinline__ float nb_force_f(const NBConst& k, float r2, float rsum, float eps, float qq) {
  const float invr = rsqrtf(r2), ir2 = invr * invr;
  const float r = r2 * invr;
  if (SW) {
    const float t2 = rsum * rsum * ir2;
    const float B = t2 * t2 * t2, A = B * B;
    const bool vin = r < k.vdwcut_f;
    const float ev = vin ? eps * (A - 2.f * B) : 0.f;
    const float gv = vin ? -12.f * eps * ir2 * (A - B) : 0.f;
    const float Ee = qq * invr;
    const float u = fmaxf(r - k.inner_f, 0.f);
    const float sw = 1.f - u * u * k.invw2_f;
    return sw * sw * (gv - Ee * ir2) + (ev + Ee) * (-4.f * k.invw2_f * u * sw) * invr;
  }
  float g = 0.f;
  // switching without a branch: below the inner cutoff u = 0, so sw = 1 and the
  // derivative term is exactly 0 (same value as the unswitched law); a branch
  // here splits warps across the switching shell, which holds ~40% of the pairs
  if (k.dovdw) {
    const float t2 = rsum * rsum * ir2;
    const float B = t2 * t2 * t2, A = B * B;
    const float gv = -12.f * eps * ir2 * (A - B);
    const float u = fmaxf(r - k.vdwinner_f, 0.f);
    const float sw = 1.f - u * u * k.vdwinvw2_f;
    const float gs = sw * sw * gv + eps * (A - 2.f * B) * (-4.f * k.vdwinvw2_f * u * sw) * invr;
    g += r < k.vdwcut_f ? gs : 0.f;
  }
  if (ELEC == 1) {
    g -= qq * invr * ir2;
  } else if (ELEC == 3) {
    const float Ee = qq * invr;
    const float ge = -Ee * ir2;
    const float u = fmaxf(r - k.inner_f, 0.f);
    const float sw = 1.f - u * u * k.invw2_f;
    g += sw * sw * ge + Ee * (-4.f * k.invw2_f * u * sw) * invr;
  } else if (ELEC == 4) {
    // Steinbach & Brooks force switch, nonbonded.cpp:798-819
    if (r > k.inner_f) {
      const float c2mr2 = k.cut2 - r2;
      g -= qq * k.sA_f * ir2 * c2mr2 * c2mr2 * (k.fsw_k + 2.f * r2) * invr;
    } else {
      g -= qq * ir2 * invr;
    }
  }
  return g;
}

// 32 rotation steps of one work item: lane i holds an i atom, (xj, pj) the
// lane's j atom already in i's frame.  Tiles: j slot jb + lane, per-pair image
// when mi.  GROUP: the j atoms of a group (slots in gent[].w, -1 = empty lane,
// parked far away), never masked, one image.
template <int ELEC, bool MASKED, bool ENERGY, bool GROUP, bool SW>
__device__ __forceinline__ void nb_rot(const DevView& v, const NBConst& k, const SystemInfo& S, int lane, int si,
                                       int ai, const float4& xi, const float4& pi, float qi, unsigned ex, unsigned m14,
                                       float4 xj, float4 pj, bool mi_tile, int jb, const float4* gent, NBAcc& I,
                                       NBAcc& J, double& ev, double& ee, double& vir) {
  const bool mi = !GROUP && mi_tile;
  float Lx = 1.f, Ly = 1.f, Lz = 1.f;
  if (!GROUP && S.periodic) {
    Lx = (float)S.box[0]; Ly = (float)S.box[1]; Lz = (float)S.box[2];
  }
  const float iLx = 1.f / Lx, iLy = 1.f / Ly, iLz = 1.f / Lz;
#pragma unroll 4
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
    double r2d = 0.0;  // (ENERGY) the pair's FP64 squared distance
    int sj = 0;        // (ENERGY) the j slot
    if (ENERGY) {
      if (listed && (!GROUP || in || r2 <= 1.01f * k.cut2)) {
        sj = GROUP ? __float_as_int(gent[(lane + kk) & 31].w) : jb + ((lane + kk) & 31);
        if (sj >= 0) {
          r2d = nb_r2_fp64(v, S, si, sj);
          in = r2d <= k.cut2_dd;
        }
      }
    } else if (listed && (fabsf(r2 - k.cut2) <= 2e-6f * k.cut2 ||
                          (!SW && fabsf(r2 - k.vdwcut2) <= 2e-6f * k.vdwcut2))) {
      // at a hard cutoff: decide, and take the distance, in FP64 (FP64 work only on this branch)
      const int sjr = GROUP ? __float_as_int(gent[(lane + kk) & 31].w) : jb + ((lane + kk) & 31);
      const double d2 = nb_r2_fp64(v, S, si, sjr);
      in = d2 <= k.cut2_dd;
      r2 = (float)d2;
    }
    if (listed && in) {
      const bool is14 = MASKED && ((m14 >> kk) & 1u);
      const float eps = pi.y * pj.y * (is14 ? k.vdw14 : 1.f);
      const float qq = qi * xj.w * (is14 ? k.elec14 : 1.f);
      const float fs = nb_force_f<ELEC, SW>(k, r2, pi.x + pj.x, eps, qq);
      if (ENERGY) {
        // energy of this pair in FP64 from FP64 positions and parameters
        const int aj = v.sorted_atom[sj];
        double fsd, rdd;
        double epsd = v.sqeps[ai] * v.sqeps[aj] * (is14 ? k.vdw14_d : 1.0);
        double qqd = v.charge[ai] * v.charge[aj] * k.econv_diel_d * (is14 ? k.elec14_d : 1.0);
        nb_pair<double, ELEC>(k, r2d, v.radius[ai] + v.radius[aj], epsd, qqd, ev, ee, fsd, rdd);
        vir += rdd;
      }
      I.fx += fs * dx; I.fy += fs * dy; I.fz += fs * dz;
      J.fx -= fs * dx; J.fy -= fs * dy; J.fz -= fs * dz;
    }
    // rotate the j atom (data + its force accumulator) one lane down
    const int src = (lane + 1) & 31;
    xj.x = __shfl_sync(0xffffffffu, xj.x, src);
    xj.y = __shfl_sync(0xffffffffu, xj.y, src);
    xj.z = __shfl_sync(0xffffffffu, xj.z, src);
    xj.w = __shfl_sync(0xffffffffu, xj.w, src);
    pj.x = __shfl_sync(0xffffffffu, pj.x, src);
    pj.y = __shfl_sync(0xffffffffu, pj.y, src);
    J.fx = __shfl_sync(0xffffffffu, J.fx, src);
    J.fy = __shfl_sync(0xffffffffu, J.fy, src);
    J.fz = __shfl_sync(0xffffffffu, J.fz, src);
  }
}

// per-tile FP32 sums enter 64-bit fixed point before they are combined, so a
// slot's total does not depend on how its tiles were grouped into work items
struct NBFix {
  long long fx, fy, fz;
};

__device__ __forceinline__ void nb_fix_in(const DevView& v, NBFix& F, const NBAcc& a) {
  fix_range(v.status, fabsf(a.fx) + fabsf(a.fy) + fabsf(a.fz));
  F.fx += fx32(a.fx);
  F.fy += fx32(a.fy);
  F.fz += fx32(a.fz);
}

__device__ __forceinline__ void nb_flush_fix(const DevView& v, int s, const NBFix& F) {
  atomic_add_ll(&v.facc[3 * s], F.fx);
  atomic_add_ll(&v.facc[3 * s + 1], F.fy);
  atomic_add_ll(&v.facc[3 * s + 2], F.fz);
}

__device__ __forceinline__ void nb_flush(const DevView& v, int s, const NBAcc& a) {
  NBFix F = {0, 0, 0};
  nb_fix_in(v, F, a);
  nb_flush_fix(v, s, F);
}

// per-tile FP64 energy sums in fixed point, combined per run of tiles
struct NBEFix {
  long long vdw, elec, vir;
};

__device__ __forceinline__ void nb_efix_in(NBEFix& F, double& ev, double& ee, double& vir) {
  F.vdw += fix_energy_d(ev);
  F.elec += fix_energy_d(ee);
  F.vir += fix_energy_d(vir);
  ev = ee = vir = 0.0;
}

__device__ __forceinline__ void nb_flush_energy(const DevView& v, int lane, int bi, NBEFix& F) {
  long long e0 = warp_sum_ll(F.vdw), e1 = warp_sum_ll(F.elec), e2 = warp_sum_ll(F.vir);
  if (lane == 0) {
    long long* E = v.eacc + (size_t)v.slot_sys[bi] * E_NSLOTS;
    atomic_add_ll(&E[E_VDW], e0);
    atomic_add_ll(&E[E_ELEC], e1);
    atomic_add_ll(&E[E_VIRIAL], e2);
  }
  F = {0, 0, 0};
}

// One warp per work item, grid-stride: the tiles left on the tile path, then the
// j-atom groups (cull: the last list build wrote them and they fit)
template <int ELEC, bool ENERGY, bool SW = false>
__global__ void __launch_bounds__(256, ENERGY ? 0 : 4) k_nb_tiles(const __grid_constant__ DevView v, const __grid_constant__ NBConst k, int cull) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool grouped = cull && v.cull_n[2];
  const int nrest = grouped ? v.cull_n[0] : *v.ntiles;
  const int nitem = nrest + (grouped ? v.cull_n[1] : 0);
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nitem; w += nwarps) {
    NBAcc I = {0.f, 0.f, 0.f}, J = {0.f, 0.f, 0.f};
    double ev = 0.0, ee = 0.0, vir = 0.0;
    int bi, sjl;
    if (w < nrest) {
      const Tile T = v.tiles[grouped ? v.cull_rest[w] : w];
      bi = T.bi;
      sjl = T.bj * 32 + lane;
      const int si = T.bi * 32 + lane;
      const float4 xi = v.xq[si], pi = v.par[si];
      const float qi = xi.w * k.econv_diel;
      const int ai = ENERGY ? v.sorted_atom[si] : 0;
      const SystemInfo& S = v.sys[v.slot_sys[T.bi]];
      unsigned ex = 0u, m14 = 0u;
      if (T.mask >= 0) {
        uint2 m = v.masks[T.mask * 32 + lane];
        ex = m.x;
        m14 = m.y;
      }
      if (T.flags & 2) ex |= diag_exclusion(lane);
      // j positions moved into i's frame (the tile's centre offset, periodic image included)
      float4 xj = v.xq[sjl];
      const float4 pj = v.par[sjl];
      xj.x += T.ox;
      xj.y += T.oy;
      xj.z += T.oz;
      const bool mi = T.flags & 1;
      if (tile_masked(T))
        nb_rot<ELEC, true, ENERGY, false, SW>(v, k, S, lane, si, ai, xi, pi, qi, ex, m14, xj, pj, mi, T.bj * 32,
                                          nullptr, I, J, ev, ee, vir);
      else
        nb_rot<ELEC, false, ENERGY, false, SW>(v, k, S, lane, si, ai, xi, pi, qi, ex, m14, xj, pj, mi, T.bj * 32,
                                           nullptr, I, J, ev, ee, vir);
      nb_flush(v, si, I);
    } else {
      const int g = w - nrest;
      bi = v.cull_bi[g];
      const float4* gent = v.cull_ent + (size_t)g * 32;
      const float4 e = gent[lane];
      sjl = __float_as_int(e.w);
      const int si = bi * 32 + lane;
      const float4 xi = v.xq[si], pi = v.par[si];
      const float qi = xi.w * k.econv_diel;
      const int ai = ENERGY ? v.sorted_atom[si] : 0;
      const SystemInfo& S = v.sys[v.slot_sys[bi]];
      float4 xj = make_float4(1.0e15f, 1.0e15f, 1.0e15f, 0.f), pj = make_float4(0.f, 0.f, 0.f, 0.f);
      if (sjl >= 0) {
        xj = v.xq[sjl];
        pj = v.par[sjl];
        xj.x += e.x;
        xj.y += e.y;
        xj.z += e.z;
      }
      nb_rot<ELEC, false, ENERGY, true, SW>(v, k, S, lane, si, ai, xi, pi, qi, 0u, 0u, xj, pj, false, 0, gent, I, J,
                                        ev, ee, vir);
      nb_flush(v, si, I);
    }
    if (sjl >= 0) nb_flush(v, sjl, J);
    if (ENERGY) {
      NBEFix EF = {0, 0, 0};
      nb_efix_in(EF, ev, ee, vir);
      nb_flush_energy(v, lane, bi, EF);
    }
  }
}

template <bool E>
static void launch_nb_mode(Context& c, const NBConst& k, int g) {
  DevView v = c.view();
  const int cull = c.cull_built ? 1 : 0;
  switch (k.elecmode) {
    case 0: k_nb_tiles<0, E><<<g, 256, 0, c.stream>>>(v, k, cull); break;
    case 1: k_nb_tiles<1, E><<<g, 256, 0, c.stream>>>(v, k, cull); break;
    case 3:
      if (k.samesw && !E) k_nb_tiles<3, false, true><<<g, 256, 0, c.stream>>>(v, k, cull);
      else k_nb_tiles<3, E><<<g, 256, 0, c.stream>>>(v, k, cull);
      break;
    default: k_nb_tiles<4, E><<<g, 256, 0, c.stream>>>(v, k, cull); break;
  }
}

int launch_nb(Context& c, const NBConst& k, bool energy) {
  c.kernel_launches += 1;
  int g = tile_grid(c);
  if (energy) launch_nb_mode<true>(c, k, g);
  else launch_nb_mode<false>(c, k, g);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

// fixed-point sorted accumulators -> N in original order; also flags overflow
__global__ void k_finalize_forces(DevView v, double* out, size_t stride, int add, double scale) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  if (a < 0) return;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    long long q = v.facc[3 * s + c];
    if (q >= (1ll << 62) || q <= -(1ll << 62)) atomicOr(v.status, (unsigned)ST_FIXED_OVERFLOW);
    double f = (double)q * (1.0 / kForceScale) * scale;
    if (add) out[a * stride + c] += f;
    else out[a * stride + c] = f;
  }
}

int launch_finalize_forces(Context& c, double* out, size_t stride_doubles, bool add, double scale) {
  c.kernel_launches += 1;
  DevView v = c.view();
  k_finalize_forces<<<(c.nslots + 255) / 256, 256, 0, c.stream>>>(v, out, stride_doubles, add ? 1 : 0, scale);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
