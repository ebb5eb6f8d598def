// k_nb.cu — LJ + Coulomb tile kernel (FF_NonBonded) and force finalisation.
//
// Pair law: PD src/mmlib/forcefields/nonbonded.cpp:687-833
//   (T_fast2 instantiation with VdwMode = EnergySwitch and ElecMode picked by
//    the dispatch at nonbonded.cpp:1222-1246).
// Every listed pair j < i inside Cutoff contributes once; bond order <= 2
// pairs are zero, 1-4 pairs are scaled by Vdw14Scaling / Elec14Scaling.
#include "pdgpu_context.cuh"

namespace pdgpu {

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
    if (S.periodic) d -= S.box[c] * rint(d / S.box[c]);
    r2 += d * d;
  }
  return r2;
}

// One warp per tile, grid-stride over tiles.
template <int ELEC, bool ENERGY>
__global__ void __launch_bounds__(256) k_nb_tiles(DevView v, NBConst k) {
  const int lane = threadIdx.x & 31;
  const int warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = warp0; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const int si = T.bi * 32 + lane, sj = T.bj * 32 + lane;
    const float4 xi = v.xq[si];
    const float4 pi = v.par[si];
    float4 xj = v.xq[sj];
    float4 pj = v.par[sj];
    const int sidx = v.slot_sys[T.bi];
    const SystemInfo& S = v.sys[sidx];
    // j positions moved into i's frame: centre offset in FP64, once per tile
    double dcx = v.center[3 * T.bj] - v.center[3 * T.bi];
    double dcy = v.center[3 * T.bj + 1] - v.center[3 * T.bi + 1];
    double dcz = v.center[3 * T.bj + 2] - v.center[3 * T.bi + 2];
    float Lx = 0.f, Ly = 0.f, Lz = 0.f;
    if (S.periodic) {
      dcx -= S.box[0] * rint(dcx / S.box[0]);
      dcy -= S.box[1] * rint(dcy / S.box[1]);
      dcz -= S.box[2] * rint(dcz / S.box[2]);
      Lx = (float)S.box[0]; Ly = (float)S.box[1]; Lz = (float)S.box[2];
    }
    xj.x += (float)dcx;
    xj.y += (float)dcy;
    xj.z += (float)dcz;
    const bool mi = T.flags & 1;
    const bool diag = T.flags & 2;
    unsigned ex = 0u, m14 = 0u;
    if (T.mask >= 0) {
      uint2 m = v.masks[T.mask * 32 + lane];
      ex = m.x;
      m14 = m.y;
    }
    if (diag) ex |= ~((lane == 0) ? 0xffffffffu : ((1u << (32 - lane)) - 1u)) | 1u;  // keep only lane+k < 32, k > 0
    float fix = 0.f, fiy = 0.f, fiz = 0.f, fjx = 0.f, fjy = 0.f, fjz = 0.f;
    double ev = 0.0, ee = 0.0, vir = 0.0;
    const float qi = xi.w * k.econv_diel;
    const int ai = ENERGY ? v.sorted_atom[si] : 0;
#pragma unroll 4
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      if (mi) {
        dx -= Lx * rintf(dx / Lx);
        dy -= Ly * rintf(dy / Ly);
        dz -= Lz * rintf(dz / Lz);
      }
      float r2 = dx * dx + dy * dy + dz * dz;
      const bool listed = !((ex >> kk) & 1u);
      bool in = r2 <= k.cut2;
      double r2d = 0.0;
      if (listed && (ENERGY || fabsf(r2 - k.cut2) <= 2e-6f * k.cut2 || fabsf(r2 - k.vdwcut2) <= 2e-6f * k.vdwcut2)) {
        r2d = r2_fp64(v, S, si, T.bj * 32 + ((lane + kk) & 31));
        in = r2d <= k.cut2_dd;
      }
      if (listed && in) {
        bool is14 = (m14 >> kk) & 1u;
        float eps = pi.y * pj.y * (is14 ? k.vdw14 : 1.f);
        float qq = qi * xj.w * (is14 ? k.elec14 : 1.f);
        float fs, rd, evf = 0.f, eef = 0.f;
        if (r2d > 0.0 && !ENERGY) r2 = (float)r2d;
        nb_pair<float, ELEC>(k, r2, pi.x + pj.x, eps, qq, evf, eef, fs, rd);
        if (ENERGY) {
          // energy of this pair in FP64 from FP64 positions and parameters
          const int aj = v.sorted_atom[T.bj * 32 + ((lane + kk) & 31)];
          double fsd, rdd;
          double epsd = v.sqeps[ai] * v.sqeps[aj] * (is14 ? k.vdw14_d : 1.0);
          double qqd = v.charge[ai] * v.charge[aj] * k.econv_diel_d * (is14 ? k.elec14_d : 1.0);
          nb_pair<double, ELEC>(k, r2d, v.radius[ai] + v.radius[aj], epsd, qqd, ev, ee, fsd, rdd);
          vir += rdd;
        }
        fix += fs * dx; fiy += fs * dy; fiz += fs * dz;
        fjx -= fs * dx; fjy -= fs * dy; fjz -= fs * dz;
      }
      // rotate the j atom (data + its force accumulator) one lane down
      const int src = (lane + 1) & 31;
      xj.x = __shfl_sync(0xffffffffu, xj.x, src);
      xj.y = __shfl_sync(0xffffffffu, xj.y, src);
      xj.z = __shfl_sync(0xffffffffu, xj.z, src);
      xj.w = __shfl_sync(0xffffffffu, xj.w, src);
      pj.x = __shfl_sync(0xffffffffu, pj.x, src);
      pj.y = __shfl_sync(0xffffffffu, pj.y, src);
      fjx = __shfl_sync(0xffffffffu, fjx, src);
      fjy = __shfl_sync(0xffffffffu, fjy, src);
      fjz = __shfl_sync(0xffffffffu, fjz, src);
    }
    if (!(fabsf(fix) + fabsf(fiy) + fabsf(fiz) + fabsf(fjx) + fabsf(fjy) + fabsf(fjz) < 1.0e18f))
      atomicOr(v.status, (unsigned)ST_NAN);
    atomic_add_ll(&v.facc[3 * si], fix_force(fix));
    atomic_add_ll(&v.facc[3 * si + 1], fix_force(fiy));
    atomic_add_ll(&v.facc[3 * si + 2], fix_force(fiz));
    atomic_add_ll(&v.facc[3 * sj], fix_force(fjx));
    atomic_add_ll(&v.facc[3 * sj + 1], fix_force(fjy));
    atomic_add_ll(&v.facc[3 * sj + 2], fix_force(fjz));
    if (!ENERGY) continue;
    long long e0 = warp_sum_ll(fix_energy_d(ev));
    long long e1 = warp_sum_ll(fix_energy_d(ee));
    long long e2 = warp_sum_ll(fix_energy_d(vir));
    if (lane == 0) {
      long long* E = v.eacc + (size_t)sidx * E_NSLOTS;
      atomic_add_ll(&E[E_VDW], e0);
      atomic_add_ll(&E[E_ELEC], e1);
      atomic_add_ll(&E[E_VIRIAL], e2);
    }
  }
}

static int grid_for_tiles(Context& c) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
  // persistent-style grid: 8 resident 256-thread CTAs per SM, grid-stride over tiles
  long long want = (c.ncand + 7) / 8;
  long long g = (long long)sms * c.tile_ctas_per_sm;
  return (int)(want < g ? (want > 0 ? want : 1) : g);
}

template <bool E>
static void launch_nb_mode(Context& c, const NBConst& k, int g) {
  DevView v = c.view();
  switch (k.elecmode) {
    case 0: k_nb_tiles<0, E><<<g, 256, 0, c.stream>>>(v, k); break;
    case 1: k_nb_tiles<1, E><<<g, 256, 0, c.stream>>>(v, k); break;
    case 3: k_nb_tiles<3, E><<<g, 256, 0, c.stream>>>(v, k); break;
    default: k_nb_tiles<4, E><<<g, 256, 0, c.stream>>>(v, k); break;
  }
}

int launch_nb(Context& c, const NBConst& k, bool energy) {
  c.kernel_launches += 1;
  int g = grid_for_tiles(c);
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
    if (q > (1ll << 62) || q < -(1ll << 62)) atomicOr(v.status, (unsigned)ST_FIXED_OVERFLOW);
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
