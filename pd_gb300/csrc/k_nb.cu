// k_nb.cu — LJ + Coulomb tile kernel (FF_NonBonded) and force finalisation.
//
// Pair law: PD src/mmlib/forcefields/nonbonded.cpp:687-833
//   (T_fast2 instantiation with VdwMode = EnergySwitch and ElecMode picked by
//    the dispatch at nonbonded.cpp:1222-1246).
// Every listed pair j < i inside Cutoff contributes once; bond order <= 2
// pairs are zero, 1-4 pairs are scaled by Vdw14Scaling / Elec14Scaling.
#include "pdgpu_context.cuh"

namespace pdgpu {

template <int ELEC>
__device__ __forceinline__ void nb_pair(const NBConst& k, float r2, float rsum, float eps, float qq, float& ev,
                                        float& ee, float& dEdr_over_r, float& r_dEdr) {
  float invr = rsqrtf(r2);
  float r = r2 * invr;
  float dv = 0.f, de = 0.f, Ev = 0.f, Ee = 0.f;
  if (k.dovdw && r < k.vdwcut) {
    float t = rsum * invr;
    float B = t * t;
    B = B * B * B;
    float A = B * B;
    Ev = eps * (A - 2.f * B);
    dv = -12.f * eps * invr * (A - B);
    if (r > k.vdwinner) {
      float u = r - k.vdwinner;
      float sw = 1.f - u * u * k.vdwinvw2;
      float dS = -4.f * k.vdwinvw2 * u * sw;
      float S = sw * sw;
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
    if (r > k.inner) {
      float u = r - k.inner;
      float sw = 1.f - u * u * k.invw2;
      float dS = -4.f * k.invw2 * u * sw;
      float S = sw * sw;
      de = S * de + Ee * dS;
      Ee *= S;
    }
  } else if (ELEC == 4) {
    // Steinbach & Brooks force switch, nonbonded.cpp:798-819
    if (r > k.inner) {
      float c2mr2 = k.cut2_d - r2;
      de = -qq * k.sA * invr * invr * c2mr2 * c2mr2 * (k.cut2_d - 3.f * k.inner2 + 2.f * r2);
      Ee = -qq * (k.sA * r * (k.sB * invr * invr + k.sC + k.sD * r2 + k.sE * r2 * r2) - k.fsw_cutV);
    } else {
      de = -qq * invr * invr;
      Ee = qq * (invr - k.eshift);
    }
  }
  ev += Ev;
  ee += Ee;
  float d = dv + de;
  dEdr_over_r = d * invr;
  r_dEdr = r * d;
}

// One warp per tile, grid-stride over tiles.
template <int ELEC>
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
    float ev = 0.f, ee = 0.f, vir = 0.f;
    const float qi = xi.w * k.econv_diel;
#pragma unroll 4
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      if (mi) {
        dx -= Lx * rintf(dx / Lx);
        dy -= Ly * rintf(dy / Ly);
        dz -= Lz * rintf(dz / Lz);
      }
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 <= k.cut2 && !((ex >> kk) & 1u)) {
        bool is14 = (m14 >> kk) & 1u;
        float eps = pi.y * pj.y * (is14 ? k.vdw14 : 1.f);
        float qq = qi * xj.w * (is14 ? k.elec14 : 1.f);
        float fs, rd;
        nb_pair<ELEC>(k, r2, pi.x + pj.x, eps, qq, ev, ee, fs, rd);
        vir += rd;
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
    long long e0 = warp_sum_ll(fix_energy(ev));
    long long e1 = warp_sum_ll(fix_energy(ee));
    long long e2 = warp_sum_ll(fix_energy(vir));
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
  long long g = (long long)sms * 8;
  return (int)(want < g ? (want > 0 ? want : 1) : g);
}

int launch_nb(Context& c, const NBConst& k, bool) {
  DevView v = c.view();
  int g = grid_for_tiles(c);
  switch (k.elecmode) {
    case 0: k_nb_tiles<0><<<g, 256, 0, c.stream>>>(v, k); break;
    case 1: k_nb_tiles<1><<<g, 256, 0, c.stream>>>(v, k); break;
    case 3: k_nb_tiles<3><<<g, 256, 0, c.stream>>>(v, k); break;
    default: k_nb_tiles<4><<<g, 256, 0, c.stream>>>(v, k); break;
  }
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
  DevView v = c.view();
  k_finalize_forces<<<(c.nslots + 255) / 256, 256, 0, c.stream>>>(v, out, stride_doubles, add ? 1 : 0, scale);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
