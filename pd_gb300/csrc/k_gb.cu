// k_gb.cu — Still Generalised Born (FastMode) and LCPO surface area.
//
// GB, PD src/mmlib/forcefields/gbff.cpp:
//   Born radii            calcBornRadii_PairwiseApprox   :432-483
//   fused GB+LJ+Coulomb   calcForcesIncludingVacuo loop1 :1546-1746 (+ self term :1740-1745)
//   Born-radius chain     calcForcesIncludingVacuo loop2 :1768-1825
// LCPO, PD src/mmlib/forcefields/lcpo.cpp:640-961 (full recalculation branch).
// GB and LCPO use plain Euclidean distances, as PD does.
#include "pdgpu_context.cuh"

namespace pdgpu {

__device__ __forceinline__ void tile_setup(const DevView& v, const Tile& T, int lane, float4& xi, float4& xj,
                                           unsigned& ex, unsigned& m14) {
  const int si = T.bi * 32 + lane, sj = T.bj * 32 + lane;
  xi = v.xq[si];
  xj = v.xq[sj];
  xj.x += (float)(v.center[3 * T.bj] - v.center[3 * T.bi]);
  xj.y += (float)(v.center[3 * T.bj + 1] - v.center[3 * T.bi + 1]);
  xj.z += (float)(v.center[3 * T.bj + 2] - v.center[3 * T.bi + 2]);
  ex = 0u;
  m14 = 0u;
  if (T.mask >= 0) {
    uint2 m = v.masks[T.mask * 32 + lane];
    ex = m.x;
    m14 = m.y;
  }
}

__device__ __forceinline__ unsigned diag_exclusion(int lane) {
  return ~((lane == 0) ? 0xffffffffu : ((1u << (32 - lane)) - 1u)) | 1u;
}

#define ROT(x) x = __shfl_sync(0xffffffffu, x, (lane + 1) & 31)

// FP64 squared distance of two sorted slots from the original positions
__device__ __forceinline__ double r2_slots_fp64(const DevView& v, int sa, int sb) {
  int a = v.sorted_atom[sa], b = v.sorted_atom[sb];
  if (a < 0 || b < 0) return 1e300;
  double dx = v.pos[3 * b] - v.pos[3 * a], dy = v.pos[3 * b + 1] - v.pos[3 * a + 1],
         dz = v.pos[3 * b + 2] - v.pos[3 * a + 2];
  return dx * dx + dy * dy + dz * dz;
}


// ---------------------------------------------------------------------------
// pass 1: Born-radius pair sums  Gpol_i += P4 Vj CCF / r^4  (bond order > 2)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gb_born(DevView v, GBConst k, long long* gpol) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    float4 xi, xj;
    unsigned ex, m14;
    tile_setup(v, T, lane, xi, xj, ex, m14);
    if (T.flags & 2) ex |= diag_exclusion(lane);
    const float4 pi = v.par[T.bi * 32 + lane];
    float4 pj = v.par[T.bj * 32 + lane];
    float gi = 0.f, gj = 0.f;
#pragma unroll 4
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      bool in = r2 <= k.still2;
      if (fabsf(r2 - k.still2) <= 2e-6f * k.still2)
        in = r2_slots_fp64(v, T.bi * 32 + lane, T.bj * 32 + ((lane + kk) & 31)) <= k.still2_d;
      if (in && !((ex >> kk) & 1u)) {
        float rs = pi.z + pj.z;
        float rdivR = r2 / (rs * rs);
        float ccf = 1.f;
        if (rdivR <= k.invP5) {
          float h = 0.5f - 0.5f * cospif(rdivR * k.P5);
          ccf = h * h;
        }
        float w = k.P4 * ccf / (r2 * r2);
        gi += w * pj.w;
        gj += w * pi.w;
      }
      ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(pj.z); ROT(pj.w); ROT(gj);
    }
    atomic_add_ll(&gpol[T.bi * 32 + lane], fix_sum(gi));
    atomic_add_ll(&gpol[T.bj * 32 + lane], fix_sum(gj));
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

// Energies of one loop-1 pair (gbff.cpp:1546-1746) in FP64.
__device__ __forceinline__ void gb_pair_energy(const GBConst& k, const DevView& v, int a, int b, double r2, bool excl,
                                               bool is14, double& evdw, double& eel, double& epol) {
  if (r2 > k.cut2_d) return;
  double r = sqrt(r2), invr = 1.0 / r;
  double qiqj = v.charge[a] * v.charge[b];
  double aiaj = v.born[a] * v.born[b];
  double u = -0.25 * r2 / aiaj;
  double s14 = is14 ? k.elec14_d : 1.0;
  double S = 1.0;
  if (r >= k.inner_d) {
    double w = r - k.inner_d;
    double sw = 1.0 - w * w * k.invw2_d;
    S = sw * sw;
  }
  double elec = 0.0;
  if (u > k.thresh_d) {
    double t = exp(u);
    double ep = k.premul_d * qiqj / sqrt(r2 + t * aiaj);
    if (!excl) elec = k.econv_in_d * s14 * qiqj * invr;
    epol += 2.0 * ep * S;
  } else if (!excl) {
    elec = k.econv_out_d * s14 * qiqj * invr;
  }
  if (excl) return;
  eel += elec * S;
  if (r < k.vdwcut_d) {
    double t = (v.radius[a] + v.radius[b]) * invr;
    double B = t * t;
    B = B * B * B;
    double A = B * B;
    double eps = v.sqeps[a] * v.sqeps[b] * (is14 ? k.vdw14_d : 1.0);
    double Ev = eps * (A - 2.0 * B);
    if (r > k.vdwinner_d) {
      double w = r - k.vdwinner_d;
      double sw = 1.0 - w * w * k.vdwinvw2_d;
      Ev *= sw * sw;
    }
    evdw += Ev;
  }
}

// ---------------------------------------------------------------------------
// pass 2: GB cross term fused with vacuum LJ + Coulomb, i > j pairs within Cutoff
// (forces, dE/da in FP32; with ENERGY the pair energies are formed in FP64)
// ---------------------------------------------------------------------------
template <bool ENERGY>
__global__ void __launch_bounds__(256) k_gb_pair(DevView v, GBConst k, const float* born, long long* deda) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    float4 xi, xj;
    unsigned ex, m14;
    tile_setup(v, T, lane, xi, xj, ex, m14);
    const unsigned dmask = (T.flags & 2) ? diag_exclusion(lane) : 0u;
    const int si = T.bi * 32 + lane, sj = T.bj * 32 + lane;
    const float4 pi = v.par[si];
    float4 pj = v.par[sj];
    const float ai = born[si];
    float aj = born[sj];
    float fix = 0.f, fiy = 0.f, fiz = 0.f, fjx = 0.f, fjy = 0.f, fjz = 0.f;
    float dai = 0.f, daj = 0.f;
    double evdw = 0.0, eel = 0.0, epol = 0.0;
    const int atom_i = v.sorted_atom[si];
#pragma unroll 2
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      const bool pair = !((dmask >> kk) & 1u);
      const bool excl = (ex >> kk) & 1u;      // bond order <= 2: GB only
      const bool is14 = (m14 >> kk) & 1u;
      if (ENERGY && pair) {
        const int sjk = T.bj * 32 + ((lane + kk) & 31);
        const int atom_j = v.sorted_atom[sjk];
        if (atom_i >= 0 && atom_j >= 0)
          gb_pair_energy(k, v, atom_i, atom_j, r2_slots_fp64(v, si, sjk), excl, is14, evdw, eel, epol);
      }
      if (r2 <= k.cut2 && pair) {
        float invr = rsqrtf(r2);
        float r = r2 * invr;
        float qiqj = xi.w * xj.w;
        float aiaj = ai * aj;
        float u = -0.25f * r2 / aiaj;
        bool gbon = u > k.thresh;
        if (fabsf(u - k.thresh) <= 2e-6f * fabsf(k.thresh)) {
          // the exp-approximation switch is discontinuous: decide it in FP64
          const int sjk = T.bj * 32 + ((lane + kk) & 31);
          const int atom_j = v.sorted_atom[sjk];
          if (atom_i >= 0 && atom_j >= 0)
            gbon = -0.25 * r2_slots_fp64(v, si, sjk) / (v.born[atom_i] * v.born[atom_j]) > k.thresh_d;
        }
        float g = 0.f;           // scalar multiplying (xj - xi) in the force on i
        float elec = 0.f, delec = 0.f;
        const float s14 = is14 ? k.elec14 : 1.f;
        if (gbon) {
          float tg = expf(u);
          float l = 1.f / (r2 + tg * aiaj);
          float fgb = sqrtf(l);
          float ep = k.premul * qiqj * fgb;
          float dedr = -ep * (r - 0.25f * r * tg) * l;
          float dalpha = -ep * tg * (1.f - u) * l;
          if (!excl) {
            elec = k.econv_in * s14 * qiqj * invr;
            delec = -elec * invr;
          }
          if (r >= k.inner) {
            float w = r - k.inner;
            float sw = 1.f - w * w * k.invw2;
            float dS = -4.f * k.invw2 * w * sw;
            float S = sw * sw;
            delec = S * delec + elec * dS;
            dedr = S * dedr + dS * ep;
            dalpha *= S;
          }
          g += 2.f * dedr * invr;
          dai += dalpha * aj;
          daj += dalpha * ai;
        } else if (!excl) {
          elec = k.econv_out * s14 * qiqj * invr;
          delec = -elec * invr;
          if (r >= k.inner) {
            float w = r - k.inner;
            float sw = 1.f - w * w * k.invw2;
            float dS = -4.f * k.invw2 * w * sw;
            float S = sw * sw;
            delec = S * delec + elec * dS;
          }
        }
        if (!excl) {
          float dvdw = 0.f;
          if (r < k.vdwcut) {
            float t = (pi.x + pj.x) * invr;
            float B = t * t;
            B = B * B * B;
            float A = B * B;
            float eps = pi.y * pj.y * (is14 ? k.vdw14 : 1.f);
            float Ev = eps * (A - 2.f * B);
            dvdw = -12.f * eps * invr * (A - B);
            if (r > k.vdwinner) {
              float w = r - k.vdwinner;
              float sw = 1.f - w * w * k.vdwinvw2;
              float dS = -4.f * k.vdwinvw2 * w * sw;
              float S = sw * sw;
              dvdw = S * dvdw + Ev * dS;
            }
          }
          g += (dvdw + delec) * invr;
        }
        fix += g * dx; fiy += g * dy; fiz += g * dz;
        fjx -= g * dx; fjy -= g * dy; fjz -= g * dz;
      }
      ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(xj.w); ROT(pj.x); ROT(pj.y); ROT(aj);
      ROT(fjx); ROT(fjy); ROT(fjz); ROT(daj);
    }
    if (!(fabsf(fix) + fabsf(fiy) + fabsf(fiz) + fabsf(fjx) + fabsf(fjy) + fabsf(fjz) + fabsf(dai) + fabsf(daj) <
          1.0e18f))
      atomicOr(v.status, (unsigned)ST_NAN);
    atomic_add_ll(&v.facc[3 * si], fix_force(fix));
    atomic_add_ll(&v.facc[3 * si + 1], fix_force(fiy));
    atomic_add_ll(&v.facc[3 * si + 2], fix_force(fiz));
    atomic_add_ll(&v.facc[3 * sj], fix_force(fjx));
    atomic_add_ll(&v.facc[3 * sj + 1], fix_force(fjy));
    atomic_add_ll(&v.facc[3 * sj + 2], fix_force(fjz));
    atomic_add_ll(&deda[si], fix_sum(dai));
    atomic_add_ll(&deda[sj], fix_sum(daj));
    if (!ENERGY) continue;
    long long e0 = warp_sum_ll(fix_energy_d(evdw));
    long long e1 = warp_sum_ll(fix_energy_d(eel));
    long long e2 = warp_sum_ll(fix_energy_d(epol));
    if (lane == 0) {
      long long* E = v.eacc + (size_t)v.slot_sys[T.bi] * E_NSLOTS;
      atomic_add_ll(&E[E_VDW], e0);
      atomic_add_ll(&E[E_ELEC], e1);
      atomic_add_ll(&E[E_POL_CROSS], e2);
    }
  }
}

// self term, total dE/da and the chain-rule prefactor a^2/166 * dE/da * P4
__global__ void k_gb_self(DevView v, const double* charge, GBConst k, double premul, const long long* deda,
                          const double* born_d, float* chain) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.nslots) return;
  int a = v.sorted_atom[s];
  if (a < 0) {
    chain[s] = 0.f;
    return;
  }
  double ai = born_d[a];
  double q = charge[a];
  double self = premul * q * q / ai;
  double da = (double)deda[s] * (1.0 / kSumScale) - self / ai;
  chain[s] = (float)(ai * ai / 166.0 * da * (double)k.P4);
  int sys = v.slot_sys[s >> 5];
  atomic_add_ll(&v.eacc[(size_t)sys * E_NSLOTS + E_POL_SELF], fix_energy_d(self));
}

// ---------------------------------------------------------------------------
// pass 3: dE/da chain rule through the Born radii, both directions of a pair
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gb_chain(DevView v, GBConst k, const float* chain) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    float4 xi, xj;
    unsigned ex, m14;
    tile_setup(v, T, lane, xi, xj, ex, m14);
    if (T.flags & 2) ex |= diag_exclusion(lane);
    const float4 pi = v.par[T.bi * 32 + lane];
    float4 pj = v.par[T.bj * 32 + lane];
    const float ci = chain[T.bi * 32 + lane];
    float cj = chain[T.bj * 32 + lane];
    float fix = 0.f, fiy = 0.f, fiz = 0.f, fjx = 0.f, fjy = 0.f, fjz = 0.f;
#pragma unroll 4
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      bool in = r2 <= k.still2;
      if (fabsf(r2 - k.still2) <= 2e-6f * k.still2)
        in = r2_slots_fp64(v, T.bi * 32 + lane, T.bj * 32 + ((lane + kk) & 31)) <= k.still2_d;
      if (in && !((ex >> kk) & 1u)) {
        float rs = pi.z + pj.z;
        float rdivR = r2 / (rs * rs);
        float ccf = 1.f, dccf = 0.f;
        if (rdivR <= k.invP5) {
          float sn, cs;
          float x = rdivR * k.P5;
          sincospif(x, &sn, &cs);
          float h = 0.5f - 0.5f * cs;
          ccf = h * h;
          dccf = 2.f * h * sn * (x * 3.14159265358979f);
        }
        float ir2 = 1.f / r2;
        float w = (ci * pj.w + cj * pi.w) * (4.f * ccf - dccf) * ir2 * ir2 * ir2;
        fix -= w * dx; fiy -= w * dy; fiz -= w * dz;
        fjx += w * dx; fjy += w * dy; fjz += w * dz;
      }
      ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(pj.z); ROT(pj.w); ROT(cj); ROT(fjx); ROT(fjy); ROT(fjz);
    }
    const int si = T.bi * 32 + lane, sj = T.bj * 32 + lane;
    atomic_add_ll(&v.facc[3 * si], fix_force(fix));
    atomic_add_ll(&v.facc[3 * si + 1], fix_force(fiy));
    atomic_add_ll(&v.facc[3 * si + 2], fix_force(fiz));
    atomic_add_ll(&v.facc[3 * sj], fix_force(fjx));
    atomic_add_ll(&v.facc[3 * sj + 1], fix_force(fjy));
    atomic_add_ll(&v.facc[3 * sj + 2], fix_force(fjz));
  }
}

static int tile_grid(Context& c) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
  long long want = (c.ncand + 7) / 8;
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
  k_gb_born<<<g, 256, 0, st>>>(v, k, c.d_gpol.p);
  k_gb_radii<<<nb, 256, 0, st>>>(v, c.d_gbT.p, c.d_gpol.p, halfeconv, born_offset, c.d_born_f.p, c.d_born_d.p);
  if (energy) k_gb_pair<true><<<g, 256, 0, st>>>(v, k, c.d_born_f.p, c.d_deda.p);
  else k_gb_pair<false><<<g, 256, 0, st>>>(v, k, c.d_born_f.p, c.d_deda.p);
  k_gb_self<<<nb, 256, 0, st>>>(v, c.d_charge.p, k, premul, c.d_deda.p, c.d_born_d.p, c.d_chain_f.p);
  k_gb_chain<<<g, 256, 0, st>>>(v, k, c.d_chain_f.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

// one GB pass on its own (timing probe): 1 Born sums, 2 fused pair (forces), 3 chain rule
int launch_gb_stage(Context& c, const GBConst& k, int stage) {
  DevView v = c.view();
  int g = tile_grid(c);
  c.kernel_launches += 1;
  if (stage == 1) k_gb_born<<<g, 256, 0, c.stream>>>(v, k, c.d_gpol.p);
  else if (stage == 2) k_gb_pair<false><<<g, 256, 0, c.stream>>>(v, k, c.d_born_f.p, c.d_deda.p);
  else k_gb_chain<<<g, 256, 0, c.stream>>>(v, k, c.d_chain_f.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// LCPO
// ---------------------------------------------------------------------------
// candidate overlaps: heavy-atom pairs (use == 1) with r < r_i + r_j
__global__ void __launch_bounds__(256) k_lcpo_cand(DevView v, const float4* lc, int* ncand, int* cand) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    float4 xi, xj;
    unsigned ex, m14;
    tile_setup(v, T, lane, xi, xj, ex, m14);
    const unsigned dmask = (T.flags & 2) ? diag_exclusion(lane) : 0u;
    const int si = T.bi * 32 + lane;
    const float4 li = lc[si];
    int sj = T.bj * 32 + lane;
    float4 lj = lc[sj];
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      float rr = li.x + lj.x;
      if (!((dmask >> kk) & 1u) && li.y > 0.f && lj.y > 0.f && r2 < rr * rr) {
        int p = atomicAdd(&ncand[si], 1);
        if (p < kLcpoCand) cand[(size_t)si * kLcpoCand + p] = sj;
        p = atomicAdd(&ncand[sj], 1);
        if (p < kLcpoCand) cand[(size_t)sj * kLcpoCand + p] = si;
      }
      ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(lj.x); ROT(lj.y); ROT(sj);
    }
  }
}

// per atom (one warp): order candidates by original atom index, keep the first
// 80 (PD's insertion order, lcpo.cpp:705-744) and store s_ij
__global__ void k_lcpo_sort(DevView v, const float4* lc, const int* ncand, const int* cand, int* nl_n, int* nl_idx,
                            float* nl_s) {
  __shared__ int sh_key[8][kLcpoCand];
  __shared__ int sh_slot[8][kLcpoCand];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= v.nslots) return;
  int n = ncand[s];
  if (n > kLcpoCand) {
    if (lane == 0) atomicOr(v.status, (unsigned)ST_LCPO_OVERFLOW);
    n = kLcpoCand;
  }
  for (int p = lane; p < kLcpoCand; p += 32) {
    int sl = p < n ? cand[(size_t)s * kLcpoCand + p] : -1;
    sh_slot[w][p] = sl;
    sh_key[w][p] = sl >= 0 ? v.sorted_atom[sl] : 0x7fffffff;
  }
  __syncwarp();
  // rank sort (keys are distinct atom indices)
  int keep = n < kLcpoMax ? n : kLcpoMax;
  for (int p = lane; p < n; p += 32) {
    int key = sh_key[w][p];
    int rank = 0;
    for (int q = 0; q < n; q++) rank += sh_key[w][q] < key;
    if (rank < keep) {
      int sj = sh_slot[w][p];
      nl_idx[(size_t)s * kLcpoMax + rank] = sj;
      // overlap of i's sphere by j: 2 pi ri (ri - d/2 - (ri^2 - rj^2)/(2d))  (lcpo.cpp:731-733)
      float4 xi = v.xq[s], xj = v.xq[sj];
      int bi = s >> 5, bj = sj >> 5;
      float dx = xj.x - xi.x + (float)(v.center[3 * bj] - v.center[3 * bi]);
      float dy = xj.y - xi.y + (float)(v.center[3 * bj + 1] - v.center[3 * bi + 1]);
      float dz = xj.z - xi.z + (float)(v.center[3 * bj + 2] - v.center[3 * bi + 2]);
      float d = sqrtf(dx * dx + dy * dy + dz * dz);
      float ri = lc[s].x, rj = lc[sj].x;
      float rr = 0.5f * (ri * ri - rj * rj) / d;
      nl_s[(size_t)s * kLcpoMax + rank] = 6.283185307179586f * ri * (ri - 0.5f * d - rr);
    }
  }
  if (lane == 0) nl_n[s] = keep;
}

// relative position of slot b seen from slot a (block-centre offsets in FP64)
__device__ __forceinline__ float3 rel_vec(const DevView& v, int a, int b) {
  float4 xa = v.xq[a], xb = v.xq[b];
  int ba = a >> 5, bb = b >> 5;
  float3 d;
  d.x = xb.x - xa.x + (float)(v.center[3 * bb] - v.center[3 * ba]);
  d.y = xb.y - xa.y + (float)(v.center[3 * bb + 1] - v.center[3 * ba + 1]);
  d.z = xb.z - xa.z + (float)(v.center[3 * bb + 2] - v.center[3 * ba + 2]);
  return d;
}

// per atom i (one warp, lanes over i's overlap partners j): SASA_i and the
// derivative terms collected on atom i (lcpo.cpp:781-949)
__global__ void k_lcpo_main(DevView v, const float4* lc, const int* nl_n, const int* nl_idx, const float* nl_s,
                            const double* P, const double* sigma, double* sasa_out, long long* facc_out,
                            long long* esurf_out, int esurf_stride) {
  const int lane = threadIdx.x & 31;
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= v.nslots) return;
  const int a = v.sorted_atom[s];
  if (a < 0) return;
  const float4 li = lc[s];
  if (li.y <= 0.f) {
    if (lane == 0) sasa_out[a] = 0.0;
    return;
  }
  const float ri = li.x;
  const float PI = 3.14159265358979f;
  const int n = nl_n[s];
  double Si2 = 0, Si3 = 0, Si4 = 0;
  double der[3] = {0, 0, 0}, d2[3] = {0, 0, 0}, d4[3] = {0, 0, 0};
  for (int jj = lane; jj < n; jj += 32) {
    const int sj = nl_idx[(size_t)s * kLcpoMax + jj];
    const int ja = v.sorted_atom[sj];
    const float Si2_t = nl_s[(size_t)s * kLcpoMax + jj];
    float3 dij = rel_vec(v, s, sj);  // j - i
    float d = sqrtf(dij.x * dij.x + dij.y * dij.y + dij.z * dij.z);
    float rj = lc[sj].x;
    float invd = 1.f / d;
    float rr = 0.5f * (ri * ri - rj * rj) * invd;
    float sji = 6.283185307179586f * rj * (rj - 0.5f * d + rr);
    rr *= 2.f * invd;
    float ddd[3] = {dij.x * invd, dij.y * invd, dij.z * invd};
    float dAdd = PI * rj * (-rr - 1.f);
    float n2[3] = {dAdd * ddd[0], dAdd * ddd[1], dAdd * ddd[2]};
    dAdd = PI * ri * (rr - 1.f);
    float a2t[3] = {dAdd * ddd[0], dAdd * ddd[1], dAdd * ddd[2]};
    float n3[3] = {0, 0, 0}, n3b[3] = {0, 0, 0}, n4b[3] = {0, 0, 0};
    float Si3_t = 0.f, Si3ik_t = 0.f;
    const int nk = nl_n[sj];
    for (int kk = 0; kk < nk; kk++) {
      const int sk = nl_idx[(size_t)sj * kLcpoMax + kk];
      if (sk == s) continue;
      const float rk = lc[sk].x;
      float3 dik = rel_vec(v, s, sk);
      float dik2 = dik.x * dik.x + dik.y * dik.y + dik.z * dik.z;
      if ((ri + rk) * (ri + rk) < dik2) continue;
      float invdik = rsqrtf(dik2);
      float dk = dik2 * invdik;
      float rrk = (ri * ri - rk * rk) * invdik * invdik;
      float dA = PI * ri * (rrk - 1.f);
      float u0 = dik.x * invdik, u1 = dik.y * invdik, u2 = dik.z * invdik;
      float sjk = nl_s[(size_t)sj * kLcpoMax + kk];
      n3[0] += dA * u0; n3[1] += dA * u1; n3[2] += dA * u2;
      dA = PI * rk * (-rrk - 1.f);
      Si3ik_t += PI * ri * (2.f * ri - dk - dk * rrk);
      n3b[0] += dA * u0; n3b[1] += dA * u1; n3b[2] += dA * u2;
      n4b[0] += sjk * dA * u0; n4b[1] += sjk * dA * u1; n4b[2] += sjk * dA * u2;
      Si3_t += sjk;
    }
    const double p2 = P[4 * ja + 1] * sigma[ja], p3 = P[4 * ja + 2] * sigma[ja], p4 = P[4 * ja + 3] * sigma[ja];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double n4 = (double)sji * n3[c] + n4b[c] + (double)n2[c] * Si3ik_t;
      double n3t = (double)n3[c] + n3b[c];
      der[c] += n2[c] * p2 + n3t * p3 + n4 * p4;
      d2[c] += a2t[c];
      d4[c] += (double)Si3_t * a2t[c];
    }
    Si4 += (double)Si3_t * Si2_t;
    Si3 += Si3_t;
    Si2 += Si2_t;
  }
  Si2 = warp_sum_d(Si2);
  Si3 = warp_sum_d(Si3);
  Si4 = warp_sum_d(Si4);
  for (int c = 0; c < 3; c++) {
    der[c] = warp_sum_d(der[c]);
    d2[c] = warp_sum_d(d2[c]);
    d4[c] = warp_sum_d(d4[c]);
  }
  if (lane == 0) {
    const double Si = 4.0 * 3.14159265358979323846 * (double)ri * ri;
    double SA = P[4 * a] * Si + P[4 * a + 1] * Si2 + P[4 * a + 2] * Si3 + P[4 * a + 3] * Si4;
    double f[3];
    for (int c = 0; c < 3; c++) f[c] = der[c] + d2[c] * (P[4 * a + 1] * sigma[a]) + d4[c] * (P[4 * a + 3] * sigma[a]);
    if (SA < 0) {
      SA = 0;
      f[0] = f[1] = f[2] = 0;
    }
    sasa_out[a] = SA;
    // PD adds SASAderiv / Angstrom; the derivative terms already hold d(sigma*SA)
    for (int c = 0; c < 3; c++) atomic_add_ll(&facc_out[3 * s + c], __double2ll_rn(f[c] * kForceScale));
    int sys = v.slot_sys[s >> 5];
    if (esurf_out) atomic_add_ll(&esurf_out[(size_t)sys * esurf_stride], fix_energy_d(SA * sigma[a]));
  }
}

int launch_lcpo(Context& c, long long* facc_out, long long* esurf_out, int esurf_stride) {
  c.kernel_launches += 3;
  DevView v = c.view();
  cudaStream_t st = c.stream;
  int g = tile_grid(c);
  cudaMemsetAsync(c.d_lc_ncand.p, 0, sizeof(int) * c.nslots, st);
  k_lcpo_cand<<<g, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_ncand.p, c.d_lc_cand.p);
  int nw = (int)(((long long)c.nslots * 32 + 255) / 256);
  k_lcpo_sort<<<nw, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_ncand.p, c.d_lc_cand.p, c.d_lc_n.p, c.d_lc_idx.p,
                                   c.d_lc_s.p);
  k_lcpo_main<<<nw, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_n.p, c.d_lc_idx.p, c.d_lc_s.p, c.d_lcpoP.p,
                                   c.d_lcpoSig.p, c.d_sasa.p, facc_out, esurf_out, esurf_stride);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
