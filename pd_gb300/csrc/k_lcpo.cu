// k_lcpo.cu — LCPO surface area (PD src/mmlib/forcefields/lcpo.cpp:640-961,
// full recalculation branch), with PD's per-atom cap of 80 overlap partners
// kept in PD's insertion (= ascending atom index) order.  Plain Euclidean
// distances, as PD does.
#include "pdgpu_tile.cuh"

namespace pdgpu {

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
    float4 xi = v.xq[T.bi * 32 + lane], xj = v.xq[T.bj * 32 + lane];
    xj.x += T.ox;
    xj.y += T.oy;
    xj.z += T.oz;
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
                            float* nl_s, float4* lpos) {
  __shared__ int sh_key[8][kLcpoCand];
  __shared__ int sh_slot[8][kLcpoCand];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= v.nslots) return;
  if (lane == 0) {
    // the triple loop's positions (w: LCPO radius): from the system's first block centre, rounded
    // once to FP32 (the same rounding the block-centre offsets get elsewhere)
    const int a = v.sorted_atom[s];
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a >= 0) {
      const int ref = v.sys[v.slot_sys[s >> 5]].block_start;
      p = make_float4((float)(v.pos[3 * a] - v.center[3 * ref]), (float)(v.pos[3 * a + 1] - v.center[3 * ref + 1]),
                      (float)(v.pos[3 * a + 2] - v.center[3 * ref + 2]), lc[s].x);
    }
    lpos[s] = p;
  }
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

// relative position of slot b seen from slot a
__device__ __forceinline__ float3 rel_vec(const float4* lpos, const float4& xa, int b) {
  const float4 xb = lpos[b];
  return make_float3(xb.x - xa.x, xb.y - xa.y, xb.z - xa.z);
}

// per atom i (one warp, lanes over i's overlap partners j): SASA_i and the
// derivative terms collected on atom i (lcpo.cpp:781-949)
__global__ void k_lcpo_main(DevView v, const float4* lc, const float4* lpos, const int* nl_n, const int* nl_idx,
                            const float* nl_s, const double* P, const double* sigma, double* sasa_out,
                            long long* facc_out, long long* esurf_out, int esurf_stride) {
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
  const float4 xi = lpos[s];
  const float PI = 3.14159265358979f;
  const int n = nl_n[s];
  double Si2 = 0, Si3 = 0, Si4 = 0;
  double der[3] = {0, 0, 0}, d2[3] = {0, 0, 0}, d4[3] = {0, 0, 0};
  for (int jj = lane; jj < n; jj += 32) {
    const int sj = nl_idx[(size_t)s * kLcpoMax + jj];
    const int ja = v.sorted_atom[sj];
    const float Si2_t = nl_s[(size_t)s * kLcpoMax + jj];
    float3 dij = rel_vec(lpos, xi, sj);  // j - i
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
      const float4 xk = lpos[sk];
      const float rk = xk.w;
      const float3 dik = make_float3(xk.x - xi.x, xk.y - xi.y, xk.z - xi.z);
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
  DevView v = c.view();
  cudaStream_t st = c.stream;
  int g = tile_grid(c);
  c.kernel_launches += 3;
  cudaMemsetAsync(c.d_lc_ncand.p, 0, sizeof(int) * c.nslots, st);
  k_lcpo_cand<<<g, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_ncand.p, c.d_lc_cand.p);
  int nw = (int)(((long long)c.nslots * 32 + 255) / 256);
  k_lcpo_sort<<<nw, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_ncand.p, c.d_lc_cand.p, c.d_lc_n.p, c.d_lc_idx.p,
                                   c.d_lc_s.p, c.d_lc_pos.p);
  k_lcpo_main<<<nw, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_pos.p, c.d_lc_n.p, c.d_lc_idx.p, c.d_lc_s.p,
                                   c.d_lcpoP.p, c.d_lcpoSig.p, c.d_sasa.p, facc_out, esurf_out, esurf_stride);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
