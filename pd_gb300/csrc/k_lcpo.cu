// k_lcpo.cu — LCPO surface area (PD src/mmlib/forcefields/lcpo.cpp:640-961,
// full recalculation branch), with PD's per-atom cap of 80 overlap partners
// kept in PD's insertion (= ascending atom index) order.  Plain Euclidean
// distances, as PD does.
#include "pdgpu_tile.cuh"

namespace pdgpu {

// ---------------------------------------------------------------------------
// LCPO
// ---------------------------------------------------------------------------
// per block (one warp, a lane per slot), once per recalculation:
//  * lpos: the slot's position from its system's first block centre, rounded once
//    to FP32 (the rounding the block-centre offsets get elsewhere), w = LCPO radius;
//  * psig: (P2, P3, P4) x sigma of the slot's atom in FP32 (zero for padding);
//  * box: the block's bounding box over its LCPO atoms in the block frame of xq,
//    lo.w = their largest LCPO radius, or -1 when the block holds none
__global__ void __launch_bounds__(256) k_lcpo_prep(DevView v, const float4* lc, const double* P, const double* sigma,
                                                   float4* lpos, float4* psig, float4* box) {
  const int lane = threadIdx.x & 31;
  const int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= v.nblocks) return;  // whole warps
  const int s = b * 32 + lane;
  const int a = v.sorted_atom[s];
  const float4 l = lc[s];
  float4 p = make_float4(0.f, 0.f, 0.f, 0.f), q = p;
  if (a >= 0) {
    const int ref = v.sys[v.slot_sys[b]].block_start;
    p = make_float4((float)(v.pos[3 * a] - v.center[3 * ref]), (float)(v.pos[3 * a + 1] - v.center[3 * ref + 1]),
                    (float)(v.pos[3 * a + 2] - v.center[3 * ref + 2]), l.x);
    q = make_float4((float)(P[4 * a + 1] * sigma[a]), (float)(P[4 * a + 2] * sigma[a]),
                    (float)(P[4 * a + 3] * sigma[a]), 0.f);
  }
  lpos[s] = p;
  psig[s] = q;
  const bool use = a >= 0 && l.y > 0.f;
  const float4 x = v.xq[s];
  float lo0 = use ? x.x : INFINITY, lo1 = use ? x.y : INFINITY, lo2 = use ? x.z : INFINITY;
  float hi0 = use ? x.x : -INFINITY, hi1 = use ? x.y : -INFINITY, hi2 = use ? x.z : -INFINITY;
  float rmax = use ? l.x : -1.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo0 = fminf(lo0, __shfl_xor_sync(0xffffffffu, lo0, o));
    lo1 = fminf(lo1, __shfl_xor_sync(0xffffffffu, lo1, o));
    lo2 = fminf(lo2, __shfl_xor_sync(0xffffffffu, lo2, o));
    hi0 = fmaxf(hi0, __shfl_xor_sync(0xffffffffu, hi0, o));
    hi1 = fmaxf(hi1, __shfl_xor_sync(0xffffffffu, hi1, o));
    hi2 = fmaxf(hi2, __shfl_xor_sync(0xffffffffu, hi2, o));
    rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  }
  if (lane == 0) {
    box[2 * b] = make_float4(lo0, lo1, lo2, rmax);
    box[2 * b + 1] = make_float4(hi0, hi1, hi2, 0.f);
  }
}

// candidate overlaps: heavy-atom pairs (use == 1) with r < r_i + r_j.  A tile
// whose two block boxes lie farther apart than their largest radii can reach
// holds none and is skipped (warp-uniform test; the margin covers rounding).
// Candidates land in any order: k_lcpo_sort orders them by atom index.
__global__ void __launch_bounds__(256) k_lcpo_cand(DevView v, const float4* lc, const float4* box, int* ncand,
                                                   int* cand) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const float4 bli = box[2 * T.bi], bhi = box[2 * T.bi + 1], blj = box[2 * T.bj], bhj = box[2 * T.bj + 1];
    if (bli.w < 0.f || blj.w < 0.f) continue;
    const float gx = fmaxf(0.f, fmaxf((blj.x + T.ox) - bhi.x, bli.x - (bhj.x + T.ox)));
    const float gy = fmaxf(0.f, fmaxf((blj.y + T.oy) - bhi.y, bli.y - (bhj.y + T.oy)));
    const float gz = fmaxf(0.f, fmaxf((blj.z + T.oz) - bhi.z, bli.z - (bhj.z + T.oz)));
    const float reach = (bli.w + blj.w) * 1.001f + 1e-3f;
    if (gx * gx + gy * gy + gz * gz > reach * reach) continue;
    float4 xi = v.xq[T.bi * 32 + lane], xj = v.xq[T.bj * 32 + lane];
    xj.x += T.ox;
    xj.y += T.oy;
    xj.z += T.oz;
    const unsigned dmask = (T.flags & 2) ? diag_exclusion(lane) : 0u;
    const int si = T.bi * 32 + lane;
    const float4 li = lc[si];
    float4 lj = lc[T.bj * 32 + lane];
    // mi: the steps at which this lane's i atom has a candidate; mj: the i lanes
    // the rotating j atom has (it rotates with the atom, so after 32 steps each
    // lane holds its own j atom's mask).  One atomic per lane and side then
    // reserves the candidates, instead of one per candidate.
    unsigned mi = 0u, mj = 0u;
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      float r2 = dx * dx + dy * dy + dz * dz;
      float rr = li.x + lj.x;
      const bool c = !((dmask >> kk) & 1u) && li.y > 0.f && lj.y > 0.f && r2 < rr * rr;
      mi |= (unsigned)c << kk;
      mj |= (unsigned)c << lane;
      ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(lj.x); ROT(lj.y); ROT(mj);
    }
    if (mi) {
      int p = atomicAdd(&ncand[si], __popc(mi));
      for (unsigned m = mi; m; m &= m - 1u, p++)
        if (p < kLcpoCand) cand[(size_t)si * kLcpoCand + p] = T.bj * 32 + ((lane + __ffs(m) - 1) & 31);
    }
    if (mj) {
      const int sj = T.bj * 32 + lane;
      int p = atomicAdd(&ncand[sj], __popc(mj));
      for (unsigned m = mj; m; m &= m - 1u, p++)
        if (p < kLcpoCand) cand[(size_t)sj * kLcpoCand + p] = T.bi * 32 + (__ffs(m) - 1);
    }
  }
}

// per atom (one warp): order candidates by original atom index, keep the first
// 80 (PD's insertion order, lcpo.cpp:705-744) and store each kept partner as a
// record: (slot, s_ij) and (its lpos, radius), so the triple loop reads a row of
// records in sequence instead of chasing slot indices
__global__ void k_lcpo_sort(DevView v, const float4* lc, const float4* lpos, const int* ncand, const int* cand,
                            int* nl_n, int2* nl_e2, float4* nl_ent) {
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
      // overlap of i's sphere by j: 2 pi ri (ri - d/2 - (ri^2 - rj^2)/(2d))  (lcpo.cpp:731-733)
      float4 xi = v.xq[s], xj = v.xq[sj];
      int bi = s >> 5, bj = sj >> 5;
      float dx = xj.x - xi.x + (float)(v.center[3 * bj] - v.center[3 * bi]);
      float dy = xj.y - xi.y + (float)(v.center[3 * bj + 1] - v.center[3 * bi + 1]);
      float dz = xj.z - xi.z + (float)(v.center[3 * bj + 2] - v.center[3 * bi + 2]);
      float d = sqrtf(dx * dx + dy * dy + dz * dz);
      float ri = lc[s].x, rj = lc[sj].x;
      float rr = 0.5f * (ri * ri - rj * rj) / d;
      const float sij = 6.283185307179586f * ri * (ri - 0.5f * d - rr);
      nl_e2[(size_t)s * kLcpoMax + rank] = make_int2(sj, __float_as_int(sij));
      nl_ent[(size_t)s * kLcpoMax + rank] = lpos[sj];
    }
  }
  if (lane == 0) nl_n[s] = keep;
}

// what one overlap partner j adds to atom i's SA and force, from the sums over
// the atoms k overlapping both (lcpo.cpp:781-949): n2, a2t along d_ij, s_ji,
// the k sums n3, n3b, n4b, Si3 (sum of s_jk), Si3ik; P x sigma weights folded in
__device__ __forceinline__ void lcpo_j_terms(const float4& qi, const float4& qj, float pa2, float pa3, float pa4,
                                             float Si2_t, float sji, const float n2[3], const float a2t[3],
                                             const float n3[3], const float n3b[3], const float n4b[3], float Si3_t,
                                             float Si3ik_t, float& sa, float fl[3]) {
  // j's weights (P2, P3, P4) sigma_j on the n2, n3, n4 terms; i's P2 sigma_i and
  // P4 sigma_i on the a2 terms (lcpo.cpp:900-949)
  const float wa = qi.x + Si3_t * qi.z;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float n4 = sji * n3[c] + n4b[c] + n2[c] * Si3ik_t;
    const float n3t = n3[c] + n3b[c];
    fl[c] += n2[c] * qj.x + n3t * qj.y + n4 * qj.z + a2t[c] * wa;
  }
  sa += pa2 * Si2_t + pa3 * Si3_t + pa4 * (Si3_t * Si2_t);
}

// per atom i (one warp, lanes over i's overlap partners j): SASA_i and the
// derivative terms collected on atom i (lcpo.cpp:781-949).  Each lane sums its
// partners' terms in FP32 (already folded with the P x sigma weights, so a lane
// carries SA and the force only); the lanes combine in 64-bit fixed point.
// The atoms k that overlap both i and j are i's own partners that j overlaps:
// i's partners are staged once in the warp's shared-memory table with their
// k-only terms (d_ik, the n3 / n3b weights along d_ik, the Si3ik term), and
// every lane walks the same table (same length, broadcast reads), testing the
// j-k overlap and recomputing s_jk from the positions.  Where j's own list
// was cut at 80 partners, a k past j's 80th atom index is not j's partner.
// An atom i whose own list was cut at 80 walks its partners' lists instead
// (k need not be among i's first 80 partners there).
// Six CTAs of 256 per SM at 40 registers: the pass is bound by load latency.
constexpr int kLcpoWarps = 8;
__global__ void __launch_bounds__(kLcpoWarps * 32, 6) k_lcpo_main(DevView v, const float4* lc, const float4* lpos,
                                                   const float4* psig, const int* nl_n, const int2* nl_e2,
                                                   const float4* nl_ent, const int* ncand, const double* P,
                                                   const double* sigma, double* sasa_out, long long* facc_out,
                                                   long long* esurf_out, int esurf_stride) {
  __shared__ float4 tab_sh[kLcpoWarps][2][kLcpoMax];   // (d_ik, r_k), (w3, w3b, Si3ik term, atom_k)
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
  const float4 qi = psig[s];
  const float pa2 = (float)P[4 * a + 1], pa3 = (float)P[4 * a + 2], pa4 = (float)P[4 * a + 3];
  const float PI = 3.14159265358979f;
  const int n = nl_n[s];
  const int2* rowi = nl_e2 + (size_t)s * kLcpoMax;
  const float4* rowix = nl_ent + (size_t)s * kLcpoMax;
  const bool cut_i = ncand[s] > kLcpoMax;
  float4 (*T)[kLcpoMax] = tab_sh[threadIdx.x >> 5];
  if (!cut_i) {
    for (int t = lane; t < n; t += 32) {
      const float4 xk = rowix[t];
      const float rk = xk.w;
      const float dx = xk.x - xi.x, dy = xk.y - xi.y, dz = xk.z - xi.z;
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float inv = rsqrtf(d2);
      const float dk = d2 * inv;
      const float rrk = (ri * ri - rk * rk) * inv * inv;
      // a k that does not overlap i at these positions (the candidate test's
      // rounding) is marked with the largest atom index and skipped
      const int atom_k = ((ri + rk) * (ri + rk) < d2) ? 0x7fffffff : v.sorted_atom[rowi[t].x];
      T[0][t] = make_float4(dx, dy, dz, rk);
      T[1][t] = make_float4(PI * ri * (rrk - 1.f) * inv, PI * rk * (-rrk - 1.f) * inv,
                            PI * ri * (2.f * ri - dk - dk * rrk), __int_as_float(atom_k));
    }
  }
  __syncwarp();
  float sa = 0.f, fl[3] = {0.f, 0.f, 0.f};
  for (int jj = lane; jj < n; jj += 32) {
    const int2 ej = rowi[jj];
    const float4 xj = rowix[jj];
    const int sj = ej.x;
    const float Si2_t = __int_as_float(ej.y);
    const float4 qj = psig[sj];
    const float3 dij = make_float3(xj.x - xi.x, xj.y - xi.y, xj.z - xi.z);  // j - i
    float d = sqrtf(dij.x * dij.x + dij.y * dij.y + dij.z * dij.z);
    float rj = xj.w;
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
    if (!cut_i) {
      // j's list cut at 80: its partners are the overlapping atoms up to its 80th atom index
      const int cap_j = ncand[sj] > kLcpoMax ? v.sorted_atom[nl_e2[(size_t)sj * kLcpoMax + kLcpoMax - 1].x]
                                             : 0x7ffffffe;
      const float rj2 = rj * rj;
      for (int t = 0; t < n; t++) {
        const float4 K = T[0][t];
        const float ex = K.x - dij.x, ey = K.y - dij.y, ez = K.z - dij.z;   // k - j
        const float d2 = ex * ex + ey * ey + ez * ez;
        const float rjk = rj + K.w;
        if (t == jj || !(d2 < rjk * rjk)) continue;
        const float4 W = T[1][t];
        if (__float_as_int(W.w) > cap_j) continue;
        const float inv = rsqrtf(d2);
        // overlap of j's sphere by k: 2 pi rj (rj - d/2 - (rj^2 - rk^2)/(2d))  (lcpo.cpp:731-733)
        const float sjk = 6.283185307179586f * rj * (rj - 0.5f * d2 * inv - 0.5f * (rj2 - K.w * K.w) * inv);
        const float w4 = sjk * W.y;
        n3[0] += W.x * K.x; n3[1] += W.x * K.y; n3[2] += W.x * K.z;
        n3b[0] += W.y * K.x; n3b[1] += W.y * K.y; n3b[2] += W.y * K.z;
        n4b[0] += w4 * K.x; n4b[1] += w4 * K.y; n4b[2] += w4 * K.z;
        Si3_t += sjk;
        Si3ik_t += W.z;
      }
    } else {
      const int nk = nl_n[sj];
      const int2* rowe = nl_e2 + (size_t)sj * kLcpoMax;
      const float4* rowx = nl_ent + (size_t)sj * kLcpoMax;
      for (int kk = 0; kk < nk; kk++) {
        const int2 ek = rowe[kk];
        if (ek.x == s) continue;
        const float4 xk = rowx[kk];
        const float rk = xk.w;
        const float3 dik = make_float3(xk.x - xi.x, xk.y - xi.y, xk.z - xi.z);
        float dik2 = dik.x * dik.x + dik.y * dik.y + dik.z * dik.z;
        if ((ri + rk) * (ri + rk) < dik2) continue;
        float invdik = rsqrtf(dik2);
        float dk = dik2 * invdik;
        float rrk = (ri * ri - rk * rk) * invdik * invdik;
        float dA = PI * ri * (rrk - 1.f);
        float u0 = dik.x * invdik, u1 = dik.y * invdik, u2 = dik.z * invdik;
        float sjk = __int_as_float(ek.y);
        n3[0] += dA * u0; n3[1] += dA * u1; n3[2] += dA * u2;
        dA = PI * rk * (-rrk - 1.f);
        Si3ik_t += PI * ri * (2.f * ri - dk - dk * rrk);
        n3b[0] += dA * u0; n3b[1] += dA * u1; n3b[2] += dA * u2;
        n4b[0] += sjk * dA * u0; n4b[1] += sjk * dA * u1; n4b[2] += sjk * dA * u2;
        Si3_t += sjk;
      }
    }
    lcpo_j_terms(qi, qj, pa2, pa3, pa4, Si2_t, sji, n2, a2t, n3, n3b, n4b, Si3_t, Si3ik_t, sa, fl);
  }
  // the lanes combine in 64-bit fixed point (2^32 per unit, exact integer sums;
  // the force scale is the accumulators' own)
  fix_range(v.status, fabsf(sa) + fabsf(fl[0]) + fabsf(fl[1]) + fabsf(fl[2]));
  const long long sum_sa = warp_sum_ll(fx32(sa));
  long long f[3];
#pragma unroll
  for (int c = 0; c < 3; c++) f[c] = warp_sum_ll(fx32(fl[c]));
  if (lane == 0) {
    const double Si = 4.0 * 3.14159265358979323846 * (double)ri * ri;
    double SA = P[4 * a] * Si + (double)sum_sa * (1.0 / 4294967296.0);
    if (SA < 0) {
      SA = 0;
      f[0] = f[1] = f[2] = 0;
    }
    sasa_out[a] = SA;
    // PD adds SASAderiv / Angstrom; the derivative terms already hold d(sigma*SA)
    for (int c = 0; c < 3; c++) atomic_add_ll(&facc_out[3 * s + c], f[c]);
    int sys = v.slot_sys[s >> 5];
    if (esurf_out) atomic_add_ll(&esurf_out[(size_t)sys * esurf_stride], fix_energy_d(SA * sigma[a]));
  }
}

int launch_lcpo(Context& c, long long* facc_out, long long* esurf_out, int esurf_stride) {
  DevView v = c.view();
  cudaStream_t st = c.stream;
  int g = tile_grid(c);
  c.kernel_launches += 4;
  cudaMemsetAsync(c.d_lc_ncand.p, 0, sizeof(int) * c.nslots, st);
  k_lcpo_prep<<<(int)(((long long)c.nblocks * 32 + 255) / 256), 256, 0, st>>>(
      v, c.d_lc_par.p, c.d_lcpoP.p, c.d_lcpoSig.p, c.d_lc_pos.p, c.d_lc_psig.p, c.d_lc_box.p);
  k_lcpo_cand<<<g, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_box.p, c.d_lc_ncand.p, c.d_lc_cand.p);
  int nw = (int)(((long long)c.nslots * 32 + 255) / 256);
  k_lcpo_sort<<<nw, 256, 0, st>>>(v, c.d_lc_par.p, c.d_lc_pos.p, c.d_lc_ncand.p, c.d_lc_cand.p, c.d_lc_n.p,
                                   c.d_lc_e2.p, c.d_lc_ent.p);
  k_lcpo_main<<<(int)(((long long)c.nslots * 32 + kLcpoWarps * 32 - 1) / (kLcpoWarps * 32)), kLcpoWarps * 32, 0, st>>>(
      v, c.d_lc_par.p, c.d_lc_pos.p, c.d_lc_psig.p, c.d_lc_n.p, c.d_lc_e2.p, c.d_lc_ent.p, c.d_lc_ncand.p, c.d_lcpoP.p, c.d_lcpoSig.p, c.d_sasa.p, facc_out, esurf_out,
                                   esurf_stride);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
