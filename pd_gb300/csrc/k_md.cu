// k_md.cu — FP64 integrators, kinetic energy and the REMD exchange, on device.
//
// PD src/mmlib/protocols/md.cpp:
//   velocity Verlet (PD's variant)   applyForces_VelocityVerletIntegration :805-855
//   Langevin                          applyForces_LangevinIntegration        :923-1063
//   kinetic energy                    calcKineticEnergy                      :521-560
// PD src/mmlib/protocols/remd.cpp:
//   alternating-pair exchange + velocity rescale  :178-215, Metropolis :349-356
//
// Positions (A) and velocities (m/s) stay FP64 in original atom order.  The
// force of atom a is read straight from the fixed-point accumulators of its
// sorted slot (plus the cached LCPO share), so no separate force array is
// written during dynamics.  Gaussian noise comes from Philox4x32-10
// (Salmon et al., SC'11) keyed by the seed and counted by (step, atom), so a
// trajectory is reproducible bit for bit.
#include "pdgpu_md.cuh"

namespace pdgpu {

// ---- Philox4x32-10 ----------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32(uint4 ctr, uint2 key) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    unsigned hi0 = __umulhi(0xD2511F53u, ctr.x), lo0 = 0xD2511F53u * ctr.x;
    unsigned hi1 = __umulhi(0xCD9E8D57u, ctr.z), lo1 = 0xCD9E8D57u * ctr.z;
    ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
    key.x += 0x9E3779B9u;
    key.y += 0xBB67AE85u;
  }
  return ctr;
}
__device__ __forceinline__ double u01(unsigned x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }
// 24-bit uniform in (0, 1) for the noise: FP32 is ample for a Gaussian draw and
// keeps the transcendental work off the FP64 pipe
__device__ __forceinline__ float u01f(unsigned x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }
// two unit normals from two uniforms (Box-Muller)
__device__ __forceinline__ void box_muller(unsigned a, unsigned b, double& n1, double& n2) {
  float r = sqrtf(-2.0f * logf(u01f(a)));
  float s, c;
  sincospif(2.0f * u01f(b), &s, &c);
  n1 = (double)(r * c);
  n2 = (double)(r * s);
}

__device__ __forceinline__ void atom_force(const MDView& m, int a, double f[3]) {
  int s = m.slot_of[a];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    long long q = m.facc[3 * s + c];
    if (m.facc_sa) q += m.facc_sa[3 * s + c];
    f[c] = (double)q * (1.0 / kForceScale) * kForceToN;
  }
}

// kinetic energy into the per-system fixed-point sum (J -> kcal/mol).  Atoms
// are in system order, so a warp almost always holds one system: it adds one
// warp sum instead of 32 atomics on the same address.  Every lane of the warp
// calls this (valid = false for lanes past the last atom).
__device__ __forceinline__ void add_ke(const MDView& m, int a, bool valid, const double v[3]) {
  long long q = 0;
  int s = -1;
  if (valid) {
    const double ke = 0.5 * m.mass[a] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    q = fix_energy_d(ke * (1.0 / kKcalMolToJ));
    s = m.atom_sys[a];
  }
  const int s0 = __shfl_sync(0xffffffffu, s, 0);
  if (__all_sync(0xffffffffu, s == s0)) {
    q = warp_sum_ll(q);
    if ((threadIdx.x & 31) == 0) atomic_add_ll(&m.ke[s0], q);
  } else if (valid) {
    atomic_add_ll(&m.ke[s], q);
  }
}

// The device step counter (kept on the device so captured graphs stay valid)
// advances once per integration step: every block reads it at its start, and the
// last block to finish (a count of finished blocks) increments it and resets the
// count for the next launch.  Every thread of the block calls this.
__device__ __forceinline__ void advance_step(const MDView& m) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(m.done, 1u) == gridDim.x - 1) {
      *m.stepc += 1;
      *m.done = 0u;
    }
  }
}

// PD velocity Verlet as written: half kick, (KE), half kick, drift t*(v+dv), kick
__global__ void k_vv(MDView m, double dt) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = a < m.natom;
  double f[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0}, p[3];
  double tm = 0.0;
  if (valid) {
    atom_force(m, a, f);
    tm = 0.5 * dt * m.mterms[a].x;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      v[c] = m.vel[3 * a + c] + f[c] * tm;
      p[c] = m.pos[3 * a + c];
    }
  }
  add_ke(m, a, valid, v);
  if (valid) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double dv = f[c] * tm;
      v[c] += dv;
      p[c] += dt * (v[c] + dv) * (1.0 / kAngstrom);
      v[c] += dv;
      m.vel[3 * a + c] = v[c];
      m.pos[3 * a + c] = p[c];
    }
  }
  advance_step(m);
}

// PD Langevin step (gamma*dt > 1e-5 branch) with per-system target temperature
// Per-launch constants are folded on the host (LangevinCoeffs: kick = (1 -
// c0/c1)/gt, drift_f = c0 c2 / c1, sv = sqrt(varv), sr = sqrt(varr)/gamma):
// one division and one square root per atom remain on the narrow FP64 pipe.
__global__ void k_langevin(MDView m, LangevinCoeffs L, int first_step, int last_step) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = a < m.natom;
  const unsigned long long step = *m.stepc;
  double f[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0};
  double2 mt = make_double2(0.0, 0.0);
  double tm = 0.0;
  if (valid) {
    atom_force(m, a, f);
    mt = m.mterms[a];
    tm = L.dt * mt.x;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      v[c] = m.vel[3 * a + c];
      if (!first_step) v[c] += L.kick * f[c] * tm;
    }
  }
  add_ke(m, a, valid, v);
  if (valid && !last_step) {
    // sqrt(k_B T / m): the temperature's root in FP32 (it only scales the noise)
    const double s = (double)sqrtf((float)m.temp[m.atom_sys[a]]) * mt.y;
    const double sigmav = s * L.sv;
    const double sigmar = s * L.sr;
    // six normals, in PD's draw order n1x n2y | n2x n1z | n1y n2z (md.cpp:1017-1019)
    uint2 key = make_uint2((unsigned)m.seed, (unsigned)(m.seed >> 32));
    uint4 r0 = philox4x32(make_uint4((unsigned)step, (unsigned)(step >> 32), (unsigned)a, 0u), key);
    uint4 r1 = philox4x32(make_uint4((unsigned)step, (unsigned)(step >> 32), (unsigned)a, 1u), key);
    double n1x, n2y, n2x, n1z, n1y, n2z;
    box_muller(r0.x, r0.y, n1x, n2y);
    box_muller(r0.z, r0.w, n2x, n1z);
    box_muller(r1.x, r1.y, n1y, n2z);
    const double n1[3] = {n1x, n1y, n1z}, n2[3] = {n2x, n2y, n2z};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double dvr = sigmav * (L.crv * n1[c] + L.sq1mcrv2 * n2[c]);
      double drr = sigmar * n1[c];
      double dr = L.dt * (L.c1 * v[c] + L.c2 * f[c] * tm) + drr;
      double dv = L.drift_f * f[c] * tm + dvr;
      m.pos[3 * a + c] += dr * (1.0 / kAngstrom);
      v[c] = v[c] * L.c0 + dv;
    }
  }
  if (valid) {
#pragma unroll
    for (int c = 0; c < 3; c++) m.vel[3 * a + c] = v[c];
  }
  advance_step(m);
}

// REMD: one thread walks the temperature ladder (remd.cpp:178-215, 349-356).
// temp_sys[r] = system holding temperature rung r; ladder[r] = temperature (K).
// Exchange sweep over rung pairs (r, r+1) of one parity (remd.cpp:178-215).
// mode[r] is the lower rung's REX_Replica::ExchangeMode (remd.h:49):
//   0 Swap:     the two structures trade temperatures (here: the systems trade
//               target temperatures; velocities scale by sqrt(T'/T));
//   1 Downward: the lower rung takes a copy of the upper structure,
//   2 Upward:   the upper rung takes a copy of the lower structure;
// in both copy modes PD rescales the velocities of both rungs after the copy
// (lower / factor, upper * factor, factor = sqrt(T_upper / T_lower)).  A copy
// is recorded as copy_src[dst] = src with copy_scale[dst]; k_remd_copy applies it.
__global__ void k_remd_exchange(const long long* eacc, int nsys, int parity, const double* ladder, int* temp_sys,
                                double* temp, double* vscale, int* accepted, unsigned long long seed,
                                unsigned long long round, const int* mode, int* copy_src, double* copy_scale) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int s = 0; s < nsys; s++) {
    vscale[s] = 1.0;
    copy_src[s] = -1;
    copy_scale[s] = 1.0;
  }
  for (int r = parity; r < nsys - 1; r += 2) {
    int lo = temp_sys[r], hi = temp_sys[r + 1];
    double Tlo = ladder[r], Thi = ladder[r + 1];
    double Elo = 0, Ehi = 0;
    for (int k = 0; k < E_NSLOTS; k++) {
      if (k == E_VIRIAL) continue;
      Elo += (double)eacc[(size_t)lo * E_NSLOTS + k];
      Ehi += (double)eacc[(size_t)hi * E_NSLOTS + k];
    }
    Elo = Elo / kEnergyScale * kKcalMolToJ;
    Ehi = Ehi / kEnergyScale * kKcalMolToJ;
    const double kB = 1.38065E-23;
    double delta = (Elo - Ehi) * (1.0 / (kB * Thi) - 1.0 / (kB * Tlo));
    uint4 rr = philox4x32(make_uint4((unsigned)round, (unsigned)(round >> 32), (unsigned)r, 7u),
                          make_uint2((unsigned)seed ^ 0x5bd1e995u, (unsigned)(seed >> 32)));
    bool acc = (delta <= 0) || (exp(-delta) > u01(rr.x));
    accepted[r] = acc ? 1 : 0;
    if (acc) {
      const double factor = sqrt(Thi / Tlo);
      const int m = mode ? mode[r] : 0;
      if (m == 1) {            // Downward: lower <- copy of upper
        copy_src[lo] = hi;
        copy_scale[lo] = 1.0 / factor;
        vscale[hi] *= factor;
      } else if (m == 2) {     // Upward: upper <- copy of lower
        copy_src[hi] = lo;
        copy_scale[hi] = factor;
        vscale[lo] *= 1.0 / factor;
      } else {
        // the structure at Tlo moves to Thi and vice versa; velocities follow sqrt(T'/T)
        temp_sys[r] = hi;
        temp_sys[r + 1] = lo;
        temp[hi] = Tlo;
        temp[lo] = Thi;
        vscale[lo] *= factor;
        vscale[hi] *= 1.0 / factor;
      }
    }
  }
}

// structure copies of the copy modes: atom i of a destination system takes atom
// i of its source (equal atom counts); sources are never destinations in a sweep
__global__ void k_remd_copy(MDView m, const SystemInfo* sys, const int* copy_src, const double* copy_scale) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m.natom) return;
  const int s = m.atom_sys[a];
  const int t = copy_src[s];
  if (t < 0) return;
  const int i = a - sys[s].atom_start;
  if (i >= sys[t].natom) return;
  const int b = sys[t].atom_start + i;
  const double f = copy_scale[s];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    m.pos[3 * a + c] = m.pos[3 * b + c];
    m.vel[3 * a + c] = m.vel[3 * b + c] * f;
  }
}

// crash rescue: flag the systems holding a non-finite position or velocity
__global__ void k_nonfinite(MDView m, int* bad) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m.natom) return;
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 3; c++) ok = ok && isfinite(m.pos[3 * a + c]) && isfinite(m.vel[3 * a + c]);
  if (!ok) atomicOr(&bad[m.atom_sys[a]], 1);
}

// crash rescue of the flagged systems: positions from the checkpoint, fresh
// Gaussian velocities sqrt(kB T / m) (setInitialSpeeds, md.cpp:359-380; the
// kinetic energy is then scaled per system by k_rescale_ke)
__global__ void k_rescue(MDView m, const int* bad, const double* pos0, unsigned long long seed, long long* ke) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m.natom) return;
  const int s = m.atom_sys[a];
  if (!bad[s]) return;
  const uint2 key = make_uint2((unsigned)seed ^ 0x2545f491u, (unsigned)(seed >> 32));
  const uint4 r = philox4x32(make_uint4((unsigned)a, 0u, 0u, 11u), key);
  double n[4];
  box_muller(r.x, r.y, n[0], n[1]);
  box_muller(r.z, r.w, n[2], n[3]);
  const double sd = sqrt(1.38065E-23 * m.temp[s] / m.mass[a]);
  double e = 0.0;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    m.pos[3 * a + c] = pos0[3 * a + c];
    const double v = n[c] * sd;
    m.vel[3 * a + c] = v;
    e += 0.5 * m.mass[a] * v * v;
  }
  atomic_add_ll(&ke[s], __double2ll_rn(e * 1e30));  // J, 1e-30 J resolution
}

__global__ void k_rescale_ke(MDView m, const int* bad, const SystemInfo* sys, const long long* ke) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m.natom) return;
  const int s = m.atom_sys[a];
  if (!bad[s]) return;
  const double have = (double)ke[s] * 1e-30;
  const double want = 1.5 * sys[s].natom * 1.38065E-23 * m.temp[s];
  const double f = have > 0 ? sqrt(want / have) : 0.0;
#pragma unroll
  for (int c = 0; c < 3; c++) m.vel[3 * a + c] *= f;
}

__global__ void k_scale_vel(MDView m, const double* vscale) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m.natom) return;
  double s = vscale[m.atom_sys[a]];
  if (s != 1.0)
    for (int c = 0; c < 3; c++) m.vel[3 * a + c] *= s;
}

// zero a fixed-point buffer (kernel form so it can sit inside a captured graph
// and be skipped on steps that keep the cached LCPO forces)
__global__ void k_zero_ll(long long* p, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0;
}

int launch_integrate(Context& c, MDState& md, bool first, bool last) {
  c.kernel_launches += 1;
  MDView m = md_view(c, md);
  int nb = (c.natom + 255) / 256;
  cudaMemsetAsync(md.d_ke.p, 0, sizeof(long long) * c.nsys, c.stream);
  if (md.p.Integrator == 0) k_vv<<<nb, 256, 0, c.stream>>>(m, md.p.Timestep);
  else k_langevin<<<nb, 256, 0, c.stream>>>(m, md.L, first ? 1 : 0, last ? 1 : 0);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_remd(Context& c, MDState& md, int parity, unsigned long long round) {
  c.kernel_launches += 3;
  MDView m = md_view(c, md);
  const int nb = (c.natom + 255) / 256;
  k_remd_exchange<<<1, 32, 0, c.stream>>>(c.d_eacc.p, c.nsys, parity, md.d_ladder.p, md.d_temp_sys.p, md.d_temp.p,
                                          md.d_vscale.p, md.d_accepted.p, md.p.seed, round, md.d_mode.p,
                                          md.d_copy_src.p, md.d_copy_scale.p);
  k_remd_copy<<<nb, 256, 0, c.stream>>>(m, c.d_sys.p, md.d_copy_src.p, md.d_copy_scale.p);
  k_scale_vel<<<nb, 256, 0, c.stream>>>(m, md.d_vscale.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_rescue(Context& c, MDState& md, unsigned long long seed, int* bad_host) {
  MDView m = md_view(c, md);
  const int nb = (c.natom + 255) / 256;
  c.kernel_launches += 1;
  if (cudaMemsetAsync(md.d_bad.p, 0, sizeof(int) * c.nsys, c.stream) != cudaSuccess) return PDGPU_ERR_CUDA;
  k_nonfinite<<<nb, 256, 0, c.stream>>>(m, md.d_bad.p);
  if (cudaMemcpyAsync(bad_host, md.d_bad.p, sizeof(int) * c.nsys, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess)
    return PDGPU_ERR_CUDA;
  bool any = false;
  for (int s = 0; s < c.nsys; s++) any = any || bad_host[s];
  if (!any) return PDGPU_OK;
  c.kernel_launches += 2;
  if (cudaMemsetAsync(md.d_ke.p, 0, sizeof(long long) * c.nsys, c.stream) != cudaSuccess) return PDGPU_ERR_CUDA;
  k_rescue<<<nb, 256, 0, c.stream>>>(m, md.d_bad.p, md.d_ckpt_pos.p, seed, md.d_ke.p);
  k_rescale_ke<<<nb, 256, 0, c.stream>>>(m, md.d_bad.p, c.d_sys.p, md.d_ke.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_zero_ll(Context& c, long long* p, size_t n) {
  if (n == 0) return PDGPU_OK;
  k_zero_ll<<<(unsigned)((n + 255) / 256), 256, 0, c.stream>>>(p, n);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
