// k_mc.cu — FF_NonBonded energy after a move of a few atoms, as PD's Monte
// Carlo protocols ask for it (calcEnergies with UsePartialRecalc,
// src/mmlib/forcefields/nonbonded.cpp:76-386, 1154-1182): the energy of the
// last reference evaluation, minus the pair energies of every pair touching a
// moved atom at the reference positions, plus the same pairs at the current
// positions.  Moved atoms are those whose position differs from the reference
// (PD compares WorkSpace::cur with WorkSpace::old).  Pair energies are FP64
// from FP64 positions, every pair of the atom's system inside Cutoff (minimum
// image in a periodic box), bond orders as PD's list holds them.
#include "pdgpu_tile.cuh"

namespace pdgpu {

__global__ void k_mc_changed(DevView v, const double* ref, unsigned char* moved, int* list, int* count) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= v.natom) return;
  const bool m = v.pos[3 * a] != ref[3 * a] || v.pos[3 * a + 1] != ref[3 * a + 1] || v.pos[3 * a + 2] != ref[3 * a + 2];
  moved[a] = m ? 1 : 0;
  if (m) list[atomicAdd(count, 1)] = a;
}

__device__ __forceinline__ double mc_r2(const double* p, const SystemInfo& S, int a, int b) {
  double r2 = 0;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double d = p[3 * b + c] - p[3 * a + c];
    if (S.periodic) d -= S.box[c] * rint(d * S.ibox[c]);
    r2 += d * d;
  }
  return r2;
}

// one warp per moved atom i, lanes over the atoms j of its system; a pair of two
// moved atoms is counted once (from its lower index)
template <int ELEC>
__global__ void k_mc_delta(const __grid_constant__ DevView v, const __grid_constant__ NBConst k, const double* ref, const int* atom_sys, const unsigned char* moved,
                           const int* list, const int* count, long long* eref) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int n = *count;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += nwarps) {
    const int i = list[w];
    const int s = atom_sys[i];
    const SystemInfo& S = v.sys[s];
    double ev = 0.0, ee = 0.0;  // new minus old
    for (int j = S.atom_start + lane; j < S.atom_start + S.natom; j += 32) {
      if (j == i || (moved[j] && j < i)) continue;
      const int bo = pair_bondorder(v, i, j);
      if (bo <= 2) continue;
      const bool is14 = bo == 3;
      const double eps = v.sqeps[i] * v.sqeps[j] * (is14 ? k.vdw14_d : 1.0);
      const double qq = v.charge[i] * v.charge[j] * k.econv_diel_d * (is14 ? k.elec14_d : 1.0);
      const double rs = v.radius[i] + v.radius[j];
      double f, rd, evn = 0.0, een = 0.0, evo = 0.0, eeo = 0.0;
      const double r2n = mc_r2(v.pos, S, i, j);
      if (r2n <= k.cut2_dd) nb_pair<double, ELEC>(k, r2n, rs, eps, qq, evn, een, f, rd);
      const double r2o = mc_r2(ref, S, i, j);
      if (r2o <= k.cut2_dd) nb_pair<double, ELEC>(k, r2o, rs, eps, qq, evo, eeo, f, rd);
      ev += evn - evo;
      ee += een - eeo;
    }
    const long long dv = warp_sum_ll(fix_energy_d(ev)), de = warp_sum_ll(fix_energy_d(ee));
    if (lane == 0) {
      atomic_add_ll(&eref[2 * s], dv);
      atomic_add_ll(&eref[2 * s + 1], de);
    }
  }
}

// the current positions become the reference for the next update
__global__ void k_mc_commit(DevView v, double* ref, const int* list, const int* count) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= *count) return;
  const int a = list[w];
#pragma unroll
  for (int c = 0; c < 3; c++) ref[3 * a + c] = v.pos[3 * a + c];
}

__global__ void k_mc_take_reference(const long long* eacc, long long* eref, int nsys) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  eref[2 * s] = eacc[(size_t)s * E_NSLOTS + E_VDW];
  eref[2 * s + 1] = eacc[(size_t)s * E_NSLOTS + E_ELEC];
}

int launch_mc_reference(Context& c) {
  c.kernel_launches += 1;
  k_mc_take_reference<<<(c.nsys + 127) / 128, 128, 0, c.stream>>>(c.d_eacc.p, c.d_mc_eref.p, c.nsys);
  if (cudaMemcpyAsync(c.d_mc_ref.p, c.d_pos.p, 24 * (size_t)c.natom, cudaMemcpyDeviceToDevice, c.stream) !=
      cudaSuccess)
    return PDGPU_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int launch_mc_update(Context& c) {
  DevView v = c.view();
  NBConst k = make_nb_const(c.nb);
  cudaStream_t st = c.stream;
  const int nb = (c.natom + 255) / 256;
  if (cudaMemsetAsync(c.d_mc_count.p, 0, sizeof(int), st) != cudaSuccess) return PDGPU_ERR_CUDA;
  c.kernel_launches += 3;
  k_mc_changed<<<nb, 256, 0, st>>>(v, c.d_mc_ref.p, c.d_mc_moved.p, c.d_mc_list.p, c.d_mc_count.p);
  const int grid = (c.natom * 32 + 255) / 256 < 4096 ? (c.natom * 32 + 255) / 256 : 4096;
  switch (k.elecmode) {
    case 0: k_mc_delta<0><<<grid, 256, 0, st>>>(v, k, c.d_mc_ref.p, c.d_atom_sys.p, c.d_mc_moved.p, c.d_mc_list.p, c.d_mc_count.p, c.d_mc_eref.p); break;
    case 1: k_mc_delta<1><<<grid, 256, 0, st>>>(v, k, c.d_mc_ref.p, c.d_atom_sys.p, c.d_mc_moved.p, c.d_mc_list.p, c.d_mc_count.p, c.d_mc_eref.p); break;
    case 3: k_mc_delta<3><<<grid, 256, 0, st>>>(v, k, c.d_mc_ref.p, c.d_atom_sys.p, c.d_mc_moved.p, c.d_mc_list.p, c.d_mc_count.p, c.d_mc_eref.p); break;
    default: k_mc_delta<4><<<grid, 256, 0, st>>>(v, k, c.d_mc_ref.p, c.d_atom_sys.p, c.d_mc_moved.p, c.d_mc_list.p, c.d_mc_count.p, c.d_mc_eref.p); break;
  }
  k_mc_commit<<<nb, 256, 0, st>>>(v, c.d_mc_ref.p, c.d_mc_list.p, c.d_mc_count.p);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
