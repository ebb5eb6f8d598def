// pdgpu_md_api.cu — dynamics, REMD and autotuning entry points of the C ABI.
//
// One MD step of every system in the batch is: list refresh on the
// UpdateNList cadence (or a position pack + skin check), forces of the chosen
// components, LCPO on its UpdateSasa cadence (its forces and energy cached in
// between, as FF_SASA_LCPO::calcForces does, lcpo.cpp:193-206), then the
// integrator.  The step sequence of each distinct flavour (rebuild / LCPO /
// energy) is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "pdgpu_md.cuh"

using namespace pdgpu;

struct pdgpu_ctx {
  Context c;
};

namespace pdgpu {

void destroy_md(Context& c) {
  if (!c.md) return;
  for (auto& kv : c.md->graphs) cudaGraphExecDestroy(kv.second);
  delete c.md;
  c.md = nullptr;
}

void drop_step_graphs(Context& c) {
  if (!c.md) return;
  for (auto& kv : c.md->graphs) cudaGraphExecDestroy(kv.second);
  c.md->graphs.clear();
}

}  // namespace pdgpu

namespace {

#define CK(expr)                                   \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return PDGPU_ERR_CUDA;  \
  } while (0)

void invalidate_graphs(MDState& md) {
  for (auto& kv : md.graphs) cudaGraphExecDestroy(kv.second);
  md.graphs.clear();
}

// per-atom mass terms of the integrators: 1 / m and sqrt(k_B / m) (md.cpp:951-960)
__global__ void k_mass_terms(const double* mass, double2* out, int n) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a < n) out[a] = make_double2(1.0 / mass[a], sqrt(1.38065E-23 / mass[a]));
}

// kinetic energies from their fixed-point sums to J (pdgpu_get_kinetic_async)
__global__ void k_ke_joules(const long long* ke, double* out, int nsys) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) out[s] = (double)ke[s] / kEnergyScale * kKcalMolToJ;
}

__global__ void k_add_surf(long long* eacc, const long long* cache, int nsys) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) eacc[(size_t)s * E_NSLOTS + E_SURF] += cache[s];
}

// enqueue one step; flags: 1 rebuild, 2 LCPO recalculation, 4 energies
int enqueue_step(Context& c, MDState& md, int flags, bool first) {
  const bool rebuild = flags & 1, sasa = flags & 2, energy = flags & 4;
  const bool has_sa = md.p.what & PDGPU_SA;
  if (has_sa && sasa) {
    CK(cudaMemsetAsync(md.d_facc_sa.p, 0, sizeof(long long) * 3 * c.nslots, c.stream));
    CK(cudaMemsetAsync(md.d_surf_cache.p, 0, sizeof(long long) * c.nsys, c.stream));
  }
  int st = enqueue_forces(c, md.p.what, energy, rebuild, md.d_facc_sa.p, md.d_surf_cache.p, 1, sasa);
  if (st != PDGPU_OK) return st;
  if (has_sa && energy) {
    k_add_surf<<<(c.nsys + 127) / 128, 128, 0, c.stream>>>(c.d_eacc.p, md.d_surf_cache.p, c.nsys);
    c.kernel_launches += 1;
    CK(cudaGetLastError());
  }
  return launch_integrate(c, md, first, false);
}

int run_step(Context& c, MDState& md, int flags, bool first) {
  if (!md.p.use_graph || first) return enqueue_step(c, md, flags, first);
  auto it = md.graphs.find(flags);
  if (it == md.graphs.end()) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    const long long before = c.kernel_launches;
    int st = enqueue_step(c, md, flags, false);
    md.graph_kernels[flags] = c.kernel_launches - before;
    c.kernel_launches = before;
    cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    if (st != PDGPU_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return PDGPU_ERR_CUDA;
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return PDGPU_ERR_CUDA;
    it = md.graphs.emplace(flags, ex).first;
  }
  CK(cudaGraphLaunch(it->second, c.stream));
  c.kernel_launches += md.graph_kernels[flags];
  return PDGPU_OK;
}

LangevinCoeffs coeffs(double gamma, double t) {
  // md.cpp:966-1003: exponential branch for gamma*t > 0.05, Taylor series otherwise
  LangevinCoeffs L{};
  double gt = gamma * t;
  L.dt = t;
  L.gamma = gamma;
  L.gt = gt;
  if (gt > 0.05) {
    L.c0 = std::exp(-gt);
    L.c1 = (1 - L.c0) / gt;
    L.c2 = (1 - L.c1) / gt;
    double eg = std::exp(-gt);
    L.varv = 1.0 - eg * eg;
    L.varr = 2.0 * gt - 3.0 + (4.0 - eg) * eg;
    L.crv = (1.0 - eg) * (1.0 - eg) / std::sqrt(L.varv * L.varr);
  } else {
    double g2 = gt * gt, g3 = gt * g2, g4 = g2 * g2, g5 = g2 * g3, g6 = g3 * g3, g7 = g3 * g4, g8 = g4 * g4,
           g9 = g4 * g5;
    L.c0 = 1 - gt + 0.5 * g2 - g3 / 6.0 + g4 / 24.0 - g5 / 120.0 + g6 / 720.0 - g7 / 5040.0 + g8 / 40320.0 -
           g9 / 362880.0;
    L.c1 = 1 - (0.5 * gt - g2 / 6.0 + g3 / 24.0 - g4 / 120.0 + g5 / 720.0 - g6 / 5040.0 + g7 / 40320.0 -
                g8 / 362880.0);
    L.c2 = 0.5 - gt / 6.0 + g2 / 24.0 - g3 / 120.0 + g4 / 720.0 - g5 / 5040.0 + g6 / 40320.0 - g7 / 362880.0;
    L.varr = 2.0 * g3 / 3.0 - g4 / 2.0 + 7.0 * g5 / 30.0 - g6 / 12.0 + 31.0 * g7 / 1260.0 - g8 / 160.0 +
             127.0 * g9 / 90720.0;
    L.varv = 2.0 * gt - 2.0 * g2 + 4.0 * g3 / 3.0 - 2.0 * g4 / 3.0 + 4.0 * g5 / 15.0 - 4.0 * g6 / 45.0 +
             8.0 * g7 / 315.0 - 2.0 * g8 / 315.0 + 4.0 * g9 / 2835.0;
    L.crv = std::sqrt(3.0) * (0.5 - 3.0 * gt / 16.0 - 17.0 * g2 / 1280.0 + 17.0 * g3 / 6144.0 +
                              40967.0 * g4 / 34406400.0 - 57203.0 * g5 / 275251200.0 -
                              1429487.0 * g6 / 13212057600.0);
  }
  L.sq1mcrv2 = std::sqrt(1.0 - L.crv * L.crv);
  L.kick = (1.0 - L.c0 / L.c1) / L.gt;
  L.drift_f = L.c0 * L.c2 / L.c1;
  L.sv = std::sqrt(L.varv);
  L.sr = std::sqrt(L.varr) / L.gamma;
  return L;
}

int read_status_md(Context& c) {
  unsigned st = 0;
  CK(cudaMemcpyAsync(&st, c.d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (st & ST_NAN) return PDGPU_ERR_NAN;
  if (st & ST_FIXED_OVERFLOW) return PDGPU_ERR_FIXED_OVERFLOW;
  if (st & (ST_LCPO_OVERFLOW | ST_TILE_OVERFLOW)) return PDGPU_ERR_LIST_OVERFLOW;
  if (st & ST_STALE_LIST) return PDGPU_ERR_STALE_LIST;
  return PDGPU_OK;
}

int md_enqueue_impl(Context& c, MDState& md, int nsteps, bool energy_on_last) {
  for (int k = 0; k < nsteps; k++) {
    const unsigned long long s = md.step;
    int flags = 0;
    if (s % (unsigned long long)md.p.UpdateNList == 0 || !c.list_built) flags |= 1;
    if ((md.p.what & PDGPU_SA) && (s % (unsigned long long)md.p.UpdateSasa == 0 || md.force_sasa)) flags |= 2;
    md.force_sasa = false;
    if (energy_on_last && k == nsteps - 1) flags |= 4;
    bool first = !md.trajectory_started;
    int st = run_step(c, md, flags, first);
    if (st != PDGPU_OK) return st;
    md.trajectory_started = true;
    md.step++;
    if (md.traj_every > 0 && md.step % (unsigned long long)md.traj_every == 0) {
      // a frame of every system's positions, queued behind the step on the context stream
      double* dst = md.traj_ring + (size_t)(md.traj_frames % md.traj_slots) * 3 * (size_t)c.natom;
      CK(cudaMemcpyAsync(dst, c.d_pos.p, 24 * (size_t)c.natom, cudaMemcpyDeviceToHost, c.stream));
      md.traj_frames++;
    }
  }
  return PDGPU_OK;
}

int md_run_impl(Context& c, MDState& md, int nsteps, bool energy_on_last) {
  CK(cudaMemsetAsync(c.d_status.p, 0, sizeof(unsigned), c.stream));
  int st = md_enqueue_impl(c, md, nsteps, energy_on_last);
  if (st != PDGPU_OK) return st;
  return read_status_md(c);
}

}  // namespace

extern "C" {

int pdgpu_md_setup(pdgpu_ctx* h, const pdgpu_md_params* p, const double* temps) {
  if (!h || !p || !temps) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.has_mass) return PDGPU_ERR_STATE;
  if (p->Timestep <= 0 || p->UpdateNList < 1 || p->UpdateSasa < 1 || (p->Integrator != 0 && p->Integrator != 1))
    return PDGPU_ERR_ARG;
  if (p->Integrator == 1 && p->FricCoeff * p->Timestep < 0.00001) return PDGPU_ERR_UNSUPPORTED;
  if ((p->what & PDGPU_NB) && !c.nb_set) return PDGPU_ERR_STATE;
  if ((p->what & PDGPU_GB) && (!c.has_gb || !c.gb_set)) return PDGPU_ERR_STATE;
  if ((p->what & PDGPU_SA) && !c.has_sa) return PDGPU_ERR_STATE;
  if ((p->what & (PDGPU_GB | PDGPU_SA)) && c.any_periodic) return PDGPU_ERR_UNSUPPORTED;
  if (!c.positions_set) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  destroy_md(c);
  c.md = new MDState();
  MDState& md = *c.md;
  md.p = *p;
  md.L = coeffs(p->FricCoeff, p->Timestep);
  const size_t N = c.natom;
  if (md.d_vel.alloc(3 * N) != cudaSuccess || md.d_mterms.alloc(N) != cudaSuccess || md.d_temp.alloc(c.nsys) != cudaSuccess ||
      md.d_ladder.alloc(c.nsys) != cudaSuccess || md.d_temp_sys.alloc(c.nsys) != cudaSuccess ||
      md.d_vscale.alloc(c.nsys) != cudaSuccess || md.d_accepted.alloc(c.nsys) != cudaSuccess ||
      md.d_ke.alloc(c.nsys) != cudaSuccess || md.d_ke_j.alloc(c.nsys) != cudaSuccess ||
      md.d_facc_sa.alloc(3 * (size_t)c.nslots) != cudaSuccess ||
      md.d_surf_cache.alloc(c.nsys) != cudaSuccess || md.d_step.alloc(1) != cudaSuccess || md.d_done.alloc(1) != cudaSuccess ||
      md.d_mode.alloc(c.nsys) != cudaSuccess || md.d_copy_src.alloc(c.nsys) != cudaSuccess ||
      md.d_copy_scale.alloc(c.nsys) != cudaSuccess || md.d_bad.alloc(c.nsys) != cudaSuccess)
    return PDGPU_ERR_CUDA;
  CK(cudaMemsetAsync(md.d_mode.p, 0, sizeof(int) * c.nsys, c.stream));
  std::vector<int> order(c.nsys);
  for (int s = 0; s < c.nsys; s++) order[s] = s;
  CK(cudaMemsetAsync(md.d_vel.p, 0, sizeof(double) * 3 * N, c.stream));
  k_mass_terms<<<(c.natom + 255) / 256, 256, 0, c.stream>>>(c.d_mass.p, md.d_mterms.p, c.natom);
  c.kernel_launches += 1;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(md.d_temp.p, temps, sizeof(double) * c.nsys, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(md.d_ladder.p, temps, sizeof(double) * c.nsys, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemcpyAsync(md.d_temp_sys.p, order.data(), sizeof(int) * c.nsys, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemsetAsync(md.d_facc_sa.p, 0, sizeof(long long) * 3 * c.nslots, c.stream));
  CK(cudaMemsetAsync(md.d_surf_cache.p, 0, sizeof(long long) * c.nsys, c.stream));
  CK(cudaMemsetAsync(md.d_ke.p, 0, sizeof(long long) * c.nsys, c.stream));
  CK(cudaMemsetAsync(md.d_step.p, 0, sizeof(unsigned long long), c.stream));
  CK(cudaMemsetAsync(md.d_done.p, 0, sizeof(unsigned), c.stream));
  CK(cudaStreamSynchronize(c.stream));
  md.ready = true;
  return PDGPU_OK;
}

int pdgpu_set_velocities(pdgpu_ctx* h, const double* v, size_t stride) {
  if (!h || !v || stride < 24 || stride % 8) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  CK(copy_xyz_rows(c.md->d_vel.p, 24, v, stride, c.natom, cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

int pdgpu_get_velocities(pdgpu_ctx* h, double* v, size_t stride) {
  if (!h || !v || stride < 24 || stride % 8) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  CK(copy_xyz_rows(v, stride, c.md->d_vel.p, 24, c.natom, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

int pdgpu_md_run(pdgpu_ctx* h, int nsteps, int energy_on_last) {
  if (!h || nsteps < 0) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md || !c.md->ready) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  return md_run_impl(c, *c.md, nsteps, energy_on_last != 0);
}

int pdgpu_md_enqueue(pdgpu_ctx* h, int nsteps, int energy_on_last) {
  if (!h || nsteps < 0) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md || !c.md->ready) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  return md_enqueue_impl(c, *c.md, nsteps, energy_on_last != 0);
}

int pdgpu_synchronize(pdgpu_ctx* h) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  int st = read_status_md(c);
  CK(cudaMemsetAsync(c.d_status.p, 0, sizeof(unsigned), c.stream));
  return st;
}

long long pdgpu_kernel_launches(pdgpu_ctx* h) { return h ? h->c.kernel_launches : -1; }

int pdgpu_time_kernel(pdgpu_ctx* h, int kernel, int reps, int flush_l2, double* avg_ms) {
  if (!h || reps < 1 || !avg_ms) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.list_built) return PDGPU_ERR_STATE;
  if (kernel == 5 && (!c.md || !c.md->ready)) return PDGPU_ERR_STATE;
  if ((kernel >= 1 && kernel <= 3) && !c.gb_set) return PDGPU_ERR_STATE;
  if (kernel == 0 && !c.nb_set) return PDGPU_ERR_STATE;
  if (kernel == 4 && !c.has_sa) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  DBuf<char> scratch;
  const size_t flush_bytes = (size_t)256 << 20;  // larger than the 126 MB L2
  if (flush_l2 && scratch.alloc(flush_bytes) != cudaSuccess) return PDGPU_ERR_CUDA;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float total = 0.f;
  int st = PDGPU_OK;
  for (int r = 0; r < reps && st == PDGPU_OK; r++) {
    if (flush_l2) CK(cudaMemsetAsync(scratch.p, r & 0xff, flush_bytes, c.stream));
    CK(cudaEventRecord(e0, c.stream));
    switch (kernel) {
      case 0: st = launch_nb(c, make_nb_const(c.nb), false); break;
      case 1: case 2: case 3: st = launch_gb_stage(c, make_gb_const(c.gb, c.list_radius_built), kernel); break;
      case 4: st = launch_lcpo(c, c.d_facc.p, nullptr, 0); break;
      case 5: st = launch_integrate(c, *c.md, false, false); break;
      case 6: st = launch_list_build(c, c.list_radius_built, c.full_radius_built, kListDevice); break;
      case 7: st = launch_pack(c, 0.f); break;
      case 8: st = launch_bonded(c, false); break;
      default: st = PDGPU_ERR_ARG;
    }
    CK(cudaEventRecord(e1, c.stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    total += ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *avg_ms = total / reps;
  return st;
}

int pdgpu_get_kinetic(pdgpu_ctx* h, double* ekin) {
  if (!h || !ekin) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  std::vector<long long> ke(c.nsys);
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(ke.data(), c.md->d_ke.p, sizeof(long long) * c.nsys, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (int s = 0; s < c.nsys; s++) ekin[s] = (double)ke[s] / kEnergyScale * kKcalMolToJ;
  return PDGPU_OK;
}

int pdgpu_get_kinetic_async(pdgpu_ctx* h, double* ekin) {
  if (!h || !ekin) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  MDState& md = *c.md;
  k_ke_joules<<<(c.nsys + 127) / 128, 128, 0, c.stream>>>(md.d_ke.p, md.d_ke_j.p, c.nsys);
  c.kernel_launches += 1;
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ekin, md.d_ke_j.p, sizeof(double) * c.nsys, cudaMemcpyDeviceToHost, c.stream));
  return PDGPU_OK;
}

int pdgpu_remd_exchange(pdgpu_ctx* h, int parity, int* accepted, double* temps) {
  if (!h || (parity != 0 && parity != 1)) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  MDState& md = *c.md;
  CK(cudaMemsetAsync(md.d_accepted.p, 0, sizeof(int) * c.nsys, c.stream));
  int st = launch_remd(c, md, parity, md.exchange_round++);
  if (st != PDGPU_OK) return st;
  std::vector<int> acc(c.nsys, 0);
  CK(cudaMemcpyAsync(acc.data(), md.d_accepted.p, sizeof(int) * c.nsys, cudaMemcpyDeviceToHost, c.stream));
  if (temps) CK(cudaMemcpyAsync(temps, md.d_temp.p, sizeof(double) * c.nsys, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (accepted && c.nsys > 1) std::copy(acc.begin(), acc.begin() + (c.nsys - 1), accepted);
  if (md.copy_modes) {
    // a copied structure jumped: new list (and skin reference) and LCPO at the next step
    bool any = false;
    for (int r = 0; r + 1 < c.nsys; r++) any = any || acc[r];
    if (any) {
      c.list_built = false;
      md.force_sasa = true;
    }
  }
  return PDGPU_OK;
}

int pdgpu_remd_set_modes(pdgpu_ctx* h, const int* modes) {
  if (!h || !modes) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  bool copy = false;
  for (int r = 0; r < c.nsys; r++) {
    if (modes[r] < PDGPU_REX_SWAP || modes[r] > PDGPU_REX_UPWARD) return PDGPU_ERR_ARG;
    copy = copy || modes[r] != PDGPU_REX_SWAP;
  }
  if (copy)
    for (int s = 1; s < c.nsys; s++)
      if (c.sys[s].natom != c.sys[0].natom) return PDGPU_ERR_UNSUPPORTED;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(c.md->d_mode.p, modes, sizeof(int) * c.nsys, cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  c.md->copy_modes = copy;
  return PDGPU_OK;
}

int pdgpu_md_set_trajectory(pdgpu_ctx* h, int every, double* host_ring, int nslots) {
  if (!h || every < 0 || (every > 0 && (!host_ring || nslots < 1))) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  c.md->traj_every = every;
  c.md->traj_ring = every > 0 ? host_ring : nullptr;
  c.md->traj_slots = every > 0 ? nslots : 0;
  c.md->traj_frames = 0;
  return PDGPU_OK;
}

long long pdgpu_md_trajectory_frames(pdgpu_ctx* h) {
  if (!h || !h->c.md) return -1;
  return h->c.md->traj_frames;
}

int pdgpu_md_checkpoint(pdgpu_ctx* h) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md) return PDGPU_ERR_STATE;
  MDState& md = *c.md;
  CK(cudaSetDevice(c.device));
  if (md.d_ckpt_pos.n < 3 * (size_t)c.natom && md.d_ckpt_pos.alloc(3 * (size_t)c.natom) != cudaSuccess)
    return PDGPU_ERR_CUDA;
  CK(cudaMemcpyAsync(md.d_ckpt_pos.p, c.d_pos.p, 24 * (size_t)c.natom, cudaMemcpyDeviceToDevice, c.stream));
  return PDGPU_OK;
}

int pdgpu_md_rescue(pdgpu_ctx* h, unsigned long long seed, int* rescued, int* count) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md || !c.md->d_ckpt_pos.p) return PDGPU_ERR_STATE;
  MDState& md = *c.md;
  CK(cudaSetDevice(c.device));
  std::vector<int> bad(c.nsys, 0);
  int st = launch_rescue(c, md, seed, bad.data());
  if (st != PDGPU_OK) return st;
  int n = 0;
  for (int s = 0; s < c.nsys; s++) n += bad[s] ? 1 : 0;
  if (rescued) std::copy(bad.begin(), bad.end(), rescued);
  if (count) *count = n;
  if (n) {
    c.list_built = false;
    md.force_sasa = true;
    CK(cudaMemsetAsync(c.d_status.p, 0, sizeof(unsigned), c.stream));
    CK(cudaStreamSynchronize(c.stream));
  }
  return PDGPU_OK;
}

int pdgpu_set_launch_shape(pdgpu_ctx* h, int ctas_per_sm) {
  if (!h || ctas_per_sm < 1 || ctas_per_sm > 64) return PDGPU_ERR_ARG;
  Context& c = h->c;
  c.tile_ctas_per_sm = ctas_per_sm;
  if (c.md) invalidate_graphs(*c.md);
  return PDGPU_OK;
}

int pdgpu_get_launch_shape(pdgpu_ctx* h, int* ctas_per_sm) {
  if (!h || !ctas_per_sm) return PDGPU_ERR_ARG;
  *ctas_per_sm = h->c.tile_ctas_per_sm;
  return PDGPU_OK;
}

int pdgpu_set_work_items(pdgpu_ctx* h, int tiles_per_item) {
  if (!h || (tiles_per_item != 1 && tiles_per_item != 2)) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (c.gb_item_tiles != tiles_per_item) {
    c.gb_item_tiles = tiles_per_item;
    c.list_built = false;  // the item list is written by the list build
    if (c.md) invalidate_graphs(*c.md);
  }
  return PDGPU_OK;
}

int pdgpu_get_work_items(pdgpu_ctx* h, int* tiles_per_item) {
  if (!h || !tiles_per_item) return PDGPU_ERR_ARG;
  *tiles_per_item = h->c.gb_item_tiles;
  return PDGPU_OK;
}

int pdgpu_set_nb_groups(pdgpu_ctx* h, int on) {
  if (!h || (on != 0 && on != 1)) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (c.nb_cull != (on != 0)) {
    c.nb_cull = on != 0;
    c.list_built = false;  // the groups are written by the list build
    if (c.md) invalidate_graphs(*c.md);
  }
  return PDGPU_OK;
}

int pdgpu_get_nb_groups(pdgpu_ctx* h, int* on, long long* ngroups, long long* nrest) {
  if (!h || !on) return PDGPU_ERR_ARG;
  Context& c = h->c;
  *on = c.nb_cull ? 1 : 0;
  long long g = 0, r = -1;
  if (c.list_built && c.cull_built) {
    CK(cudaSetDevice(c.device));
    int n[6];
    CK(cudaMemcpyAsync(n, c.d_counters.p, sizeof(n), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (n[5]) {
      g = n[4];
      r = n[3];
    }
  }
  if (ngroups) *ngroups = g;
  if (nrest) *nrest = r;
  return PDGPU_OK;
}

int pdgpu_md_autotune(pdgpu_ctx* h, int trial_steps, int* update_nlist, int* ctas_per_sm) {
  if (!h || trial_steps < 1) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.md || !c.md->ready) return PDGPU_ERR_STATE;
  MDState& md = *c.md;
  CK(cudaSetDevice(c.device));
  // save the state; every trial starts from it
  const size_t N3 = 3 * (size_t)c.natom;
  DBuf<double> pos0, vel0;
  if (pos0.alloc(N3) != cudaSuccess || vel0.alloc(N3) != cudaSuccess) return PDGPU_ERR_CUDA;
  CK(cudaMemcpyAsync(pos0.p, c.d_pos.p, N3 * 8, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(vel0.p, md.d_vel.p, N3 * 8, cudaMemcpyDeviceToDevice, c.stream));
  const unsigned long long step0 = md.step;
  const bool started0 = md.trajectory_started;
  const pdgpu_md_params p0 = md.p;
  std::vector<long long> sa0(3 * (size_t)c.nslots);
  CK(cudaMemcpyAsync(sa0.data(), md.d_facc_sa.p, sa0.size() * 8, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));

  // 1. work-item size of the GB kernels (single tiles or tile pairs) and launch
  //    shape of the tile kernels (grid = CTAs per SM x SMs): force evaluations on
  //    the saved state, timed with events
  const int shapes[] = {2, 4, 8, 16};
  const unsigned pair_what = md.p.what & (PDGPU_NB | PDGPU_GB);
  int best_s = c.tile_ctas_per_sm, best_items = c.gb_item_tiles;
  if (pair_what) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    const int n_items = (pair_what & PDGPU_GB) ? 2 : 1;
    for (int ii = 0; ii < n_items; ii++) {
      if (pair_what & PDGPU_GB) c.gb_item_tiles = 2 - ii;
      c.list_built = false;
      if (rebuild_list_impl(c) != PDGPU_OK) return PDGPU_ERR_CUDA;
      for (int shape : shapes) {
        c.tile_ctas_per_sm = shape;
        float ms = 0.f;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; rep++) {  // first repetition warms up
          CK(cudaEventRecord(e0, c.stream));
          ok = enqueue_forces(c, pair_what, false, false, c.d_facc.p, nullptr, 0, false) == PDGPU_OK;
          CK(cudaEventRecord(e1, c.stream));
          CK(cudaEventSynchronize(e1));
          float t = 0.f;
          CK(cudaEventElapsedTime(&t, e0, e1));
          if (rep) ms += t;
        }
        if (ok && ms < best_ms) {
          best_ms = ms;
          best_s = shape;
          best_items = c.gb_item_tiles;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  c.tile_ctas_per_sm = best_s;
  c.gb_item_tiles = best_items;
  c.list_built = false;

  // 2. list cadence with that shape, with and without the NB j-atom groups (their
  //    build cost counts, per rebuild): short dynamics from the saved state
  const int cadences[] = {1, 2, 3, 5, 10, 20, 40, 80};
  const bool cull0 = c.nb_cull;
  const bool try_groups = (md.p.what & PDGPU_NB) && c.nb_set && c.cull_cap > 0 && c.lp.check_skin;
  double best = 1e300;
  int best_n = p0.UpdateNList;
  bool best_cull = cull0;
  for (int gi = 0; gi < (try_groups ? 2 : 1); gi++) {
    if (try_groups) c.nb_cull = gi == 0;
    for (int n : cadences) {
      md.p.UpdateNList = n;
      invalidate_graphs(md);
      CK(cudaMemcpyAsync(c.d_pos.p, pos0.p, N3 * 8, cudaMemcpyDeviceToDevice, c.stream));
      CK(cudaMemcpyAsync(md.d_vel.p, vel0.p, N3 * 8, cudaMemcpyDeviceToDevice, c.stream));
      md.step = step0;
      md.trajectory_started = started0;
      c.list_built = false;
      int warm = std::min(trial_steps, n);
      if (md_run_impl(c, md, warm, false) != PDGPU_OK) continue;
      // whole rebuild windows, so every cadence pays its list builds; per step
      const int timed = (trial_steps + n - 1) / n * n;
      auto t0 = std::chrono::steady_clock::now();
      int st = md_run_impl(c, md, timed, false);
      auto t1 = std::chrono::steady_clock::now();
      if (st != PDGPU_OK) continue;  // stale list (or worse): cadence too long
      // the cadence must also survive a longer stretch (4 rebuild windows)
      if (md_run_impl(c, md, 4 * n, false) != PDGPU_OK) continue;
      double dt = std::chrono::duration<double>(t1 - t0).count() / timed;
      if (dt < best) {
        best = dt;
        best_n = n;
        best_cull = c.nb_cull;
      }
    }
  }
  c.nb_cull = best >= 1e300 ? cull0 : best_cull;
  // restore the state and keep the winner
  md.p = p0;
  md.p.UpdateNList = best_n;
  invalidate_graphs(md);
  CK(cudaMemcpyAsync(c.d_pos.p, pos0.p, N3 * 8, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(md.d_vel.p, vel0.p, N3 * 8, cudaMemcpyDeviceToDevice, c.stream));
  CK(cudaMemcpyAsync(md.d_facc_sa.p, sa0.data(), sa0.size() * 8, cudaMemcpyHostToDevice, c.stream));
  CK(cudaMemsetAsync(md.d_step.p, 0, sizeof(unsigned long long), c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (step0) {
    // restore the device step counter too
    CK(cudaMemcpy(md.d_step.p, &step0, sizeof(step0), cudaMemcpyHostToDevice));
  }
  md.step = step0;
  md.trajectory_started = started0;
  c.list_built = false;
  if (best >= 1e300) return PDGPU_ERR_STALE_LIST;
  if (update_nlist) *update_nlist = best_n;
  if (ctas_per_sm) *ctas_per_sm = best_s;
  return PDGPU_OK;
}

}  // extern "C"
