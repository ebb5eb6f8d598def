// pdgpu_md.cuh — device state of molecular dynamics / REMD on a context.
#pragma once
#include <map>

#include "pdgpu_context.cuh"

namespace pdgpu {

// Langevin coefficients (md.cpp:941-1003), FP64
struct LangevinCoeffs {
  double dt, gamma, gt, c0, c1, c2, varv, varr, crv, sq1mcrv2;
  double kick, drift_f, sv, sr;   // (1 - c0/c1)/gt, c0 c2 / c1, sqrt(varv), sqrt(varr)/gamma
};

struct MDState {
  bool ready = false;
  pdgpu_md_params p{};
  LangevinCoeffs L{};
  unsigned long long step = 0;        // global step counter (RNG counter, cadences)
  unsigned long long exchange_round = 0;
  bool trajectory_started = false;
  DBuf<double> d_vel;                 // [natom*3] m/s
  DBuf<double2> d_mterms;             // [natom] (1 / mass, sqrt(k_B / mass)), SI
  DBuf<unsigned long long> d_step;    // [1] device copy of the step counter
  DBuf<unsigned> d_done;              // [1] integrator blocks finished in the running launch (0 between launches)
  DBuf<double> d_temp;                // [nsys] target temperature of each system (K)
  DBuf<double> d_ladder;              // [nsys] temperature of each rung (K)
  DBuf<int> d_temp_sys;               // [nsys] system holding each rung
  DBuf<double> d_vscale;              // [nsys]
  DBuf<int> d_accepted;               // [nsys]
  DBuf<long long> d_ke;               // [nsys] kinetic energy, fixed point kcal/mol
  DBuf<double> d_ke_j;                // [nsys] the same in J (asynchronous reads)
  DBuf<long long> d_facc_sa;          // [nslots*3] cached LCPO forces
  DBuf<long long> d_surf_cache;       // [nsys] cached LCPO energy
  DBuf<int> d_mode;                   // [nsys] exchange mode of each rung's lower replica (0 swap, 1 down, 2 up)
  DBuf<int> d_copy_src;               // [nsys] structure source of each system in the last sweep (-1 none)
  DBuf<double> d_copy_scale;          // [nsys] velocity factor of copied structures
  DBuf<double> d_ckpt_pos;            // [natom*3] positions at the last checkpoint (crash rescue)
  DBuf<int> d_bad;                    // [nsys] systems flagged non-finite
  bool copy_modes = false;            // some rung copies structures (list and LCPO cache refreshed after)
  // trajectory frames copied to a caller's host ring without a synchronisation
  int traj_every = 0;
  double* traj_ring = nullptr;
  int traj_slots = 0;
  long long traj_frames = 0;
  bool force_sasa = false;            // recompute LCPO at the next step
  std::map<int, cudaGraphExec_t> graphs;
  std::map<int, long long> graph_kernels;  // kernel nodes of each captured flavour
};

struct MDView {
  int natom;
  const int* slot_of;
  const int* atom_sys;
  const double* mass;
  const double2* mterms;     // (1 / mass, sqrt(k_B / mass)): no FP64 divide or root per step
  double* pos;
  double* vel;
  const double* temp;
  const long long* facc;
  const long long* facc_sa;   // may be null
  long long* ke;
  unsigned long long seed;
  unsigned long long* stepc;   // read by every block; the last block to finish advances it
  unsigned* done;
};

inline MDView md_view(Context& c, MDState& md) {
  MDView m;
  m.natom = c.natom;
  m.slot_of = c.d_slot_of.p;
  m.atom_sys = c.d_atom_sys.p;
  m.mass = c.d_mass.p;
  m.mterms = md.d_mterms.p;
  m.pos = c.d_pos.p;
  m.vel = md.d_vel.p;
  m.temp = md.d_temp.p;
  m.facc = c.d_facc.p;
  m.facc_sa = (md.p.what & PDGPU_SA) ? md.d_facc_sa.p : nullptr;
  m.ke = md.d_ke.p;
  m.seed = md.p.seed;
  m.stepc = md.d_step.p;
  m.done = md.d_done.p;
  return m;
}

int launch_integrate(Context& c, MDState& md, bool first, bool last);
int launch_remd(Context& c, MDState& md, int parity, unsigned long long round);
int launch_zero_ll(Context& c, long long* p, size_t n);
// crash rescue: flags non-finite systems into bad_host (nsys ints, synchronous)
// and restores them from the checkpoint with fresh velocities
int launch_rescue(Context& c, MDState& md, unsigned long long seed, int* bad_host);

}  // namespace pdgpu
