// pdgpu_api.cu — the C ABI declared in include/pdgpu.h.
//
// Host orchestration only: validation, parameter conversion to the internal
// units (kcal/mol, Angstrom), buffer management and the launch sequence of one
// evaluation.  No function throws; errors come back as status codes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "pdgpu_context.cuh"

using namespace pdgpu;

struct pdgpu_ctx {
  Context c;
};

namespace {

int cuda_status(cudaError_t e, Context* c = nullptr, const char* what = "") {
  if (e == cudaSuccess) return PDGPU_OK;
  if (c) {
    c->last_error = PDGPU_ERR_CUDA;
    c->last_msg = std::string(what) + ": " + cudaGetErrorString(e);
  }
  return PDGPU_ERR_CUDA;
}

#define CK(expr)                                              \
  do {                                                        \
    cudaError_t _e = (expr);                                  \
    if (_e != cudaSuccess) return cuda_status(_e, &c, #expr); \
  } while (0)

template <typename T>
cudaError_t upload(DBuf<T>& b, const T* h, size_t n) {
  cudaError_t e = b.alloc(n);
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpy(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice);
}

// The GB object's FF_NonBonded settings: as set, else PD's defaults for the GB
// object (its cutoffs and 1-4 scalings, Dielectric 1, energy switch).
pdgpu_nb_params gb_vacuum_params(const Context& c) {
  if (c.gb_vac_set) return c.gb_vac;
  pdgpu_nb_params p{};
  p.Cutoff = c.gb.Cutoff;
  p.InnerCutoff = c.gb.InnerCutoff;
  p.VdwCutoff = c.gb.VdwCutoff;
  p.VdwInnerCutoff = c.gb.VdwInnerCutoff;
  p.Vdw14Scaling = c.gb.Vdw14Scaling;
  p.Elec14Scaling = c.gb.Elec14Scaling;
  p.Dielectric = 1.0;
  p.EnergySwitch = 1;
  p.ForceSwitch = 0;
  p.DoVdw = 1;
  p.DoElec = 1;
  return p;
}

double list_radius(const Context& c) {
  double r = 0;
  if (c.nb_set) r = std::max(r, std::max(c.nb.Cutoff, c.nb.VdwCutoff));
  if (c.gb_set) r = std::max(r, std::max(c.gb.Cutoff, c.gb.VdwCutoff));
  if (c.has_sa) r = std::max(r, 7.0);  // FF_SASA_LCPO::setup requests 7 A (lcpo.cpp:37)
  return r + c.lp.Padding;
}

// Distance below which no cutoff or switch of the set components acts (tiles
// entirely inside it skip those tests); 0 when the skin check is off, since the
// full-tile margin is only guaranteed by the per-step displacement check.
double full_radius(const Context& c) {
  if (!c.lp.check_skin || (!c.nb_set && !c.gb_set)) return 0.0;
  double r = 1e300;
  if (c.nb_set) r = std::min(r, std::min(c.nb.InnerCutoff, c.nb.VdwInnerCutoff));
  if (c.gb_set) r = std::min(r, std::min(std::min(c.gb.InnerCutoff, c.gb.VdwInnerCutoff), c.gb.GbsaStillCutoff));
  return r;
}

int read_status(Context& c) {
  unsigned st = 0;
  cudaError_t e = cudaMemcpyAsync(&st, c.d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return cuda_status(e, &c, "status");
  if (st & ST_NAN) return PDGPU_ERR_NAN;
  if (st & ST_FIXED_OVERFLOW) return PDGPU_ERR_FIXED_OVERFLOW;
  if (st & (ST_LCPO_OVERFLOW | ST_TILE_OVERFLOW)) return PDGPU_ERR_LIST_OVERFLOW;
  if (st & ST_STALE_LIST) return PDGPU_ERR_STALE_LIST;
  return PDGPU_OK;
}

}  // namespace

NBConst pdgpu::make_nb_const(const pdgpu_nb_params& p) {
  NBConst k{};
  double C = p.Cutoff, I = p.InnerCutoff;
  k.cut2 = (float)(C * C);
  k.cut2_dd = C * C;
  k.vdwcut2 = (float)(p.VdwCutoff * p.VdwCutoff);
  k.vdwcut_d = p.VdwCutoff;
  k.vdwinner_d = p.VdwInnerCutoff;
  k.inner_d = I;
  double vw = p.VdwCutoff - p.VdwInnerCutoff, w = C - I;
  k.vdwinvw2_d = vw > 0 ? 1.0 / (vw * vw) : 0.0;
  k.invw2_d = w > 0 ? 1.0 / (w * w) : 0.0;
  k.econv_diel_d = econv_kcal() / p.Dielectric;
  k.econv_diel = (float)k.econv_diel_d;
  k.vdw14 = (float)p.Vdw14Scaling;
  k.elec14 = (float)p.Elec14Scaling;
  k.vdw14_d = p.Vdw14Scaling;
  k.elec14_d = p.Elec14Scaling;
  // Steinbach-Brooks force-switch constants (nonbonded.cpp:620-636)
  double C2 = C * C, I2 = I * I;
  k.sA = 1.0 / ((C2 - I2) * (C2 - I2) * (C2 - I2));
  k.sB = -(C2 * C2 * C2 - 3.0 * C2 * C2 * I2);
  k.sC = 6.0 * C2 * I2;
  k.sD = -(C2 + I2);
  k.sE = 2.0 / 5.0;
  double innerV = k.sA * (k.sB / I + k.sC * I + k.sD * I * I * I + k.sE * I * I * I * I * I);
  k.fsw_cutV = k.sA * (k.sB / C + k.sC * C + k.sD * C * C * C + k.sE * C * C * C * C * C);
  k.eshift = I < C ? 1.0 / I + (innerV - k.fsw_cutV) : 0.0;
  k.cut2_d = C2;
  k.inner2_d = I2;
  k.vdwcut_f = (float)p.VdwCutoff;
  k.vdwinner_f = (float)p.VdwInnerCutoff;
  k.vdwinvw2_f = (float)k.vdwinvw2_d;
  k.inner_f = (float)I;
  k.invw2_f = (float)k.invw2_d;
  k.inner2_f = (float)I2;
  k.sA_f = (float)k.sA;
  k.fsw_k = (float)(C2 - 3.0 * I2);
  k.elecmode = 1;
  if (p.EnergySwitch) k.elecmode = 3;
  if (p.ForceSwitch) k.elecmode = 4;
  if (!p.DoElec) k.elecmode = 0;
  k.dovdw = p.DoVdw ? 1 : 0;
  k.samesw = (k.elecmode == 3 && k.dovdw && p.VdwCutoff == p.Cutoff && p.VdwInnerCutoff == p.InnerCutoff) ? 1 : 0;
  return k;
}

GBConst pdgpu::make_gb_const(const pdgpu_gb_params& p, double listR) {
  GBConst k{};
  double C = p.Cutoff, I = p.InnerCutoff;
  k.cut2 = (float)(C * C);
  k.inner = (float)I;
  double w = C - I, vw = p.VdwCutoff - p.VdwInnerCutoff;
  k.invw2 = w > 0 ? (float)(1.0 / (w * w)) : 0.f;
  k.vdwcut = (float)p.VdwCutoff;
  k.vdwinner = (float)p.VdwInnerCutoff;
  k.vdwinvw2 = vw > 0 ? (float)(1.0 / (vw * vw)) : 0.f;
  double still = std::min(p.GbsaStillCutoff, listR);
  k.still2 = (float)(still * still);
  double ec = econv_kcal();
  k.econv_in = (float)(ec / p.DielectricSolute);
  k.econv_out = (float)(ec / p.DielectricSolvent);
  k.premul = (float)(-0.5 * ec * (1.0 / p.DielectricSolute - 1.0 / p.DielectricSolvent));
  k.vdw14 = (float)p.Vdw14Scaling;
  k.elec14 = (float)p.Elec14Scaling;
  k.thresh = (float)p.ExpApproxThreshold;
  k.P4 = (float)p.P4;
  k.P5 = (float)p.P5;
  k.invP5 = (float)(1.0 / p.P5);
  k.cut2_d = C * C;
  k.inner_d = I;
  k.invw2_d = w > 0 ? 1.0 / (w * w) : 0.0;
  k.vdwcut_d = p.VdwCutoff;
  k.vdwinner_d = p.VdwInnerCutoff;
  k.vdwinvw2_d = vw > 0 ? 1.0 / (vw * vw) : 0.0;
  k.still2_d = still * still;
  k.econv_in_d = ec / p.DielectricSolute;
  k.econv_out_d = ec / p.DielectricSolvent;
  k.premul_d = -0.5 * ec * (1.0 / p.DielectricSolute - 1.0 / p.DielectricSolvent);
  k.vdw14_d = p.Vdw14Scaling;
  k.elec14_d = p.Elec14Scaling;
  k.thresh_d = p.ExpApproxThreshold;
  k.fast = 1;
  k.e64_r2 = 4.5f * 4.5f;
  const double K = -4.0 * (p.ExpApproxThreshold - 4e-6 * std::fabs(p.ExpApproxThreshold));
  k.sqrtK = K > 0 ? (float)std::sqrt(std::min(K, 1e36)) : 0.f;
  k.inv_sqrtK = K > 0 ? (float)(1.0 / std::sqrt(std::min(K, 1e36))) : 0.f;
  k.sq_eout = (float)std::sqrt(ec / p.DielectricSolvent);
  k.inv_eout = (float)(p.DielectricSolvent / ec);
  k.in_over_out_m1 = (float)(p.DielectricSolvent / p.DielectricSolute - 1.0);
  k.sqrt12 = (float)std::sqrt(12.0);
  return k;
}



extern "C" {

const char* pdgpu_error_string(int status) {
  switch (status) {
    case PDGPU_OK: return "ok";
    case PDGPU_ERR_ARG: return "invalid argument";
    case PDGPU_ERR_CUDA: return "CUDA runtime error";
    case PDGPU_ERR_LIST_OVERFLOW: return "LCPO overlap list or tile list overflow";
    case PDGPU_ERR_FIXED_OVERFLOW: return "fixed-point accumulator overflow";
    case PDGPU_ERR_NAN: return "NaN energy or force";
    case PDGPU_ERR_TIMEOUT: return "device wait timed out";
    case PDGPU_ERR_UNSUPPORTED: return "unsupported option";
    case PDGPU_ERR_STALE_LIST: return "an atom moved more than Padding/2 since the list was built";
    case PDGPU_ERR_STATE: return "call sequence error";
    case PDGPU_ERR_CAPACITY: return "beyond what the allocation-free entry point holds (static scratch or list arrays)";
    default: return "unknown status";
  }
}

pdgpu_ctx* pdgpu_create(int device, const pdgpu_system_desc* d, int* status) {
  auto fail = [&](int st) -> pdgpu_ctx* {
    if (status) *status = st;
    return nullptr;
  };
  if (!d || d->nsystems < 1 || !d->natoms || !d->box || !d->charge || !d->radius || !d->epsilon)
    return fail(PDGPU_ERR_ARG);
  if (cudaSetDevice(device) != cudaSuccess) return fail(PDGPU_ERR_CUDA);
  pdgpu_ctx* h = new (std::nothrow) pdgpu_ctx();
  if (!h) return fail(PDGPU_ERR_ARG);
  Context& c = h->c;
  c.device = device;
  auto bad = [&](int st) -> pdgpu_ctx* {
    release_streams(c);
    delete h;
    return fail(st);
  };
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming) != cudaSuccess)
    return bad(PDGPU_ERR_CUDA);

  // systems and padded layout
  c.nsys = d->nsystems;
  int atom = 0, slot = 0, block = 0;
  long long pairs = 0;
  c.any_periodic = false;
  c.all_periodic = true;
  for (int s = 0; s < c.nsys; s++) {
    if (d->natoms[s] < 1) return bad(PDGPU_ERR_ARG);
    SystemInfo S{};
    S.atom_start = atom;
    S.natom = d->natoms[s];
    S.pad_start = slot;
    S.npad = (S.natom + 31) / 32 * 32;
    S.block_start = block;
    S.nblocks = S.npad / 32;
    S.grid_start = block;   // one grid cell per block
    S.grid_cells = S.nblocks;
    if (S.nblocks > kMaxSystemBlocks) return bad(PDGPU_ERR_CAPACITY);
    int per = 0;
    for (int k = 0; k < 3; k++) {
      S.box[k] = d->box[3 * s + k];
      S.ibox[k] = S.box[k] > 0 ? 1.0 / S.box[k] : 0.0;
      if (S.box[k] > 0) per++;
    }
    if (per != 0 && per != 3) return bad(PDGPU_ERR_ARG);
    S.periodic = per == 3;
    c.any_periodic |= S.periodic;
    c.all_periodic &= S.periodic;
    c.sys.push_back(S);
    atom += S.natom;
    slot += S.npad;
    block += S.nblocks;
    pairs += (long long)S.nblocks * (S.nblocks + 1) / 2;
    c.max_sys_blocks = std::max(c.max_sys_blocks, S.nblocks);
  }
  c.natom = atom;
  c.nslots = slot;
  c.nblocks = block;
  c.npairs_all = pairs;
  // the list build counts tiles in 32-bit integers
  if (pairs > 2147483647LL) return bad(PDGPU_ERR_CAPACITY);
  const int N = c.natom;

  c.h_atom_sys.resize(N);
  std::vector<int> block_sys(c.nblocks);
  for (int s = 0; s < c.nsys; s++) {
    for (int a = 0; a < c.sys[s].natom; a++) c.h_atom_sys[c.sys[s].atom_start + a] = s;
    for (int b = 0; b < c.sys[s].nblocks; b++) block_sys[c.sys[s].block_start + b] = s;
  }

  // per-atom parameters in internal units
  const double sq = std::sqrt(kNa / kKcal2J);  // sqrt(J) -> sqrt(kcal/mol)
  std::vector<double> sqeps(N);
  for (int a = 0; a < N; a++) sqeps[a] = d->epsilon[a] * sq;

  // bonded pairs: band masks (|i-j| <= 64) and a far list
  std::vector<unsigned long long> bex(N, 0ull), b14(N, 0ull);
  std::vector<std::vector<std::pair<int, int>>> far(N);
  for (int k = 0; k < d->nexcl; k++) {
    int i = d->excl[3 * k], j = d->excl[3 * k + 1], bo = d->excl[3 * k + 2];
    if (i < 0 || j < 0 || i >= N || j >= N || c.h_atom_sys[i] != c.h_atom_sys[j]) return bad(PDGPU_ERR_ARG);
    int lo = std::min(i, j), hi = std::max(i, j), dd = hi - lo;
    if (dd == 0 || bo > 3) continue;
    if (dd <= kBandWidth) {
      unsigned long long bit = 1ull << (dd - 1);
      if (bo <= 2) bex[lo] |= bit;
      else b14[lo] |= bit;
    } else {
      far[lo].push_back(std::make_pair(hi, bo));
    }
  }
  std::vector<int> fstart(N + 1, 0), fidx, fbo;
  for (int a = 0; a < N; a++) {
    fstart[a + 1] = fstart[a] + (int)far[a].size();
    for (auto& p : far[a]) {
      fidx.push_back(p.first);
      fbo.push_back(p.second);
    }
  }
  // exclusion-mask table: a tile gets a mask only when it is diagonal, holds a
  // padding slot (the last block of a system) or a bonded pair, so this bounds
  // the masks of any list
  {
    long long bonded = (long long)fidx.size();
    for (int a = 0; a < N; a++) bonded += __builtin_popcountll(bex[a] | b14[a]);
    long long cap = c.nblocks + bonded;
    for (const SystemInfo& S : c.sys)
      if (S.natom != S.npad) cap += S.nblocks;
    c.mask_cap = (int)std::min(std::min(cap, c.npairs_all), 2147483647LL / 32);
  }
  if (fidx.empty()) {
    fidx.push_back(-1);
    fbo.push_back(7);
  }

  cudaError_t e = cudaSuccess;
#define UP(buf, ptr, n) \
  if (e == cudaSuccess) e = upload(buf, ptr, n)
  UP(c.d_sys, c.sys.data(), c.sys.size());
  UP(c.d_atom_sys, c.h_atom_sys.data(), (size_t)N);
  UP(c.d_block_sys, block_sys.data(), block_sys.size());
  UP(c.d_charge, d->charge, (size_t)N);
  UP(c.d_radius, d->radius, (size_t)N);
  UP(c.d_sqeps, sqeps.data(), (size_t)N);
  UP(c.d_band_excl, bex.data(), (size_t)N);
  UP(c.d_band_14, b14.data(), (size_t)N);
  UP(c.d_far_start, fstart.data(), fstart.size());
  UP(c.d_far_idx, fidx.data(), fidx.size());
  UP(c.d_far_bo, fbo.data(), fbo.size());
  if (d->mass) {
    UP(c.d_mass, d->mass, (size_t)N);
    c.has_mass = true;
  }
  if (d->gb_radius && d->gb_vj && d->gb_terms123) {
    c.has_gb = true;
    UP(c.d_gbR, d->gb_radius, (size_t)N);
    UP(c.d_gbVj, d->gb_vj, (size_t)N);
    UP(c.d_gbT, d->gb_terms123, (size_t)N);
  }
  if (d->lcpo_radius && d->lcpo_p && d->lcpo_sigma && d->lcpo_use) {
    c.has_sa = true;
    std::vector<double> sig(N);
    for (int a = 0; a < N; a++) sig[a] = d->lcpo_sigma[a] * (kNa / kKcal2J);
    UP(c.d_lcpoR, d->lcpo_radius, (size_t)N);
    UP(c.d_lcpoP, d->lcpo_p, (size_t)N * 4);
    UP(c.d_lcpoSig, sig.data(), (size_t)N);
    UP(c.d_lcpoUse, d->lcpo_use, (size_t)N);
  }
  // bonded terms, energies converted from J to kcal/mol
  const double J2k = kNa / kKcal2J;
  c.nbond = std::max(0, d->nbond);
  c.nangle = std::max(0, d->nangle);
  c.ntors = std::max(0, d->ntors);
  c.nimpr = std::max(0, d->nimpr);
  if (c.nbond && (!d->bond_idx || !d->bond_par)) return bad(PDGPU_ERR_ARG);
  if (c.nangle && (!d->angle_idx || !d->angle_par)) return bad(PDGPU_ERR_ARG);
  if (c.ntors && (!d->tors_idx || !d->tors_par)) return bad(PDGPU_ERR_ARG);
  if (c.nimpr && (!d->impr_idx || !d->impr_par)) return bad(PDGPU_ERR_ARG);
  {
    // every bonded index must name an atom of this batch
    auto in_range = [&](const int* idx, int count, int width, int used) {
      for (int k = 0; k < count; k++)
        for (int w = 0; w < used; w++)
          if (idx[(size_t)k * width + w] < 0 || idx[(size_t)k * width + w] >= N) return false;
      return true;
    };
    if (!in_range(d->bond_idx, c.nbond, 2, 2) || !in_range(d->angle_idx, c.nangle, 3, 3) ||
        !in_range(d->tors_idx, c.ntors, 5, 4) || !in_range(d->impr_idx, c.nimpr, 5, 4))
      return bad(PDGPU_ERR_ARG);
    for (int k = 0; k < c.ntors; k++)
      if (d->tors_idx[5 * k + 4] < 0 || d->tors_idx[5 * k + 4] > 4) return bad(PDGPU_ERR_ARG);
    for (int k = 0; k < c.nimpr; k++)
      if (d->impr_idx[5 * k + 4] < 0 || d->impr_idx[5 * k + 4] > 4) return bad(PDGPU_ERR_ARG);
  }
  {
    std::vector<double> bp(2 * (size_t)c.nbond), ap(2 * (size_t)c.nangle), tp(12 * (size_t)c.ntors),
        ip(12 * (size_t)c.nimpr);
    for (int k = 0; k < c.nbond; k++) {
      bp[2 * k] = d->bond_par[2 * k];
      bp[2 * k + 1] = d->bond_par[2 * k + 1] * J2k;
    }
    for (int k = 0; k < c.nangle; k++) {
      ap[2 * k] = d->angle_par[2 * k];
      ap[2 * k + 1] = d->angle_par[2 * k + 1] * J2k;
    }
    for (int k = 0; k < c.ntors; k++)
      for (int t = 0; t < 4; t++) {
        tp[12 * k + 3 * t] = d->tors_par[12 * k + 3 * t] * J2k;
        tp[12 * k + 3 * t + 1] = d->tors_par[12 * k + 3 * t + 1];
        tp[12 * k + 3 * t + 2] = d->tors_par[12 * k + 3 * t + 2];
      }
    for (int k = 0; k < c.nimpr; k++)
      for (int t = 0; t < 4; t++) {
        ip[12 * k + 3 * t] = d->impr_par[12 * k + 3 * t] * J2k;
        ip[12 * k + 3 * t + 1] = d->impr_par[12 * k + 3 * t + 1];
        ip[12 * k + 3 * t + 2] = d->impr_par[12 * k + 3 * t + 2];
      }
    UP(c.d_bidx, d->bond_idx, 2 * (size_t)c.nbond);
    UP(c.d_bpar, bp.data(), bp.size());
    UP(c.d_aidx, d->angle_idx, 3 * (size_t)c.nangle);
    UP(c.d_apar, ap.data(), ap.size());
    UP(c.d_tidx, d->tors_idx, 5 * (size_t)c.ntors);
    UP(c.d_tpar, tp.data(), tp.size());
    UP(c.d_iidx, d->impr_idx, 5 * (size_t)c.nimpr);
    UP(c.d_ipar, ip.data(), ip.size());
    c.has_bonded = c.nbond + c.nangle + c.ntors + c.nimpr > 0;
  }
#undef UP

  // dynamic buffers
  const size_t ncells = (size_t)c.nsys * kCellsPerSystem;
  const size_t nsb = (ncells + 1023) / 1024;
  if (e == cudaSuccess) e = c.d_pos.alloc(3 * (size_t)N);
  if (e == cudaSuccess) e = c.d_fout.alloc(3 * (size_t)N);
  if (e == cudaSuccess) e = c.d_bucket.alloc(N);
  if (e == cudaSuccess) e = c.d_count.alloc(ncells);
  if (e == cudaSuccess) e = c.d_offset.alloc(ncells);
  if (e == cudaSuccess) e = c.d_cursor.alloc(ncells);
  if (e == cudaSuccess) e = c.d_scan_tmp.alloc(nsb + 1);
  if (e == cudaSuccess) e = c.d_tmp_sorted.alloc(N);
  if (e == cudaSuccess) e = c.d_sys_lo.alloc(3 * (size_t)c.nsys);
  if (e == cudaSuccess) e = c.d_sys_hi.alloc(3 * (size_t)c.nsys);
  if (e == cudaSuccess) e = c.d_sys_hmax.alloc(3 * (size_t)c.nsys);
  if (e == cudaSuccess) e = c.d_bgrid.alloc(c.nsys);
  if (e == cudaSuccess) e = c.d_bcell.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_bcell_count.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_bcell_off.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_bcell_cursor.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_bcell_scan_tmp.alloc((c.nblocks + 1023) / 1024 + 1);
  if (e == cudaSuccess) e = c.d_bcell_blocks.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_row_cnt.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_row_start.alloc(c.nblocks);
  if (e == cudaSuccess) e = c.d_sorted_atom.alloc(c.nslots);
  if (e == cudaSuccess) e = c.d_slot_of.alloc(N);
  if (e == cudaSuccess) e = c.d_center.alloc(3 * (size_t)c.nblocks);
  if (e == cudaSuccess) e = c.d_half.alloc(c.nblocks);
  // (the tile arrays are sized by the first list build, from its tile count)
  if (e == cudaSuccess) e = c.d_counters.alloc(8);
  if (e == cudaSuccess) e = cudaMemset(c.d_counters.p, 0, sizeof(int) * 8);
  if (e == cudaSuccess) e = c.d_masks.alloc((size_t)c.mask_cap * 32);
  if (e == cudaSuccess) e = c.d_mlist.alloc(c.mask_cap);
  if (e == cudaSuccess) e = c.d_xq.alloc(c.nslots);
  if (e == cudaSuccess) e = c.d_par.alloc(c.nslots);
  if (e == cudaSuccess) e = c.d_rel0.alloc(c.nslots);
  if (e == cudaSuccess) e = c.d_facc.alloc(3 * (size_t)c.nslots);
  if (e == cudaSuccess) e = c.d_eacc.alloc((size_t)c.nsys * E_NSLOTS);
  if (e == cudaSuccess) e = c.d_status.alloc(1);
  if (c.has_gb) {
    if (e == cudaSuccess) e = c.d_gpol.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_deda.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_born_f.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_chain_f.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_born_d.alloc(N);
    if (e == cudaSuccess) e = c.d_epos.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_epar.alloc(c.nslots);
  }
  if (c.has_sa) {
    if (e == cudaSuccess) e = c.d_lc_ncand.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_lc_cand.alloc((size_t)c.nslots * kLcpoCand);
    if (e == cudaSuccess) e = c.d_lc_n.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_lc_e2.alloc((size_t)c.nslots * kLcpoMax);
    if (e == cudaSuccess) e = c.d_lc_ent.alloc((size_t)c.nslots * kLcpoMax);
    if (e == cudaSuccess) e = c.d_lc_psig.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_lc_box.alloc((size_t)c.nblocks * 2);
    if (e == cudaSuccess) e = c.d_sasa.alloc(N);
    if (e == cudaSuccess) e = c.d_lc_par.alloc(c.nslots);
    if (e == cudaSuccess) e = c.d_lc_pos.alloc(c.nslots);
  }
  if (e == cudaSuccess) e = cudaMemset(c.d_status.p, 0, sizeof(unsigned));
  if (e != cudaSuccess) return bad(PDGPU_ERR_CUDA);
  c.h_eacc.resize((size_t)c.nsys * E_NSLOTS);

  // PD defaults: FF_NonBonded::settodefault (nonbonded.cpp:985-1021),
  // FF_GeneralizedBorn_Still constructor (gbff.cpp:33-55), NeighbourList Padding 0.5
  c.nb = pdgpu_nb_params{15.0, 12.0, 15.0, 12.0, 1.0, 1.0, 1.0, 0, 1, 1, 1};
  c.gb = pdgpu_gb_params{15.0, 12.0, 15.0, 12.0, 1.0, 1.0, 1.0, 80.0, 10.0, -4.0, 0.0, 15.236, 1.254};
  c.lp = pdgpu_list_params{0.5, 1};
  if (status) *status = PDGPU_OK;
  return h;
}

int pdgpu_destroy(pdgpu_ctx* h) {
  if (!h) return PDGPU_ERR_ARG;
  cudaSetDevice(h->c.device);
  if (h->c.stream) cudaStreamSynchronize(h->c.stream);
  if (h->c.side) cudaStreamSynchronize(h->c.side);
  destroy_md(h->c);
  // the streams and events outlive the context's device buffers
  cudaStream_t st = h->c.stream, side = h->c.side;
  cudaEvent_t a = h->c.ev_fork, b = h->c.ev_join;
  h->c.stream = h->c.side = nullptr;
  h->c.ev_fork = h->c.ev_join = nullptr;
  delete h;
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (side) cudaStreamDestroy(side);
  if (st) cudaStreamDestroy(st);
  return PDGPU_OK;
}

}  // extern "C"

// the first positions of a context with its parameters set build the list,
// which sizes the tile arrays (later builds reuse them, growing only when the
// tile count outgrows them), so that calls which may not allocate find them
static int size_list(Context& c) {
  if (c.tile_cap > 0 || (!c.nb_set && !c.gb_set && !c.has_sa)) return PDGPU_OK;
  return rebuild_list_impl(c);
}

// NB j-atom group buffers: the per-row arrays with the NB parameters (never
// inside a stream capture), the per-tile ones with the tile arrays
static int alloc_cull(Context& c) {
  if (c.d_cull_row.p) return PDGPU_OK;
  cudaError_t e = cudaSetDevice(c.device);
  if (e == cudaSuccess) e = c.d_cull_row.alloc(4 * (size_t)c.nblocks);
  if (e == cudaSuccess) e = c.d_cull_scan_tmp.alloc((c.nblocks + 1023) / 1024 + 1);
  if (e != cudaSuccess) {
    c.d_cull_row.release();
    c.d_cull_scan_tmp.release();
    cudaGetLastError();
    return PDGPU_ERR_CUDA;
  }
  return c.tile_cap > 0 ? alloc_cull_tiles(c) : PDGPU_OK;
}

// at most 32 entries per tile plus one open group per row, held to 8192
// entries per row (a list that needs more keeps the tile path)
int pdgpu::alloc_cull_tiles(Context& c) {
  c.cull_cap = 0;
  if (!c.d_cull_row.p || c.tile_cap == 0) return PDGPU_OK;
  const long long cap = std::min(32LL * c.tile_cap + 32LL * c.nblocks, 8192LL * c.nblocks);
  cudaError_t e = c.d_cull_mask.alloc(c.tile_cap);
  if (e == cudaSuccess) e = c.d_cull_rest.alloc(c.tile_cap);
  if (e == cudaSuccess) e = c.d_cull_ent.alloc(cap);
  if (e == cudaSuccess) e = c.d_cull_bi.alloc(cap / 32);
  if (e != cudaSuccess) {
    c.d_cull_mask.release();
    c.d_cull_rest.release();
    c.d_cull_ent.release();
    c.d_cull_bi.release();
    cudaGetLastError();
    return PDGPU_ERR_CUDA;
  }
  c.cull_cap = cap;
  return PDGPU_OK;
}

// the tile list and everything sized by it, for `tiles` tiles with a quarter
// of headroom (never more than every block pair); captured step graphs hold the
// old addresses and are dropped
int pdgpu::alloc_tiles(Context& c, long long tiles) {
  const long long cap = std::min(c.npairs_all, std::max(tiles + tiles / 4 + 256, 1LL));
  drop_step_graphs(c);
  c.tile_cap = 0;
  c.cull_cap = 0;
  cudaError_t e = c.d_tiles.alloc(cap);
  if (e == cudaSuccess && c.has_gb) e = c.d_items.alloc(cap);
  if (e == cudaSuccess) e = c.d_tile_flag.alloc(cap);
  if (e == cudaSuccess) e = c.d_tile_pos.alloc(cap);
  if (e == cudaSuccess) e = c.d_tile_need.alloc(cap / 32 + 1);
  if (e == cudaSuccess) e = c.d_scan_tmp2.alloc((cap + 1023) / 1024 + 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PDGPU_ERR_CUDA;
  }
  c.tile_cap = cap;
  return alloc_cull_tiles(c);
}

extern "C" {

int pdgpu_set_nb_params(pdgpu_ctx* h, const pdgpu_nb_params* p) {
  if (!h || !p || p->Cutoff <= 0 || p->InnerCutoff > p->Cutoff || p->VdwInnerCutoff > p->VdwCutoff ||
      p->Dielectric == 0)
    return PDGPU_ERR_ARG;
  const int st = alloc_cull(h->c);
  if (st != PDGPU_OK) return st;
  h->c.nb = *p;
  h->c.nb_set = true;
  h->c.list_built = false;
  return PDGPU_OK;
}

int pdgpu_set_gb_params(pdgpu_ctx* h, const pdgpu_gb_params* p) {
  if (!h || !p || p->Cutoff <= 0 || p->InnerCutoff > p->Cutoff || p->DielectricSolute == 0 ||
      p->DielectricSolvent == 0 || p->P5 == 0)
    return PDGPU_ERR_ARG;
  h->c.gb = *p;
  h->c.gb_set = true;
  h->c.list_built = false;
  return PDGPU_OK;
}

int pdgpu_set_gb_mode(pdgpu_ctx* h, int fast_mode, const pdgpu_nb_params* vacuum) {
  if (!h || (fast_mode != 0 && fast_mode != 1)) return PDGPU_ERR_ARG;
  if (vacuum && (vacuum->Cutoff <= 0 || vacuum->InnerCutoff > vacuum->Cutoff || vacuum->Dielectric == 0))
    return PDGPU_ERR_ARG;
  Context& c = h->c;
  const bool same = c.gb_fast == (fast_mode != 0) && c.gb_vac_set == (vacuum != nullptr) &&
                    (!vacuum || std::memcmp(&c.gb_vac, vacuum, sizeof(pdgpu_nb_params)) == 0);
  if (same) return PDGPU_OK;
  if (c.md) return PDGPU_ERR_STATE;  // captured step graphs hold the launch sequence
  c.gb_fast = fast_mode != 0;
  c.gb_vac_set = vacuum != nullptr;
  if (vacuum) c.gb_vac = *vacuum;
  return PDGPU_OK;
}

int pdgpu_set_list_params(pdgpu_ctx* h, const pdgpu_list_params* p) {
  if (!h || !p || p->Padding < 0) return PDGPU_ERR_ARG;
  h->c.lp = *p;
  h->c.list_built = false;
  return PDGPU_OK;
}

static int enqueue_compute(Context& c, unsigned what, bool energy);

// the energy pass a parameter gradient reads (Born radii, Gpol sums, dE/da and
// energies); the GB chain-rule pass only forms forces and is left out
static int enqueue_grad_energies(Context& c, unsigned what) {
  c.gb_no_chain = true;
  const int st = enqueue_compute(c, what & ~PDGPU_ENERGY, true);
  c.gb_no_chain = false;
  return st;
}

int pdgpu_update_params(pdgpu_ctx* h, const double* charge, const double* radius, const double* epsilon,
                        const double* gb_radius, const double* gb_vj, const double* gb_terms123) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if ((gb_radius || gb_vj || gb_terms123) && !c.has_gb) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  const size_t N = c.natom;
  if (charge) CK(cudaMemcpyAsync(c.d_charge.p, charge, N * 8, cudaMemcpyHostToDevice, c.stream));
  if (radius) CK(cudaMemcpyAsync(c.d_radius.p, radius, N * 8, cudaMemcpyHostToDevice, c.stream));
  if (epsilon) {
    std::vector<double> sq(N);
    const double f = std::sqrt(kNa / kKcal2J);
    for (size_t a = 0; a < N; a++) sq[a] = epsilon[a] * f;
    CK(cudaMemcpyAsync(c.d_sqeps.p, sq.data(), N * 8, cudaMemcpyHostToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
  }
  if (gb_radius) CK(cudaMemcpyAsync(c.d_gbR.p, gb_radius, N * 8, cudaMemcpyHostToDevice, c.stream));
  if (gb_vj) CK(cudaMemcpyAsync(c.d_gbVj.p, gb_vj, N * 8, cudaMemcpyHostToDevice, c.stream));
  if (gb_terms123) CK(cudaMemcpyAsync(c.d_gbT.p, gb_terms123, N * 8, cudaMemcpyHostToDevice, c.stream));
  // the list itself does not depend on the parameters: refresh the per-slot copies
  if (c.list_built) {
    int st = launch_slot_params(c);
    if (st != PDGPU_OK) return st;
  }
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

}  // extern "C"

static __global__ void k_scale_copy(double* dst, const double* src, size_t n, double f) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] * f;
}

extern "C" {

int pdgpu_update_params_device(pdgpu_ctx* h, const double* d_charge, const double* d_radius,
                               const double* d_epsilon, const double* d_gb_radius, const double* d_gb_vj,
                               const double* d_gb_terms123) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if ((d_gb_radius || d_gb_vj || d_gb_terms123) && !c.has_gb) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  const size_t N = c.natom;
  const cudaMemcpyKind dd = cudaMemcpyDeviceToDevice;
  if (d_charge) CK(cudaMemcpyAsync(c.d_charge.p, d_charge, N * 8, dd, c.stream));
  if (d_radius) CK(cudaMemcpyAsync(c.d_radius.p, d_radius, N * 8, dd, c.stream));
  if (d_epsilon && N) {
    c.kernel_launches += 1;
    k_scale_copy<<<(unsigned)((N + 255) / 256), 256, 0, c.stream>>>(c.d_sqeps.p, d_epsilon, N,
                                                                     std::sqrt(kNa / kKcal2J));
    CK(cudaGetLastError());
  }
  if (d_gb_radius) CK(cudaMemcpyAsync(c.d_gbR.p, d_gb_radius, N * 8, dd, c.stream));
  if (d_gb_vj) CK(cudaMemcpyAsync(c.d_gbVj.p, d_gb_vj, N * 8, dd, c.stream));
  if (d_gb_terms123) CK(cudaMemcpyAsync(c.d_gbT.p, d_gb_terms123, N * 8, dd, c.stream));
  if (c.list_built) return launch_slot_params(c);
  return PDGPU_OK;
}

static int param_grad_check(const Context& c, unsigned what) {
  if (what & PDGPU_PD_ENERGIES) return PDGPU_ERR_ARG;
  if ((what & PDGPU_GB) && !c.gb_fast) return PDGPU_ERR_UNSUPPORTED;  // gradients of FastMode's energy
  const unsigned pair = what & (PDGPU_NB | PDGPU_GB);
  if (pair != PDGPU_NB && pair != PDGPU_GB) return PDGPU_ERR_ARG;
  if (what & ~(PDGPU_NB | PDGPU_GB | PDGPU_SA | PDGPU_BONDED | PDGPU_ENERGY)) return PDGPU_ERR_ARG;
  return PDGPU_OK;
}

static int mc_alloc(Context& c) {
  if (c.d_mc_ref.p) return PDGPU_OK;
  const size_t N = c.natom;
  if (c.d_mc_ref.alloc(3 * N) != cudaSuccess || c.d_mc_eref.alloc(2 * (size_t)c.nsys) != cudaSuccess ||
      c.d_mc_moved.alloc(N) != cudaSuccess || c.d_mc_list.alloc(N) != cudaSuccess ||
      c.d_mc_count.alloc(1) != cudaSuccess)
    return PDGPU_ERR_CUDA;
  return PDGPU_OK;
}

static void mc_energies(Context& c, const std::vector<long long>& e, pdgpu_energies* out) {
  for (int s = 0; s < c.nsys; s++) {
    pdgpu_energies o{};
    o.vdw = (double)e[2 * s] / kEnergyScale * kKcalMolToJ;
    o.elec = (double)e[2 * s + 1] / kEnergyScale * kKcalMolToJ;
    o.epot = o.vdw + o.elec;
    out[s] = o;
  }
}

int pdgpu_nb_energy_full(pdgpu_ctx* h, pdgpu_energies* out) {
  if (!h || !out) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.nb_set) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  int st = mc_alloc(c);
  if (st != PDGPU_OK) return st;
  st = enqueue_compute(c, PDGPU_NB, true);
  if (st != PDGPU_OK) return st;
  st = launch_mc_reference(c);
  if (st != PDGPU_OK) return st;
  std::vector<long long> e(2 * (size_t)c.nsys);
  CK(cudaMemcpyAsync(e.data(), c.d_mc_eref.p, sizeof(long long) * e.size(), cudaMemcpyDeviceToHost, c.stream));
  st = read_status(c);
  if (st != PDGPU_OK) return st;
  c.mc_ready = true;
  mc_energies(c, e, out);
  return PDGPU_OK;
}

int pdgpu_nb_energy_update(pdgpu_ctx* h, pdgpu_energies* out, int* nmoved) {
  if (!h || !out) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.nb_set || !c.mc_ready) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  int st = launch_mc_update(c);
  if (st != PDGPU_OK) return st;
  std::vector<long long> e(2 * (size_t)c.nsys);
  int n = 0;
  CK(cudaMemcpyAsync(e.data(), c.d_mc_eref.p, sizeof(long long) * e.size(), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaMemcpyAsync(&n, c.d_mc_count.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (nmoved) *nmoved = n;
  mc_energies(c, e, out);
  return PDGPU_OK;
}

int pdgpu_param_grad_device(pdgpu_ctx* h, unsigned what, const pdgpu_param_grads* g) {
  if (!h || !g) return PDGPU_ERR_ARG;
  Context& c = h->c;
  int st = param_grad_check(c, what);
  if (st != PDGPU_OK) return st;
  CK(cudaSetDevice(c.device));
  st = enqueue_grad_energies(c, what);
  if (st != PDGPU_OK) return st;
  return launch_adjoint(c, what, g->charge, g->radius, g->epsilon, g->gb_radius, g->gb_vj, g->gb_terms123);
}

int pdgpu_param_grad_device_noalloc(pdgpu_ctx* h, unsigned what, const pdgpu_param_grads* g) {
  if (!h || !g) return PDGPU_ERR_ARG;
  Context& c = h->c;
  int st = param_grad_check(c, what);
  if (st != PDGPU_OK) return st;
  if (c.nslots > kNoAllocMaxSlots) return PDGPU_ERR_CAPACITY;
  CK(cudaSetDevice(c.device));
  c.no_alloc = true;
  st = enqueue_grad_energies(c, what);
  c.no_alloc = false;
  if (st != PDGPU_OK) return st;
  return launch_adjoint_static(c, what, g->charge, g->radius, g->epsilon, g->gb_radius, g->gb_vj, g->gb_terms123);
}

int pdgpu_param_grad(pdgpu_ctx* h, unsigned what, pdgpu_energies* out, const pdgpu_param_grads* g) {
  if (!h || !g) return PDGPU_ERR_ARG;
  Context& c = h->c;
  int st = param_grad_check(c, what);
  if (st != PDGPU_OK) return st;
  CK(cudaSetDevice(c.device));
  const size_t N = c.natom;
  if (c.d_adj_out.n < 6 * N && c.d_adj_out.alloc(6 * N) != cudaSuccess) return PDGPU_ERR_CUDA;
  double* host[6] = {g->charge, g->radius, g->epsilon, g->gb_radius, g->gb_vj, g->gb_terms123};
  double* dev[6];
  for (int k = 0; k < 6; k++) dev[k] = host[k] ? c.d_adj_out.p + k * N : nullptr;
  st = enqueue_grad_energies(c, what);
  if (st != PDGPU_OK) return st;
  st = launch_adjoint(c, what, dev[0], dev[1], dev[2], dev[3], dev[4], dev[5]);
  if (st != PDGPU_OK) return st;
  for (int k = 0; k < 6; k++)
    if (host[k]) CK(cudaMemcpyAsync(host[k], dev[k], N * 8, cudaMemcpyDeviceToHost, c.stream));
  st = read_status(c);
  if (st != PDGPU_OK) return st;
  if (out) return pdgpu_get_energies(h, out);
  return PDGPU_OK;
}

int pdgpu_set_positions(pdgpu_ctx* h, const double* xyz, size_t stride) {
  if (!h || !xyz || stride < 24 || stride % 8) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  CK(copy_xyz_rows(c.d_pos.p, 24, xyz, stride, c.natom, cudaMemcpyHostToDevice, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  c.positions_set = true;
  return size_list(c);
}

int pdgpu_set_positions_device(pdgpu_ctx* h, const double* d_xyz) {
  if (!h || !d_xyz) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(c.d_pos.p, d_xyz, 24 * (size_t)c.natom, cudaMemcpyDeviceToDevice, c.stream));
  c.positions_set = true;
  return size_list(c);
}

int pdgpu_set_positions_async(pdgpu_ctx* h, const double* xyz) {
  if (!h || !xyz) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.positions_set) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(c.d_pos.p, xyz, 24 * (size_t)c.natom, cudaMemcpyHostToDevice, c.stream));
  return PDGPU_OK;
}

int pdgpu_get_positions_async(pdgpu_ctx* h, double* xyz) {
  if (!h || !xyz) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(xyz, c.d_pos.p, 24 * (size_t)c.natom, cudaMemcpyDeviceToHost, c.stream));
  return PDGPU_OK;
}

int pdgpu_get_positions(pdgpu_ctx* h, double* xyz, size_t stride) {
  if (!h || !xyz || stride < 24 || stride % 8) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  CK(copy_xyz_rows(xyz, stride, c.d_pos.p, 24, c.natom, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

}  // extern "C"

int pdgpu::rebuild_list_impl(Context& c) {
  if (!c.positions_set) return PDGPU_ERR_STATE;
  if (!c.nb_set && !c.gb_set && !c.has_sa) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  float R = (float)list_radius(c);
  float F = (float)std::min(full_radius(c), (double)R);
  // a captured step cannot read the tile count back; the allocation-free
  // entry point may not resize
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(c.stream, &cs));
  const ListSizing sizing =
      cs != cudaStreamCaptureStatusNone ? kListDevice : (c.no_alloc ? kListCheck : kListReadback);
  int st = launch_list_build(c, R, F, sizing);
  if (st != PDGPU_OK) return st;
  c.list_radius_built = R;
  c.full_radius_built = F;
  c.list_built = true;
  return PDGPU_OK;
}

extern "C" {

int pdgpu_rebuild_list(pdgpu_ctx* h) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  CK(cudaMemsetAsync(c.d_status.p, 0, sizeof(unsigned), c.stream));
  return rebuild_list_impl(c);
}

}  // extern "C"

// One force evaluation on the context stream (no host synchronisation).
// rebuild: rebuild the list first (else pack the positions and check the skin).
// LCPO forces go to lcpo_f and its energy to lcpo_e (stride lcpo_e_stride) when
// run_lcpo; dynamics points them at the cached-LCPO buffers.
// (set-up failure) the context's streams and events
void pdgpu::release_streams(Context& c) {
  if (c.ev_fork) cudaEventDestroy(c.ev_fork);
  if (c.ev_join) cudaEventDestroy(c.ev_join);
  if (c.side) cudaStreamDestroy(c.side);
  if (c.stream) cudaStreamDestroy(c.stream);
  c.ev_fork = c.ev_join = nullptr;
  c.side = c.stream = nullptr;
}

int pdgpu::enqueue_forces(Context& c, unsigned what, bool energy, bool rebuild, long long* lcpo_f,
                          long long* lcpo_e, int lcpo_e_stride, bool run_lcpo) {
  if (rebuild || !c.list_built) {
    int st = rebuild_list_impl(c);
    if (st != PDGPU_OK) return st;
  } else {
    int st = launch_pack(c, c.lp.check_skin ? (float)(0.5 * c.lp.Padding) : 0.f);
    if (st != PDGPU_OK) return st;
  }
  CK(cudaMemsetAsync(c.d_facc.p, 0, sizeof(long long) * 3 * c.nslots, c.stream));
  if (energy) CK(cudaMemsetAsync(c.d_eacc.p, 0, sizeof(long long) * E_NSLOTS * c.nsys, c.stream));
  int st = PDGPU_OK;
  // the LCPO recalculation (positions, packed slots and tile list) and the bonded
  // terms (positions) need nothing from the pair kernels: they run on the side
  // stream beside them, adding into the same fixed-point accumulators (integer
  // sums: the result does not depend on how the two streams interleave)
  const bool side_sa = (what & PDGPU_SA) && run_lcpo, side_bonded = (what & PDGPU_BONDED) != 0;
  const bool forked = side_sa || side_bonded;
  if (forked) {
    CK(cudaEventRecord(c.ev_fork, c.stream));
    CK(cudaStreamWaitEvent(c.side, c.ev_fork, 0));
    cudaStream_t main = c.stream;
    c.stream = c.side;
    if (side_sa) st = launch_lcpo(c, lcpo_f, lcpo_e, lcpo_e_stride);
    if (st == PDGPU_OK && side_bonded) st = launch_bonded(c, energy);
    c.stream = main;
    // joined back below on every path, so a stream capture always closes
    CK(cudaEventRecord(c.ev_join, c.side));
  }
  if (st == PDGPU_OK && (what & PDGPU_NB)) st = launch_nb(c, make_nb_const(c.nb), energy);
  if (st == PDGPU_OK && (what & PDGPU_GB)) {
    GBConst k = make_gb_const(c.gb, c.list_radius_built);
    // FastMode off, or PD's calcEnergies (gbff.cpp:178-183: calcBornEnergy, no
    // ExpApproxThreshold): the GB part alone plus the vacuum part from the GB
    // object's own FF_NonBonded settings
    const bool pd_energies = (what & PDGPU_PD_ENERGIES) != 0;
    if (!c.gb_fast || pd_energies) {
      k.fast = 0;
      if (pd_energies) {
        k.thresh = -1e30f;
        k.thresh_d = -1e300;
      }
      st = launch_nb(c, make_nb_const(gb_vacuum_params(c)), energy);
    }
    double ec = econv_kcal();
    double premul = -0.5 * ec * (1.0 / c.gb.DielectricSolute - 1.0 / c.gb.DielectricSolvent);
    if (st == PDGPU_OK) st = launch_gb(c, k, 0.5 * ec, c.gb.BornRadiusOffset, premul, energy);
  }
  if (forked) CK(cudaStreamWaitEvent(c.stream, c.ev_join, 0));
  return st;
}

extern "C" {

static int enqueue_compute(Context& c, unsigned what, bool energy) {
  if (!c.positions_set) return PDGPU_ERR_STATE;
  if ((what & PDGPU_NB) && !c.nb_set) return PDGPU_ERR_STATE;
  if ((what & PDGPU_GB) && (!c.has_gb || !c.gb_set)) return PDGPU_ERR_STATE;
  if ((what & PDGPU_SA) && !c.has_sa) return PDGPU_ERR_STATE;
  if ((what & (PDGPU_GB | PDGPU_SA)) && c.any_periodic) return PDGPU_ERR_UNSUPPORTED;
  CK(cudaMemsetAsync(c.d_status.p, 0, sizeof(unsigned), c.stream));
  return enqueue_forces(c, what, energy, false, c.d_facc.p, energy ? c.d_eacc.p + E_SURF : nullptr, E_NSLOTS, true);
}

int pdgpu_get_energies(pdgpu_ctx* h, pdgpu_energies* out) {
  if (!h || !out) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(c.h_eacc.data(), c.d_eacc.p, sizeof(long long) * E_NSLOTS * c.nsys, cudaMemcpyDeviceToHost,
                     c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (int s = 0; s < c.nsys; s++) {
    const long long* E = &c.h_eacc[(size_t)s * E_NSLOTS];
    auto J = [&](int k) { return (double)E[k] / kEnergyScale * kKcalMolToJ; };
    pdgpu_energies& o = out[s];
    o.vdw = J(E_VDW);
    o.elec = J(E_ELEC);
    o.pol_cross = J(E_POL_CROSS);
    o.pol_self = J(E_POL_SELF);
    o.pol = o.pol_cross + o.pol_self;
    o.surf = J(E_SURF);
    o.virial = J(E_VIRIAL);
    o.bond = J(E_BOND);
    o.angle = J(E_ANGLE);
    o.torsion = J(E_TORS);
    o.improper = J(E_IMPR);
    o.epot = o.vdw + o.elec + o.pol + o.surf + o.bond + o.angle + o.torsion + o.improper;
  }
  return PDGPU_OK;
}

int pdgpu_compute(pdgpu_ctx* h, unsigned what, pdgpu_energies* out, double* f, size_t stride) {
  if (!h || (f && (stride < 24 || stride % 8))) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  int st = enqueue_compute(c, what, out != nullptr);
  if (st != PDGPU_OK) return st;
  if (f) {
    st = launch_finalize_forces(c, c.d_fout.p, 3, false, kForceToN);
    if (st != PDGPU_OK) return st;
    c.h_stage.resize(3 * (size_t)c.natom);
    CK(cudaMemcpyAsync(c.h_stage.data(), c.d_fout.p, 24 * (size_t)c.natom, cudaMemcpyDeviceToHost, c.stream));
  }
  st = read_status(c);
  if (st != PDGPU_OK) return st;
  if (f) {
    const size_t sd = stride / 8;
    for (int a = 0; a < c.natom; a++)
      for (int k = 0; k < 3; k++) f[a * sd + k] += c.h_stage[3 * (size_t)a + k];
  }
  if (out) return pdgpu_get_energies(h, out);
  return PDGPU_OK;
}

int pdgpu_compute_device(pdgpu_ctx* h, unsigned what, double* d_f) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  CK(cudaSetDevice(c.device));
  int st = enqueue_compute(c, what, (what & PDGPU_ENERGY) != 0);
  if (st != PDGPU_OK) return st;
  if (d_f) st = launch_finalize_forces(c, d_f, 3, false, kForceToN);
  return st;
}

int pdgpu_get_born_radii(pdgpu_ctx* h, double* born) {
  if (!h || !born) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.has_gb) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(born, c.d_born_d.p, 8 * (size_t)c.natom, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

int pdgpu_get_sasa(pdgpu_ctx* h, double* sasa) {
  if (!h || !sasa) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.has_sa) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(sasa, c.d_sasa.p, 8 * (size_t)c.natom, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

int pdgpu_list_stats(pdgpu_ctx* h, long long* ntiles, long long* nmasked, long long* nslots) {
  if (!h) return PDGPU_ERR_ARG;
  Context& c = h->c;
  int cnt[2] = {0, 0};
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(cnt, c.d_counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  if (ntiles) *ntiles = cnt[0];
  if (nmasked) *nmasked = cnt[1];
  if (nslots) *nslots = c.nslots;
  return PDGPU_OK;
}

int pdgpu_list_tiles(pdgpu_ctx* h, int* tiles, long long cap, long long* ntiles, long long* tile_cap,
                     long long* list_bytes) {
  if (!h || (cap > 0 && !tiles) || cap < 0) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.list_built) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  int nt = 0;
  CK(cudaMemcpyAsync(&nt, c.d_counters.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  const long long n = std::min<long long>(nt, cap);
  if (n > 0) {
    std::vector<Tile> t(n);
    CK(cudaMemcpyAsync(t.data(), c.d_tiles.p, sizeof(Tile) * n, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    for (long long k = 0; k < n; k++) {
      tiles[3 * k] = t[k].bi;
      tiles[3 * k + 1] = t[k].bj;
      tiles[3 * k + 2] = t[k].flags;
    }
  }
  if (ntiles) *ntiles = nt;
  if (tile_cap) *tile_cap = c.tile_cap;
  if (list_bytes) {
    // the arrays whose size follows the list
    *list_bytes = (long long)(c.d_tiles.n * sizeof(Tile) + c.d_items.n * 4 + c.d_tile_flag.n * 4 +
                              c.d_tile_pos.n * 4 + c.d_scan_tmp2.n * 4 + c.d_tile_need.n * 4 + c.d_mlist.n * 4 +
                              c.d_masks.n * sizeof(uint2) + c.d_cull_mask.n * 4 + c.d_cull_rest.n * 4 +
                              c.d_cull_ent.n * sizeof(float4) + c.d_cull_bi.n * 4);
  }
  return PDGPU_OK;
}

int pdgpu_list_slots(pdgpu_ctx* h, int* atom_of_slot) {
  if (!h || !atom_of_slot) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.list_built) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  CK(cudaMemcpyAsync(atom_of_slot, c.d_sorted_atom.p, sizeof(int) * c.nslots, cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  return PDGPU_OK;
}

void* pdgpu_stream(pdgpu_ctx* h) { return h ? (void*)h->c.stream : nullptr; }

}  // extern "C"

int pdgpu_device_allocations(long long* count, long long* bytes) {
  if (count) *count = g_device_allocs.load();
  if (bytes) *bytes = g_device_bytes.load();
  return PDGPU_OK;
}

int pdgpu_host_alloc(size_t bytes, void** ptr) {
  if (!ptr || bytes == 0) return PDGPU_ERR_ARG;
  *ptr = nullptr;
  if (cudaHostAlloc(ptr, bytes, cudaHostAllocDefault) != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();  // leave no pending error for the caller's next runtime call
    return PDGPU_ERR_CUDA;
  }
  return PDGPU_OK;
}

int pdgpu_host_free(void* ptr) {
  if (!ptr) return PDGPU_OK;
  return cudaFreeHost(ptr) == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int pdgpu_pair_census(pdgpu_ctx* h, long long* counts) {
  if (!h || !counts) return PDGPU_ERR_ARG;
  Context& c = h->c;
  if (!c.list_built) return PDGPU_ERR_STATE;
  CK(cudaSetDevice(c.device));
  DBuf<unsigned long long> d;
  CK(d.alloc(5));
  CK(cudaMemsetAsync(d.p, 0, 5 * sizeof(unsigned long long), c.stream));
  const bool gb = c.gb_set && c.has_gb;
  int st = launch_census(c, make_nb_const(c.nb), make_gb_const(c.gb, c.list_radius_built), c.nb_set, gb, d.p);
  if (st != PDGPU_OK) return st;
  unsigned long long h_out[5];
  CK(cudaMemcpyAsync(h_out, d.p, sizeof(h_out), cudaMemcpyDeviceToHost, c.stream));
  CK(cudaStreamSynchronize(c.stream));
  for (int k = 0; k < 5; k++) counts[k] = (long long)h_out[k];
  return PDGPU_OK;
}

int pdgpu_fp32_peak(int device, double* tflops_ffma, double* tflops_ffma2) {
  if (device < 0) return PDGPU_ERR_ARG;
  return measure_fp32_peak(device, tflops_ffma, tflops_ffma2);
}
