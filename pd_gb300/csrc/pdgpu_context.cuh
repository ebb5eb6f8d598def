// pdgpu_context.cuh — host-side context: device buffers, parameters, stream.
#pragma once
#include <atomic>
#include <string>
#include <vector>

#include "pdgpu_common.cuh"

namespace pdgpu {

// Every device allocation of the library goes through DBuf; these process-wide
// counters (cudaMalloc calls made, bytes held) back pdgpu_device_allocations.
inline std::atomic<long long> g_device_allocs{0};
inline std::atomic<long long> g_device_bytes{0};

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    g_device_allocs.fetch_add(1);
    g_device_bytes.fetch_add((long long)(count * sizeof(T)));
    return cudaSuccess;
  }
  void release() {
    if (p) {
      cudaFree(p);
      g_device_bytes.fetch_sub((long long)(n * sizeof(T)));
    }
    p = nullptr;
    n = 0;
  }
  ~DBuf() { release(); }
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  // work that reads positions only (bonded terms, the LCPO recalculation) runs on
  // `side` beside the pair kernels, forked from and joined back to `stream`
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int nsys = 0, natom = 0, nslots = 0, nblocks = 0;
  long long npairs_all = 0;    // block pairs bi <= bj of every system (every pair a tile)
  long long tile_cap = 0;      // tile list capacity: sized from the count of a build, with headroom
  int mask_cap = 0;            // exclusion-mask table: diagonal, padded and bonded tiles (a strict bound)
  int max_sys_blocks = 0;      // blocks of the largest system
  bool no_alloc = false;       // inside pdgpu_param_grad_device_noalloc: list builds may not resize
  bool any_periodic = false, all_periodic = true;
  bool has_gb = false, has_sa = false, has_bonded = false, has_mass = false;
  bool positions_set = false, list_built = false;
  std::vector<SystemInfo> sys;
  std::vector<int> h_atom_sys;

  // parameters
  pdgpu_nb_params nb{};
  pdgpu_gb_params gb{};
  pdgpu_list_params lp{};
  bool nb_set = false, gb_set = false;
  bool gb_fast = true;             // FF_GeneralizedBorn_Still::FastMode
  bool gb_no_chain = false;        // energies only: skip the GB chain-rule (force) pass
  pdgpu_nb_params gb_vac{};        // the GB object's own FF_NonBonded settings (FastMode off, calcEnergies)
  bool gb_vac_set = false;
  float list_radius_built = 0.f;
  float full_radius_built = 0.f;   // tiles flagged full: max distance + full_margin() below this
  // displacement margin of full tiles: every atom stays within half of it of its
  // position at the build (checked every step by the position pack)
  float full_margin() const { return (float)(lp.Padding > 10.0 ? lp.Padding : 10.0); }
  bool nb_cull = true;         // NB j-atom groups (needs the per-step skin check)
  bool cull_built = false;     // the last list build wrote the groups
  int tile_ctas_per_sm = 8;    // launch shape of the tile kernels (autotuned)
  int gb_item_tiles = 2;       // GB work items: 1 single tiles, 2 tile pairs where the list allows (autotuned)
  long long kernel_launches = 0;  // kernels this context has put on its stream (graph replays included)

  // static per-atom data (original order)
  DBuf<SystemInfo> d_sys;
  DBuf<int> d_atom_sys;        // [natom]
  DBuf<int> d_block_sys;       // [nblocks]
  DBuf<double> d_charge, d_radius, d_sqeps;   // sqeps in sqrt(kcal/mol)
  DBuf<double> d_gbR, d_gbVj, d_gbT;          // GB raw radius, Vj, terms123
  DBuf<double> d_lcpoR, d_lcpoP, d_lcpoSig;   // lcpo radius, P1..P4, sigma (kcal/mol/A^2)
  DBuf<int> d_lcpoUse;
  DBuf<unsigned long long> d_band_excl, d_band_14;
  DBuf<int> d_far_start, d_far_idx, d_far_bo;
  DBuf<double> d_mass;                         // kg

  // dynamic state
  DBuf<double> d_pos;          // [natom*3] Angstrom
  DBuf<double> d_fout;         // [natom*3] N (device-side output buffer)

  // list build scratch
  DBuf<int> d_bucket;          // [natom]
  DBuf<int> d_count, d_offset, d_cursor;      // [nsys*kCellsPerSystem]
  DBuf<int> d_scan_tmp;
  DBuf<int> d_tmp_sorted;      // [natom]
  DBuf<float> d_sys_lo, d_sys_hi;              // [nsys*3]
  DBuf<int> d_sorted_atom;     // [nslots]
  DBuf<int> d_slot_of;         // [natom] sorted slot of each atom
  DBuf<double> d_center;       // [nblocks*3]
  DBuf<float4> d_half;         // [nblocks]
  DBuf<float> d_sys_hmax;      // [nsys*3] largest block half-extent (ordered ints)
  DBuf<BlockGrid> d_bgrid;     // [nsys]
  DBuf<int> d_bcell;           // [nblocks] cell of each block
  DBuf<int> d_bcell_count, d_bcell_off, d_bcell_cursor, d_bcell_scan_tmp;  // [nblocks] cells
  DBuf<int> d_bcell_blocks;    // [nblocks] blocks in cell order
  DBuf<int> d_row_cnt, d_row_start;  // [nblocks] tiles per row, first tile of each row
  DBuf<Tile> d_tiles;          // [tile_cap] rows contiguous (any order), ascending columns
  DBuf<int> d_tile_flag, d_tile_pos, d_scan_tmp2;  // [tile_cap] compaction scratch (GB items, NB groups)
  DBuf<unsigned> d_tile_need;  // [tile_cap/32 + 1] one bit per tile: in the mask list
  DBuf<int> d_mlist;           // [mask_cap] tiles that get their exclusion bits (diagonal, padded, bonded)
  // [0] ntiles, [1] nmasks, [2] nitems, [3..5] NB groups (rest tiles, groups, fit),
  // [6] tiles the rows found (before the capacity clamp), [7] mask-list length
  DBuf<int> d_counters;
  DBuf<unsigned> d_items;      // [tile_cap] GB work items (with GB only)
  DBuf<uint2> d_masks;         // [mask_cap*32]
  DBuf<float4> d_xq, d_par, d_rel0;  // [nslots]
  // NB j-atom groups (allocated with the NB parameters)
  DBuf<unsigned> d_cull_mask;        // [tile_cap] j lanes kept per tile
  DBuf<int> d_cull_rest;             // [tile_cap]
  DBuf<int> d_cull_row;              // [4*nblocks] per row: kept j atoms, first tile, groups, first group
  DBuf<int> d_cull_scan_tmp;
  DBuf<float4> d_cull_ent;           // [cull_cap]
  DBuf<int> d_cull_bi;               // [cull_cap / 32]
  long long cull_cap = 0;

  // accumulators
  DBuf<long long> d_facc;      // [nslots*3]
  DBuf<long long> d_eacc;      // [nsys*E_NSLOTS]
  DBuf<unsigned> d_status;

  // GB
  DBuf<long long> d_gpol, d_deda;   // [nslots]
  DBuf<float> d_born_f;             // [nslots]
  DBuf<float> d_chain_f;            // [nslots] a^2/166 * dE/da * P4
  DBuf<double> d_born_d;            // [natom] original order
  DBuf<double4> d_epos;             // [nslots] FP64 position + charge per slot (energy evaluations)
  DBuf<double2> d_epar;             // [nslots] FP64 LJ radius + sqrt(eps) per slot
  // Monte Carlo partial energy updates (allocated on first use)
  DBuf<double> d_mc_ref;            // [natom*3] positions of the reference evaluation
  DBuf<long long> d_mc_eref;        // [nsys*2] reference vdw, elec (fixed point, energy scale)
  DBuf<unsigned char> d_mc_moved;   // [natom]
  DBuf<int> d_mc_list, d_mc_count;  // [natom], [1]
  bool mc_ready = false;
  // parameter gradients (allocated on first use)
  DBuf<long long> d_adj;            // [5*nslots] dE/dq, dE/dRmin, dE/dsqrt(eps), dE/dR_gb, dE/dVj
  DBuf<float> d_adj_w;              // [nslots] dE/dGpol
  DBuf<double> d_adj_out;           // [6*natom] staging for the host-array entry point
  // LCPO
  DBuf<int> d_lc_ncand;             // [nslots]
  DBuf<int> d_lc_cand;              // [nslots*kLcpoCand]
  DBuf<int> d_lc_n;                 // [nslots]
  DBuf<int2> d_lc_e2;               // [nslots*kLcpoMax] (partner slot, s_ij bits), ascending original index
  DBuf<float4> d_lc_ent;            // [nslots*kLcpoMax] partner position (lc_pos frame) and LCPO radius
  DBuf<float4> d_lc_psig;           // [nslots] (P2, P3, P4) x sigma of the slot's atom, FP32
  DBuf<float4> d_lc_box;            // [nblocks*2] block box over its LCPO atoms (lo + max radius, hi)
  DBuf<double> d_sasa;              // [natom]
  DBuf<float4> d_lc_par;            // [nslots] (radius, use, -, -)
  DBuf<float4> d_lc_pos;            // [nslots] position from its system's first block centre (FP32), radius

  // bonded
  int nbond = 0, nangle = 0, ntors = 0, nimpr = 0;
  DBuf<int> d_bidx, d_aidx, d_tidx, d_iidx;
  DBuf<double> d_bpar, d_apar, d_tpar, d_ipar;

  // dynamics state (pdgpu_md_setup), owned by the context
  MDState* md = nullptr;

  // host staging
  std::vector<long long> h_eacc;
  std::vector<double> h_stage;
  int last_error = 0;
  std::string last_msg;

  DevView view() const {
    DevView v;
    v.nsys = nsys;
    v.natom = natom;
    v.nslots = nslots;
    v.nblocks = nblocks;
    v.sys = d_sys.p;
    v.slot_sys = d_block_sys.p;
    v.pos = d_pos.p;
    v.charge = d_charge.p;
    v.radius = d_radius.p;
    v.sqeps = d_sqeps.p;
    v.born = d_born_d.p;
    v.epos = d_epos.p;
    v.epar = d_epar.p;
    v.sorted_atom = d_sorted_atom.p;
    v.xq = d_xq.p;
    v.par = d_par.p;
    v.rel0 = d_rel0.p;
    v.center = d_center.p;
    v.half = d_half.p;
    v.band_excl = d_band_excl.p;
    v.band_14 = d_band_14.p;
    v.far_start = d_far_start.p;
    v.far_idx = d_far_idx.p;
    v.far_bo = d_far_bo.p;
    v.tiles = d_tiles.p;
    v.ntiles = d_counters.p;
    v.items = d_items.p;
    v.nitems = d_counters.p + 2;
    v.masks = d_masks.p;
    v.nmasks = d_counters.p + 1;
    v.mask_cap = mask_cap;
    v.cull_ent = d_cull_ent.p;
    v.cull_bi = d_cull_bi.p;
    v.cull_rest = d_cull_rest.p;
    v.cull_n = d_counters.p + 3;
    v.cull_cap = cull_cap;
    v.facc = d_facc.p;
    v.eacc = d_eacc.p;
    v.status = d_status.p;
    return v;
  }
};

// n rows of 3 doubles between a packed device array and a host array with
// `pitch` bytes per row: one contiguous copy when the host rows are packed as
// well (a 2D copy of 24-byte rows moves row by row, far below copy bandwidth)
inline cudaError_t copy_xyz_rows(void* dst, size_t dpitch, const void* src, size_t spitch, size_t n,
                                 cudaMemcpyKind kind, cudaStream_t st) {
  if (dpitch == 24 && spitch == 24) return cudaMemcpyAsync(dst, src, 24 * n, kind, st);
  return cudaMemcpy2DAsync(dst, dpitch, src, spitch, 24, n, kind, st);
}

// unit conversions (PD PhysicsConst, src/mmlib/forcefields/forcefield.cpp:35-55)
constexpr double kKcal2J = 4184.0;
constexpr double kNa = 6.0221418E23;
constexpr double kAngstrom = 1E-10;
constexpr double kKcalMolToJ = kKcal2J / kNa;                  // kcal/mol -> J per molecule
constexpr double kForceToN = kKcalMolToJ / kAngstrom;           // kcal/mol/A -> N
inline double econv_kcal() {
  const double e = 1.60217645E-19, e0 = 8.854187817E-12, pi = 3.14159265358979323846;
  return ((1.0 / kKcal2J) * kNa * e * e) / (4.0 * pi * e0 * kAngstrom);
}

}  // namespace pdgpu
