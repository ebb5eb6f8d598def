// pdgpu_common.cuh — shared definitions for the GB300 nonbonded / GB / LCPO path.
//
// Layout (one context may hold several independent systems, "a batch"):
//   * original order  : atoms as the host numbers them, systems concatenated.
//   * sorted order    : per system, atoms ordered along a 3-D Hilbert curve of a
//                       32^3 cell grid, padded to a multiple of 32; slot s holds
//                       original atom sorted_atom[s] (or -1 for padding).
//   * blocks          : 32 consecutive sorted slots of one system.
//   * tiles           : block pairs (bi <= bj) of one system whose bounding boxes
//                       come within the list radius; one warp evaluates the
//                       32x32 interactions of a tile by shuffle rotation.
// Forces, Born-radius sums, dE/da and energies are accumulated in 64-bit fixed
// point, so results are bit-identical run to run whatever the tile order.
// Internal units: Angstrom, kcal/mol, e; conversion to PD units (J, N) happens
// once per atom / per energy at the end.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pdgpu.h"

namespace pdgpu {

constexpr int kWarp = 32;
constexpr int kHilbertBits = 5;                       // 32 cells per dimension
constexpr int kCellsPerSystem = 1 << (3 * kHilbertBits);
constexpr int kMaxSystemBlocks = 65536;               // blocks of one system (2^21 atoms): the list-build bitmap
constexpr int kBandWidth = 64;                        // bonded partners within +-64 indices use the band masks
constexpr int kLcpoMax = 80;                          // PD caps an atom's LCPO overlap list at 80 (lcpo.h:24)
constexpr int kLcpoCand = 160;                        // candidate capacity before the cap is applied

// fixed-point scales
constexpr double kForceScale = 4294967296.0;          // 2^32 per kcal/mol/A
constexpr double kEnergyScale = 4294967296.0;         // 2^32 per kcal/mol (|E| < 2^31 kcal/mol per slot)
constexpr double kSumScale = 4294967296.0;            // 2^32 per unit (Born sums, dE/da)

// per-system energy slots (fixed point)
enum EnergySlot { E_VDW = 0, E_ELEC, E_POL_CROSS, E_POL_SELF, E_SURF, E_VIRIAL, E_BOND, E_ANGLE, E_TORS, E_IMPR, E_NSLOTS };

// status bits set by kernels
enum StatusBits : unsigned {
  ST_LCPO_OVERFLOW = 1u,
  ST_FIXED_OVERFLOW = 2u,
  ST_NAN = 4u,
  ST_STALE_LIST = 8u,
  // the tile list or its exclusion-mask table outgrew its capacity in a build
  // that could not resize it (a captured step); the list is incomplete
  ST_TILE_OVERFLOW = 16u,
};

struct SystemInfo {
  int atom_start;   // first atom (original order)
  int natom;
  int pad_start;    // first slot (sorted order)
  int npad;         // multiple of 32
  int block_start;
  int nblocks;
  int grid_start;   // first cell of this system's block grid (list build)
  int grid_cells;   // its cell budget: one per block
  int periodic;
  double box[3];
  double ibox[3];   // 1 / box (periodic systems)
};

struct __align__(16) Tile {
  int bi, bj;
  int mask;    // index into the exclusion-mask table or -1
  int flags;   // bit0: per-pair minimum image needed, bit1: diagonal tile,
               // bit2: every pair inside all cutoffs and switch radii (with margin)
  // centre of block bj seen from block bi (its periodic image in a box), formed
  // in FP64 at the list build and rounded once: the pair kernels add it to the
  // j positions without per-tile FP64 work
  float ox, oy, oz, pad;
};

// Grid over one system's block centres (list build), remade every build: cells
// of about equal edge over the periodic box, or over the bounding box of the
// system's atoms in open space, at most one cell per block
struct BlockGrid {
  double origin[3];
  double cell[3];   // cell edges
  int dims[3];
  int start;        // first cell in the context's cell arrays
  float hmax[3];    // largest block half-extent of the system per axis
  float pad;
};

// Pair-law constants for the LJ + Coulomb kernel (FF_NonBonded)
// (the _d members are the same constants in FP64, for the energy arithmetic)
struct NBConst {
  float cut2, vdwcut2, vdw14, elec14, econv_diel;
  double cut2_dd, vdwcut_d, vdwinner_d, inner_d, vdwinvw2_d, invw2_d, econv_diel_d, vdw14_d, elec14_d;
  double sA, sB, sC, sD, sE, fsw_cutV, eshift, cut2_d, inner2_d;
  // FP32 copies for the force pair law
  float vdwcut_f, vdwinner_f, vdwinvw2_f, inner_f, invw2_f, inner2_f, sA_f, fsw_k;  // fsw_k = cut2 - 3 inner2
  int elecmode;            // 0 none, 1 plain, 3 energy switch, 4 force switch
  int dovdw;
  // 1: LJ and Coulomb switched over the same radii (Cutoff = VdwCutoff,
  // InnerCutoff = VdwInnerCutoff, energy switch, LJ on): one switch serves both
  int samesw;
};

// Constants for the GB fast path (FF_GeneralizedBorn_Still::calcForcesIncludingVacuo)
struct GBConst {
  float cut2, inner, invw2, vdwcut, vdwinner, vdwinvw2;
  float still2;            // min(GbsaStillCutoff, list radius)^2
  float econv_in, econv_out, premul;  // kcal units
  float vdw14, elec14, thresh;
  float P4, P5, invP5;
  // FP64 copies for the energy arithmetic
  double cut2_d, inner_d, invw2_d, vdwcut_d, vdwinner_d, vdwinvw2_d, still2_d;
  double econv_in_d, econv_out_d, premul_d, vdw14_d, elec14_d, thresh_d;
  // 1: FastMode (GB fused with LJ + Coulomb, εout Coulomb below the threshold);
  // 0: calcBornForces (GB term alone for every pair, premul q q / r below it)
  int fast;
  // energy passes: pairs closer than sqrt(e64_r2) take their energies in FP64
  // from FP64 positions and parameters (0: none, every pair in FP32)
  float e64_r2;
  // the force-only all-inside body: Born radii scaled by sqrtK, so that
  // a_i a_j K >= r^2 holds for every pair the threshold test may switch on
  // (K = -4 x the threshold widened by 4e-6 relative); charges scaled by
  // sqrt(econv_out), sqrt(eps) by sqrt(12)
  float sqrtK, inv_sqrtK, sq_eout, inv_eout, in_over_out_m1, sqrt12;
};

// Device-side view of a context, passed by value to kernels.
struct DevView {
  int nsys, natom, nslots, nblocks;
  const SystemInfo* sys;
  const int* slot_sys;       // [nblocks] system of each block
  // original order
  const double* pos;         // natom*3
  const double* charge;      // natom, e
  const double* radius;      // natom, LJ Rmin/2
  const double* sqeps;       // natom, sqrt(kcal/mol)
  const double* born;        // natom, Born radii of the last GB pass (FP64)
  // (GB energy evaluations) FP64 records per sorted slot, written by
  // k_energy_records before the energy pass: (x, y, z, charge) and (LJ radius,
  // sqrt(eps kcal/mol)); padding slots: far away, radius -1
  const double4* epos;
  const double2* epar;
  // sorted order
  const int* sorted_atom;    // [nslots]
  float4* xq;                // rel pos + charge
  float4* par;               // LJ radius, sqrt(eps kcal), GB R (raw), GB Vj
  float4* rel0;              // rel pos at list build (displacement check)
  double* center;            // [nblocks*3]
  float4* half;              // [nblocks] half extents
  unsigned long long* band_excl;   // [natom*2]? (see below) per atom: bit d-1 => partner i+d excluded (bo<=2)
  unsigned long long* band_14;     // per atom: bit d-1 => partner i+d is a 1-4 pair
  const int* far_start;      // CSR of partners beyond the band, per atom
  const int* far_idx;
  const int* far_bo;
  Tile* tiles;
  int* ntiles;
  // GB work items over the tile list: tile index, bit 31 set when the item is the
  // tile pair (t, t + 1) (same row, adjacent columns, both unmasked off-diagonal)
  unsigned* items;
  int* nitems;
  uint2* masks;              // [mask_cap*32] per lane: (excluded bits, 1-4 bits) in rotation order
  int* nmasks;
  int mask_cap;
  // NB j-atom groups: per i-block row, the j atoms of its unmasked, off-diagonal,
  // single-image tiles that lie within the list radius of the i block's box,
  // packed 32 to a group; the other tiles stay on the tile path (cull_rest)
  float4* cull_ent;          // [cull_cap] j offset into the i block's frame (x, y, z), j slot (int bits; -1 empty)
  int* cull_bi;              // [cull_cap / 32] i block of each group
  int* cull_rest;            // [tile capacity] tiles left on the tile path (any order)
  int* cull_n;               // [0] rest tiles, [1] groups, [2] 1 when the groups fit the capacity
  long long cull_cap;        // entries
  long long* facc;           // [nslots*3]
  long long* eacc;           // [nsys*E_NSLOTS]
  unsigned* status;
};

// ---------------------------------------------------------------------------
// fixed point helpers
// ---------------------------------------------------------------------------
// energies: 2^32 per kcal/mol.  The resolution matters: a converted partial
// sum keeps only whole units, so many small partial sums of one sign (the far
// attractive LJ tail, per lane and tile) would be lost at a coarse scale.
__device__ __forceinline__ long long fix_energy_d(double x) { return __double2ll_rn(x * 4294967296.0); }
// float -> 64-bit fixed point with 32 fractional bits using integer operations
// only (|x| < 2^31; larger magnitudes saturate near 2^62 so the overflow check
// trips).  Rounds half away from zero.  The hardware float->int64 conversion
// runs on the FP64 pipe, which is narrow on this GPU.
__device__ __forceinline__ long long fx32(float x) {
  const unsigned b = __float_as_uint(x);
  const int e = (int)((b >> 23) & 0xffu);
  const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 118;  // x * 2^32 = m * 2^(e - 150 + 32)
  unsigned long long r;
  if (e == 0) r = 0ull;
  else if (sh >= 39) r = 1ull << 62;
  else if (sh >= 0) r = m << sh;
  else if (sh > -25) r = (m + (1ull << (-sh - 1))) >> (-sh);
  else r = 0ull;
  return (b >> 31) ? -(long long)r : (long long)r;
}

// Range of FP32 partial sums about to enter 64-bit fixed point (2^32 per unit):
// m is the sum of their magnitudes.  NaN or infinity sets ST_NAN; 2^28 or more
// sets ST_FIXED_OVERFLOW.  One conversion holds up to 2^30 and a slot's total
// up to 2^31, so flagging every partial sum at 2^28 keeps a few large ones
// from wrapping a total past the final check unnoticed.  (PD has no such
// limit; 2^28 kcal/mol/A lies far beyond any physical force.)
__device__ __forceinline__ void fix_range(unsigned* status, float m) {
  if (!(m < 268435456.f)) atomicOr(status, !(m < 1.0e18f) ? (unsigned)ST_NAN : (unsigned)ST_FIXED_OVERFLOW);
}

__device__ __forceinline__ void atomic_add_ll(long long* p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(v));
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// host-side launchers (defined in the .cu files)
// ---------------------------------------------------------------------------
struct Context;
int tile_grid(Context& c);   // grid of the tile kernels (grid-stride, one tile per warp item)
// full_radius: distance below which every cutoff and switch of the set
// components is inactive (0 = never mark tiles full).  sizing: how the tile
// count meets the capacity:
//   kListReadback  read the count back, grow the tile arrays when it exceeds them
//   kListCheck     read it back, PDGPU_ERR_CAPACITY when it exceeds them (no allocation)
//   kListDevice    no host round trip (a captured step): an overflow leaves the
//                  list short and sets ST_TILE_OVERFLOW
enum ListSizing { kListReadback = 0, kListCheck = 1, kListDevice = 2 };
int launch_list_build(Context& c, float list_radius, float full_radius, ListSizing sizing);
// tile arrays (and the NB group arrays sized from them) for `tiles` tiles
int alloc_tiles(Context& c, long long tiles);
// the NB j-atom group arrays for the current tile capacity
int alloc_cull_tiles(Context& c);
int launch_pack(Context& c, float check_disp);
int launch_nb(Context& c, const NBConst& k, bool need_virial);
int launch_gb(Context& c, const GBConst& k, double halfeconv, double born_offset, double premul, bool energy);
int launch_lcpo(Context& c, long long* facc_out, long long* esurf_out, int esurf_stride);
int launch_gb_stage(Context& c, const GBConst& k, int stage);
// parameter gradients after an energy evaluation of NB or GB (device outputs,
// original atom order, J per parameter unit; null pointers are skipped)
int launch_adjoint(Context& c, unsigned what, double* d_q, double* d_r, double* d_e, double* d_R, double* d_V,
                   double* d_T);
// the same into a static device array: no allocation during the call (at most
// kNoAllocMaxSlots sorted slots; one scratch per device shared by all contexts)
constexpr int kNoAllocMaxSlots = 65536;
int launch_adjoint_static(Context& c, unsigned what, double* d_q, double* d_r, double* d_e, double* d_R, double* d_V,
                          double* d_T);
// Monte Carlo partial NB energies: take the reference from the last energy
// evaluation / update it by the pairs of the moved atoms
int launch_mc_reference(Context& c);
int launch_mc_update(Context& c);
// static per-slot parameters refreshed from the per-atom arrays (after a parameter update)
int launch_slot_params(Context& c);
// measurement aids (k_diag.cu): the pair census of the current list into out[5]
// (device, zeroed by the caller) and the FP32 FMA ceiling of a device
int launch_census(Context& c, const NBConst& nk, const GBConst& gk, bool do_nb, bool do_gb, unsigned long long* out);
int measure_fp32_peak(int device, double* tflops_ffma, double* tflops_ffma2);
NBConst make_nb_const(const pdgpu_nb_params& p);
GBConst make_gb_const(const pdgpu_gb_params& p, double listR);
int launch_bonded(Context& c, bool energy);
int launch_finalize_forces(Context& c, double* out, size_t stride_doubles, bool add, double scale);
// host-side orchestration shared by the evaluation and dynamics entry points
int rebuild_list_impl(Context& c);
void release_streams(Context& c);
int enqueue_forces(Context& c, unsigned what, bool energy, bool rebuild, long long* lcpo_f, long long* lcpo_e,
                   int lcpo_e_stride, bool run_lcpo);
struct MDState;
void destroy_md(Context& c);
// captured step graphs hold buffer addresses: dropped when a buffer is replaced
void drop_step_graphs(Context& c);

}  // namespace pdgpu
