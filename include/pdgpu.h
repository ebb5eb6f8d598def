/* pdgpu.h — C ABI of the GB300 nonbonded / Generalised-Born / LCPO path for PD.
 *
 * Plain C types only: pointers, sizes, doubles and ints.  The library owns all
 * device memory of a context; host arrays passed in are borrowed for the
 * duration of the call.  No function throws; every function returns a status
 * (PDGPU_OK == 0, negative on error, see pdgpu_error_string()).
 *
 * Units are PD's WorkSpace units throughout: positions in Angstrom, energies in
 * J per molecule, forces in N, velocities in m/s, masses in kg, per-atom LJ
 * epsilon stored as sqrt(J) and LJ radius as Rmin/2 in Angstrom
 * (PD src/mmlib/system/fundamentals.h:191-197).
 *
 * The reference interfaces each entry point replaces are cited beside it
 * (paths inside the PD project).  A context is bound to one CUDA device and one
 * stream and is not re-entrant; distinct contexts may be used concurrently.
 */
#ifndef PDGPU_H
#define PDGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define PDGPU_OK 0
#define PDGPU_ERR_ARG (-1)            /* invalid argument (PD: ProcedureException)          */
#define PDGPU_ERR_CUDA (-2)           /* CUDA runtime error                                  */
#define PDGPU_ERR_LIST_OVERFLOW (-3)  /* an LCPO overlap list, or the tile list inside a
                                         captured dynamics step, exceeded its capacity      */
#define PDGPU_ERR_FIXED_OVERFLOW (-4) /* a fixed-point accumulator left its range            */
#define PDGPU_ERR_NAN (-5)            /* NaN energy or force (PD: assertStability)           */
#define PDGPU_ERR_TIMEOUT (-6)        /* a device wait exceeded its iteration limit          */
#define PDGPU_ERR_UNSUPPORTED (-7)    /* option not supported (e.g. GB in a periodic box)    */
#define PDGPU_ERR_STALE_LIST (-8)     /* an atom moved more than Padding/2 since the rebuild */
#define PDGPU_ERR_STATE (-9)          /* call sequence error (e.g. compute before positions) */
#define PDGPU_ERR_CAPACITY (-10)      /* larger than a fixed-size entry point's static scratch,
                                         or a list that would need arrays such a call may
                                         not allocate (pdgpu_param_grad_device_noalloc)     */

/* ---- what to compute ------------------------------------------------------ */
#define PDGPU_NB 1u      /* FF_NonBonded: LJ + Coulomb with PD's switching     */
#define PDGPU_GB 2u      /* FF_GeneralizedBorn_Still, FastMode (incl. vacuum LJ/Coulomb) */
#define PDGPU_SA 4u      /* FF_SASA_LCPO                                        */
#define PDGPU_BONDED 8u  /* FF_Bonded: bonds, angles, torsions, impropers       */
#define PDGPU_ENERGY 0x100u /* pdgpu_compute_device: also form the energies        */
/* with PDGPU_GB: the energies as FF_GeneralizedBorn_Still::calcEnergies forms them
 * (gbff.cpp:178-183: Born radii, FF_NonBonded::calcEnergies with the GB object's
 * own settings, calcBornEnergy without ExpApproxThreshold, gbff.cpp:537-596);
 * forces, if asked for, are those of that energy */
#define PDGPU_PD_ENERGIES 0x200u

/* Per-system energies in J per molecule; the fields mirror PD's Hamiltonian
 * (src/mmlib/workspace/hamiltonian.h:43-66). */
typedef struct {
    double epot, vdw, elec, pol, pol_self, pol_cross, surf, virial;
    double bond, angle, torsion, improper;
} pdgpu_energies;

/* Static description of one or more independent systems (a batch).  All
 * per-atom arrays are concatenated over systems in system order; index arrays
 * use these global atom indices.  Optional arrays may be NULL. */
typedef struct {
    int nsystems;
    const int *natoms;           /* [nsystems] */
    const double *box;           /* [nsystems*3]; all zero => infinite space */
    const double *charge;        /* [N] e */
    const double *radius;        /* [N] LJ Rmin/2, Angstrom */
    const double *epsilon;       /* [N] sqrt(eps [J]) */
    const double *mass;          /* [N] kg (needed only for dynamics) */
    /* Still GB (optional): raw type radius, Vj, terms123 as set up by
     * FF_GeneralizedBorn_Still::calcFixedBornRadiiTerms (gbff.cpp:324-398) */
    const double *gb_radius, *gb_vj, *gb_terms123;
    /* LCPO (optional): radius (+1.4 probe), P1..P4 [N*4], sigma (J/A^2), use flag */
    const double *lcpo_radius, *lcpo_p, *lcpo_sigma;
    const int *lcpo_use;
    /* bonded pairs as PD's neighbour list classifies them: (i, j, bondorder),
     * bondorder 0..3 (1-2 = 1, 1-3 = 2, 1-4 = 3); pairs not listed are ordinary */
    int nexcl;
    const int *excl;
    /* FF_Bonded terms (optional), PD units: bond (i,j)+(l,k); angle (i,a,j)+(theta0,k);
     * torsion/improper (i,a,b,j,terms)+(Vn,n,gamma)x4 */
    int nbond;  const int *bond_idx;  const double *bond_par;
    int nangle; const int *angle_idx; const double *angle_par;
    int ntors;  const int *tors_idx;  const double *tors_par;
    int nimpr;  const int *impr_idx;  const double *impr_par;
} pdgpu_system_desc;

/* FF_NonBonded public parameters (src/mmlib/forcefields/nonbonded.h:62-231). */
typedef struct {
    double Cutoff, InnerCutoff, VdwCutoff, VdwInnerCutoff;
    double Vdw14Scaling, Elec14Scaling, Dielectric;
    int EnergySwitch, ForceSwitch, DoVdw, DoElec;
} pdgpu_nb_params;

/* FF_GeneralizedBorn_Still public parameters (src/mmlib/forcefields/gbff.h:123-203). */
typedef struct {
    double Cutoff, InnerCutoff, VdwCutoff, VdwInnerCutoff;
    double Vdw14Scaling, Elec14Scaling;
    double DielectricSolute, DielectricSolvent, GbsaStillCutoff, ExpApproxThreshold, BornRadiusOffset;
    double P4, P5;
} pdgpu_gb_params;

/* NeighbourList settings (src/mmlib/workspace/neighbourlist.h:54-126). */
typedef struct {
    double Padding;      /* list skin, Angstrom (PD default 0.5) */
    int check_skin;      /* 1: flag PDGPU_ERR_STALE_LIST when an atom moved > Padding/2 */
} pdgpu_list_params;

typedef struct pdgpu_ctx pdgpu_ctx;

/* ---- life cycle ----------------------------------------------------------- */
/* Replaces the setup() of FF_NonBonded / FF_GeneralizedBorn_Still / FF_SASA_LCPO
 * (nonbonded.cpp:1025-1053, gbff.cpp:57-104, lcpo.cpp:33-127): copies every
 * parameter to the device.  Returns NULL and sets *status on failure. */
pdgpu_ctx *pdgpu_create(int device, const pdgpu_system_desc *desc, int *status);
int pdgpu_destroy(pdgpu_ctx *ctx);
const char *pdgpu_error_string(int status);

int pdgpu_set_nb_params(pdgpu_ctx *ctx, const pdgpu_nb_params *p);
int pdgpu_set_gb_params(pdgpu_ctx *ctx, const pdgpu_gb_params *p);
int pdgpu_set_list_params(pdgpu_ctx *ctx, const pdgpu_list_params *p);
/* FF_GeneralizedBorn_Still::FastMode (gbff.cpp:37, 185-197).  1 (PD's default):
 * calcForcesIncludingVacuo, GB fused with LJ + Coulomb.  0: FF_NonBonded::
 * calcForces with the GB object's own settings (`vacuum`) plus calcBornForces
 * (gbff.cpp:1189-1437: the GB term of every pair within Cutoff, bonded pairs
 * too, premul q q / r below ExpApproxThreshold).  vacuum may be NULL: the GB
 * cutoffs and 1-4 scalings with Dielectric 1 and the energy switch, PD's
 * defaults for the GB object; it also serves PDGPU_PD_ENERGIES.  Parameter
 * gradients need FastMode on.  Set it before pdgpu_md_setup (PDGPU_ERR_STATE
 * after it: captured step graphs hold the launch sequence). */
int pdgpu_set_gb_mode(pdgpu_ctx *ctx, int fast_mode, const pdgpu_nb_params *vacuum);
/* Per-atom charges / LJ radius / epsilon (PD's sqrt(J) storage) / GB radius,
 * Vj, terms123 (all optional, NULL keeps) — the parameter update after FF
 * re-setup.  The list is kept; the per-slot copies are refreshed. */
int pdgpu_update_params(pdgpu_ctx *ctx, const double *charge, const double *radius, const double *epsilon,
                        const double *gb_radius, const double *gb_vj, const double *gb_terms123);
/* Same with device arrays (no host synchronisation); the per-slot copies are
 * refreshed on the context stream without rebuilding the list. */
int pdgpu_update_params_device(pdgpu_ctx *ctx, const double *d_charge, const double *d_radius,
                               const double *d_epsilon, const double *d_gb_radius, const double *d_gb_vj,
                               const double *d_gb_terms123);

/* ---- state ---------------------------------------------------------------- */
/* Upload positions (Angstrom).  stride_bytes is the distance between atoms;
 * 24 for packed xyz, 72 for PD's SnapShotAtom {p, f, v} (snapshot.h:33-39). */
int pdgpu_set_positions(pdgpu_ctx *ctx, const double *xyz, size_t stride_bytes);
/* Same from device memory already on this context's device (packed xyz). */
int pdgpu_set_positions_device(pdgpu_ctx *ctx, const double *d_xyz);
int pdgpu_get_positions(pdgpu_ctx *ctx, double *xyz, size_t stride_bytes);
/* Asynchronous forms for page-locked host memory (pdgpu_host_alloc), packed
 * xyz: the copy is queued on the context stream in order with the work around
 * it and the call returns at once; the caller leaves the buffer alone until
 * pdgpu_synchronize returns.  A dynamics loop can then move every step's
 * positions in and out with no host round trip per step (PD's per-step
 * WorkSpace exchange without the wait).  set: the context's positions must
 * have been set once with pdgpu_set_positions (that call sizes the list). */
int pdgpu_set_positions_async(pdgpu_ctx *ctx, const double *xyz);
int pdgpu_get_positions_async(pdgpu_ctx *ctx, double *xyz);

/* ---- neighbour list ------------------------------------------------------- */
/* Replaces NeighbourList::calcNewList (neighbourlist.cpp:222-439): cell-grid
 * sort, block bounding boxes and the tile list at radius max(cutoffs)+Padding,
 * found through a grid over the block centres.  The tile arrays are sized by
 * the first build (the first pdgpu_set_positions after the parameters) with a
 * quarter of headroom and grow at any build outside a captured dynamics step
 * that finds more tiles; inside a captured step an overflow is reported as
 * PDGPU_ERR_LIST_OVERFLOW by the step's status, and the next call of this
 * function grows them. */
int pdgpu_rebuild_list(pdgpu_ctx *ctx);

/* ---- evaluation ----------------------------------------------------------- */
/* Replaces ForcefieldBase::calcForces of the selected components
 * (nonbonded.cpp:1222-1246, gbff.cpp:185-197, lcpo.cpp:193-206).  Energies for
 * each system are written to out[0..nsystems) (may be NULL).  Forces in N are
 * ADDED into f (may be NULL) at stride_bytes per atom, as PD components add
 * into WorkSpace::cur.atom[i].f. */
int pdgpu_compute(pdgpu_ctx *ctx, unsigned what, pdgpu_energies *out, double *f, size_t stride_bytes);
/* Device variant: forces in N written (not added) to d_f (packed xyz, device
 * memory) without any host synchronisation.  Energies are formed only when
 * `what` includes PDGPU_ENERGY and stay on the device until pdgpu_get_energies().
 * Forces are FP32 pair math with 64-bit fixed-point sums.  Energies, when
 * requested: GB pair energies in FP64 from FP64 positions and parameters for
 * pairs closer than 4.5 A, from FP32 terms beyond, summed in FP64 and fixed
 * point; FF_NonBonded pair energies in FP64. */
int pdgpu_compute_device(pdgpu_ctx *ctx, unsigned what, double *d_f);
int pdgpu_get_energies(pdgpu_ctx *ctx, pdgpu_energies *out);
/* Born radii (Angstrom, original atom order) and LCPO per-atom SASA (A^2) from
 * the last evaluation that computed them. */
int pdgpu_get_born_radii(pdgpu_ctx *ctx, double *born);
int pdgpu_get_sasa(pdgpu_ctx *ctx, double *sasa);

/* ---- Monte Carlo energies (FF_NonBonded::calcEnergies, nonbonded.cpp:1154-1182)
 * pdgpu_nb_energy_full evaluates the FF_NonBonded energies (vdw, elec, epot;
 * other fields zero) of every system and keeps them with the current positions
 * as the reference.  pdgpu_nb_energy_update (UsePartialRecalc,
 * nonbonded.cpp:76-386) then returns the energies after the atoms whose
 * positions differ from the reference moved: the reference minus every pair
 * touching a moved atom at its reference position plus the same pairs now
 * (FP64 pair energies, all pairs of the system inside Cutoff), and makes the
 * current positions the reference.  nmoved (may be NULL) counts the moved
 * atoms.  Call pdgpu_nb_energy_full again after a list-changing event, as PD
 * does after a full list update. */
int pdgpu_nb_energy_full(pdgpu_ctx *ctx, pdgpu_energies *out);
int pdgpu_nb_energy_update(pdgpu_ctx *ctx, pdgpu_energies *out, int *nmoved);

/* ---- parameter gradients (adjoint) ----------------------------------------
 * PD has no counterpart: its parameter derivatives are finite differences of
 * Forcefield::calcEnergies with setup() re-run after each edit
 * (src/mmlib/forcefields/nonbonded.cpp:1078-1084).  One call evaluates the
 * energies (GB pairs from FP32 terms summed in FP64, |dE|/|E| ~ 1e-6: they
 * weight a loss; pdgpu_compute gives the closer ones) and dE/dp for every
 * per-atom parameter array of
 * pdgpu_system_desc, in original atom order, J per unit of the parameter as
 * it is given there (charge e, radius A, epsilon sqrt(J), gb_radius A, gb_vj
 * A^3, gb_terms123 its own unit); E is the system's own energy, so atoms of
 * different systems get the gradient of their own system's energy.  `what`
 * names exactly one of PDGPU_NB / PDGPU_GB (SA / BONDED may be added; they
 * contribute energies only).  The GB gradient is the exact derivative of the
 * energy through the Born radii, including the fixed terms' inputs gb_vj and
 * gb_terms123 (their own dependence on gb_radius is the caller's chain rule).
 * Null pointers are skipped. */
typedef struct {
    double *charge, *radius, *epsilon;          /* LJ + Coulomb (and GB charge terms) */
    double *gb_radius, *gb_vj, *gb_terms123;    /* GB only (zero for PDGPU_NB) */
} pdgpu_param_grads;
int pdgpu_param_grad(pdgpu_ctx *ctx, unsigned what, pdgpu_energies *out, const pdgpu_param_grads *g);
/* Device-array form: queued on the context stream; energies stay on the device
 * until pdgpu_get_energies(), status via pdgpu_synchronize().  The gradient
 * calls evaluate energies only: forces read after one of them are not the
 * system's forces until the next force evaluation. */
int pdgpu_param_grad_device(pdgpu_ctx *ctx, unsigned what, const pdgpu_param_grads *d_g);
/* Same result as pdgpu_param_grad_device, with no device allocation in the
 * call.  It has no counterpart in PD.  It is for hosts that cannot let a call
 * run cudaMalloc: the allocation synchronises the whole device (stalling the
 * host's other streams), or the host's own pool already holds the free memory.
 * The scratch is a static device array of the library, sized for 65,536
 * sorted slots (about as many atoms; each system is padded to 32-atom
 * blocks): a larger context gets PDGPU_ERR_CAPACITY and nothing is queued.
 * The first call on a device looks up the array's address and may load the
 * library's device code; make that call before any stream capture.  Each call
 * clears its accumulators on the context stream.  All contexts on a device
 * share the array, so calls whose GPU work overlaps race. */
int pdgpu_param_grad_device_noalloc(pdgpu_ctx *ctx, unsigned what, const pdgpu_param_grads *d_g);

/* ---- dynamics: MolecularDynamics / REX_Local --------------------------------- */
/* Integrator settings (PD src/mmlib/protocols/md.h, defaults md.cpp:60-86). */
typedef struct {
    int Integrator;              /* 0: PD velocity Verlet (md.cpp:805-855); 1: Langevin (md.cpp:923-1063) */
    double Timestep;             /* s (PD default 1e-15) */
    double FricCoeff;            /* Langevin friction, 1/s (PD default 1e13) */
    int UpdateNList;             /* neighbour-list rebuild cadence in steps (PD default 10) */
    int UpdateSasa;              /* LCPO recalculation cadence in steps (PD default 5, lcpo.cpp:193-206) */
    unsigned what;               /* components: PDGPU_NB | PDGPU_GB | PDGPU_SA | PDGPU_BONDED */
    unsigned long long seed;     /* Philox key of the Langevin noise and of the exchange draws */
    int use_graph;               /* 1: replay captured CUDA graphs of the step */
} pdgpu_md_params;

/* Replaces MolecularDynamics::setup for every system of the batch; temps gives
 * each system's target temperature (K).  Velocities start at zero. */
int pdgpu_md_setup(pdgpu_ctx *ctx, const pdgpu_md_params *p, const double *temps);
int pdgpu_set_velocities(pdgpu_ctx *ctx, const double *v, size_t stride_bytes);
int pdgpu_get_velocities(pdgpu_ctx *ctx, double *v, size_t stride_bytes);
/* Replaces MolecularDynamics::run_core (md.cpp:219-283) for nsteps steps of
 * every system at once: list refresh on the UpdateNList cadence
 * (protocolbase.cpp:135-144), forces, integrator; the trajectory continues
 * across calls.  With energy_on_last the energies of the last step are formed
 * (pdgpu_get_energies) — the exchange criterion needs them. */
int pdgpu_md_run(pdgpu_ctx *ctx, int nsteps, int energy_on_last);
/* Same without waiting: the steps are queued on the context stream and the
 * device status (NaN, stale list, overflow) is collected by pdgpu_synchronize(). */
int pdgpu_md_enqueue(pdgpu_ctx *ctx, int nsteps, int energy_on_last);
int pdgpu_synchronize(pdgpu_ctx *ctx);
/* Kinetic energy of each system after the last step (J), PD's calcKineticEnergy. */
int pdgpu_get_kinetic(pdgpu_ctx *ctx, double *ekin);
/* Same, queued on the context stream into page-locked host memory (see
 * pdgpu_set_positions_async): valid after pdgpu_synchronize returns. */
int pdgpu_get_kinetic_async(pdgpu_ctx *ctx, double *ekin);
/* One REX_Local exchange sweep (remd.cpp:178-215): rungs (parity, parity+1),
 * (parity+2, parity+3)... of the temperature ladder, Metropolis on the last
 * energies (remd.cpp:349-356), accepted swaps exchange the systems' target
 * temperatures and rescale their velocities by sqrt(T'/T).  accepted[r] (may be
 * NULL) reports rung pair r; temps (may be NULL) returns each system's new
 * target temperature. */
int pdgpu_remd_exchange(pdgpu_ctx *ctx, int parity, int *accepted, double *temps);
/* REX_Replica::ExchangeMode per rung (remd.h:49, applied at remd.cpp:186-200;
 * the lower replica's mode governs a pair).  Swap trades temperatures (the
 * default); Downward copies the upper structure onto the lower rung, Upward the
 * lower onto the upper, with PD's velocity rescaling of both rungs.  The copy
 * modes need systems of one molecule (equal atom counts, else
 * PDGPU_ERR_UNSUPPORTED); after a copy the list is rebuilt at the next step. */
#define PDGPU_REX_SWAP 0
#define PDGPU_REX_DOWNWARD 1
#define PDGPU_REX_UPWARD 2
int pdgpu_remd_set_modes(pdgpu_ctx *ctx, const int *modes);
/* Crash rescue of REX_Local::runcore (remd.cpp:118-147): pdgpu_md_checkpoint
 * saves the positions (call it at the start of a round); after a round that
 * failed (a non-finite atom ends it with PDGPU_ERR_NAN, _FIXED_OVERFLOW or
 * _STALE_LIST, whichever its kernels meet first), pdgpu_md_rescue puts every system holding a
 * non-finite position or velocity back to its saved positions with fresh
 * Maxwell-Boltzmann velocities at its target temperature (PD's 200 conjugate-
 * gradient minimisation steps are not run).  rescued (nsystems ints, may be
 * NULL) flags them, count gets their number. */
int pdgpu_md_checkpoint(pdgpu_ctx *ctx);
/* Trajectory frames without stalling the step stream (PD writes a frame every
 * UpdateTra steps, md.cpp:277, through OutTra, fileio/tra.h:78-87): every
 * `every` steps the positions of all systems (original order, Angstrom, natom*3
 * doubles) are copied asynchronously on the context stream into slot
 * frame % nslots of host_ring, which the caller owns (page-locked memory keeps
 * the copy asynchronous; the ring must outlive the run).  Frames are complete
 * once pdgpu_synchronize / pdgpu_md_run returns; a slot is overwritten after
 * nslots further frames.  every = 0 switches it off.  pdgpu_md_trajectory_frames
 * counts the frames queued since the last pdgpu_md_set_trajectory. */
int pdgpu_md_set_trajectory(pdgpu_ctx *ctx, int every, double *host_ring, int nslots);
long long pdgpu_md_trajectory_frames(pdgpu_ctx *ctx);
int pdgpu_md_rescue(pdgpu_ctx *ctx, unsigned long long seed, int *rescued, int *count);
/* Project autotuner (state restored afterwards): first the GB work-item size
 * (pdgpu_set_work_items) and the launch shape of the tile kernels (CTAs per SM
 * of their grid-stride grid), timed together on force evaluations of the
 * current state; then the list-rebuild cadence together with the LJ/Coulomb
 * j-atom groups on or off (pdgpu_set_nb_groups), timed per step on short
 * trial runs of whole rebuild windows (at least trial_steps steps), keeping
 * the fastest whose list never goes stale.  Outputs may be NULL; the chosen
 * work-item size and groups setting are read with pdgpu_get_work_items and
 * pdgpu_get_nb_groups. */
int pdgpu_md_autotune(pdgpu_ctx *ctx, int trial_steps, int *update_nlist, int *ctas_per_sm);
/* Launch shape of the pair-tile kernels (what the autotuner sets): CTAs per SM
 * of their grid (1..64).  Results do not depend on it (per-tile sums enter
 * fixed point). */
int pdgpu_set_launch_shape(pdgpu_ctx *ctx, int ctas_per_sm);
int pdgpu_get_launch_shape(pdgpu_ctx *ctx, int *ctas_per_sm);
/* Work-item size of the GB tile kernels (what the autotuner sets): 1 = one
 * 32x32 tile per warp item, 2 = two tiles of one row that share their i block
 * where the list allows (one rotation of that block serves both: fewer shuffles
 * per pair, half as many items).  No counterpart in PD.  The item list is
 * rewritten at the next list build; results agree to FP32 rounding of the
 * per-item sums. */
int pdgpu_set_work_items(pdgpu_ctx *ctx, int tiles_per_item);
int pdgpu_get_work_items(pdgpu_ctx *ctx, int *tiles_per_item);
/* LJ/Coulomb j-atom groups (on by default; what the autotuner sets): at each
 * list build, the j atoms of a row's plain tiles (no exclusions, off-diagonal,
 * one periodic image) that lie within the list radius of the i block's box are
 * packed 32 to a work item, so the pair kernel skips most out-of-cutoff pairs
 * of a 32x32 tile.  Used only with the per-step displacement check
 * (pdgpu_list_params.check_skin), which it keeps on in open space too.  No
 * counterpart in PD.  Results agree with the tile path to FP32 rounding of the
 * per-item sums.  get: the setting, and the groups and tiles the last list build
 * left to the kernel (0 and -1 when it wrote no groups or they did not fit). */
int pdgpu_set_nb_groups(pdgpu_ctx *ctx, int on);
int pdgpu_get_nb_groups(pdgpu_ctx *ctx, int *on, long long *ngroups, long long *nrest_tiles);

/* ---- diagnostics ---------------------------------------------------------- */
/* Tile / pair counts of the current list: ntiles, nmasked tiles, slots. */
int pdgpu_list_stats(pdgpu_ctx *ctx, long long *ntiles, long long *nmasked, long long *nslots);
/* The current tile list as (bi, bj, flags) per tile, each row's tiles
 * together with ascending columns, rows in any order (block b holds sorted
 * slots 32b..32b+31);
 * at most `cap` tiles are written, *ntiles gets the list length.  Flags: bit 0
 * per-pair minimum image, bit 1 diagonal, bit 2 every pair inside all cutoffs.
 * Also the device memory the list arrays hold (tile capacity, bytes). */
int pdgpu_list_tiles(pdgpu_ctx *ctx, int *tiles, long long cap, long long *ntiles, long long *tile_cap,
                     long long *list_bytes);
/* The atom in each sorted slot of the current list (-1 for a padding slot). */
int pdgpu_list_slots(pdgpu_ctx *ctx, int *atom_of_slot);
/* Number of kernels this context has launched so far (graph replays count
 * every kernel node they run). */
long long pdgpu_kernel_launches(pdgpu_ctx *ctx);
/* Timing probe: runs one kernel of the path `reps` times on the current state
 * (0 LJ/Coulomb tiles, 1 GB Born sums, 2 GB fused pair, 3 GB chain rule,
 * 4 LCPO, 5 integrator (advances the dynamics), 6 list build, 7 position pack,
 * 8 bonded), each launch bracketed by CUDA events on the context stream, with
 * an optional 256 MB L2 flush before each; returns the mean duration in ms. */
int pdgpu_time_kernel(pdgpu_ctx *ctx, int kernel, int reps, int flush_l2, double *avg_ms);
/* Stream the context launches on (cudaStream_t as void*), for event timing. */
void *pdgpu_stream(pdgpu_ctx *ctx);
/* Pair census of the current list at the positions of the last evaluation, by
 * the branch each pair takes in the pair kernels (FP32 decisions, as they take
 * them): counts[0] FF_NonBonded pairs inside Cutoff (bond order > 2);
 * counts[1] GB pairs inside the GB Cutoff; counts[2] of those, the pairs above
 * ExpApproxThreshold (GB cross term evaluated, gbff.cpp:1592-1678; Born radii
 * of the last GB evaluation); counts[3] Born-radius pairs inside
 * GbsaStillCutoff (bond order > 2, gbff.cpp:432-483); counts[4] of those, the
 * close-contact pairs (CCF < 1).  No counterpart in PD; the benchmark's
 * roofline counts flops per branch with it. */
int pdgpu_pair_census(pdgpu_ctx *ctx, long long counts[5]);
/* FP32 FMA throughput of a device, measured: kernels of independent FFMA (and
 * packed FFMA2) chains, best of 5 launches timed with CUDA events, in TFLOP/s
 * (FMA = 2 flops).  Outputs may be NULL.  No counterpart in PD; the ceiling the
 * benchmark's pair-kernel roofline divides by. */
int pdgpu_fp32_peak(int device, double *tflops_ffma, double *tflops_ffma2);
/* Device memory of the library in this process, over all contexts: cudaMalloc
 * calls made so far (count, never decreases) and bytes held now (either may be
 * NULL).  No counterpart in PD; a diagnostic (e.g. to check that a call
 * allocated nothing). */
int pdgpu_device_allocations(long long *count, long long *bytes);

/* ---- host memory ------------------------------------------------------------ */
/* Page-locked host memory for buffers the library fills asynchronously (the
 * trajectory ring of pdgpu_md_set_trajectory), so callers need no CUDA runtime
 * of their own.  No counterpart in PD (its trajectory writer reads ordinary
 * host memory).  PDGPU_ERR_CUDA when the runtime cannot provide it (e.g. no
 * GPU): ordinary memory also works, with copies that wait for the step. */
int pdgpu_host_alloc(size_t bytes, void **ptr);
int pdgpu_host_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif /* PDGPU_H */
