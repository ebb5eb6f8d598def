/* pdoracle — CPU restatement (FP64, plain C) of PD's nonbonded energy/force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path and
 * the timed CPU baseline; nothing in the product links or calls it.  Parity of
 * this restatement with PD itself is pinned by the .npz files in tests/golden, which were
 * produced by the compiled PD reference (oracle/ref_driver.cpp).
 *
 * Units follow PD's WorkSpace: positions in Angstrom, energies in J per
 * molecule, forces in N (J/m), per-atom epsilon stored as sqrt(J), LJ radius
 * as Rmin/2 (PD src/mmlib/system/fundamentals.h:191-197,
 * src/mmlib/forcefields/ffparam.cpp:1216,1593).
 *
 * Every entry point ADDS into the force array it is given (PD components add
 * into WorkSpace::cur.atom[i].f) and OVERWRITES the energy record.
 */
#ifndef PDORACLE_H
#define PDORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* PhysicsConst (PD src/mmlib/forcefields/forcefield.cpp:35-55) */
#define PDO_KCAL2J 4184.0
#define PDO_NA 6.0221418E23
#define PDO_KB 1.38065E-23
#define PDO_ANGSTROM 1E-10
#define PDO_E_CHARGE 1.60217645E-19
#define PDO_E0 8.854187817E-12

double pdo_econv_joule(void);   /* e^2/(4 pi e0 A)            [J]          */
double pdo_halfeconv(void);     /* econv/2 in kcal A / mol                 */

typedef struct {
    int natom;
    const double *pos;     /* natom*3 */
    const double *charge;  /* e */
    const double *radius;  /* Rmin/2 [A] */
    const double *epsilon; /* sqrt(eps [J]) */
    int nexcl;
    const int *excl;       /* nexcl*3 : (i, j, bondorder), bondorder 0..3, pairs not listed are 7 */
    double box[3];         /* orthogonal periodic box [A]; all zero => infinite space */
} pdo_system;

typedef struct {
    double Cutoff, InnerCutoff, VdwCutoff, VdwInnerCutoff;
    double Vdw14Scaling, Elec14Scaling, Dielectric;
    int EnergySwitch, ForceSwitch, DoVdw, DoElec;
    int VdwCor;
    double VdwCorDensity, VdwCorEpsilon, VdwCorRadius, VdwCorCutoff; /* VdwCorEpsilon in kcal/mol */
    double ListCutoff;     /* Cutoff + Padding: pairs beyond it are never listed */
} pdo_nb_params;

typedef struct {
    double Cutoff, InnerCutoff, VdwCutoff, VdwInnerCutoff;
    double Vdw14Scaling, Elec14Scaling;
    double DielectricSolute, DielectricSolvent;
    double GbsaStillCutoff, ExpApproxThreshold, DielectricOffset, BornRadiusOffset;
    double P1, P2, P3, P4, P5;
    double ListCutoff;
    int FastMode;   /* 1: calcForcesIncludingVacuo (GB + LJ + Coulomb); 0: calcBornForces (GB only,
                       gbff.cpp:1189-1437; the vacuum part is FF_NonBonded's, pdo_nonbonded) */
} pdo_gb_params;

typedef struct {
    double epot, vdw, elec, pol, pol_self, pol_cross, surf, virial;
} pdo_energies;

/* --- neighbour list (PD src/mmlib/workspace/neighbourlist.cpp:247-439) --- */
/* Half list (j < i) at min-image r^2 <= ListCutoff^2, reported as per-atom
 * count, sum of j and sum of j^2 (checksums). */
int pdo_list_checksums(const pdo_system *s, double list_cutoff, int32_t *count, int64_t *sumj, int64_t *sumj2);

/* --- LJ + Coulomb (PD src/mmlib/forcefields/nonbonded.cpp:559-910) --- */
int pdo_nonbonded(const pdo_system *s, const pdo_nb_params *p, int nthreads, pdo_energies *e, double *force);

/* Stored half list as PD keeps it between rebuilds (neighbourlist.cpp:336-439):
 * for each i the j < i within ListCutoff at minimum image, with the image shift
 * fixed at build time.  pdo_list_build allocates; pdo_list_free releases. */
typedef struct {
    int natom;
    int64_t *start;    /* natom+1 */
    int32_t *j;
    double *shift;     /* 3 per entry: image shift added to pj - pi */
} pdo_list;
int pdo_list_build(const pdo_system *s, double list_cutoff, int nthreads, pdo_list *out);
void pdo_list_free(pdo_list *l);
/* LJ + Coulomb over a stored list (the per-step work of PD's MD loop) */
int pdo_nonbonded_list(const pdo_system *s, const pdo_list *l, const pdo_nb_params *p, int nthreads,
                       pdo_energies *e, double *force);

/* scalar pair law (PD src/mmlib/forcefields/nonbonded.cpp:400-534) */
void pdo_pair_law(const pdo_nb_params *p, double r, double radiusij, double epsilon, double qi, double qj,
                  double *vdw_pot, double *vdw_force, double *elec_pot, double *elec_force);

/* --- Generalised Born, Still (PD src/mmlib/forcefields/gbff.cpp) --- */
/* fixed (connectivity-only) terms, gbff.cpp:324-398 */
void pdo_gb_fixed_terms(int natom, const double *gb_radius, int ncov12, const int *cov12, const double *d12,
                        int ncov13, const int *cov13, const double *d13, const pdo_gb_params *p,
                        double *vj, double *terms123);
/* Born radii, gbff.cpp:432-483 */
int pdo_gb_born_radii(const pdo_system *s, const pdo_gb_params *p, const double *gb_radius, const double *vj,
                      const double *terms123, int nthreads, double *born);
/* FastMode forces incl. vacuum LJ/Coulomb, gbff.cpp:1466-1835 (radii recomputed first, gbff.cpp:185-197) */
int pdo_gb_forces(const pdo_system *s, const pdo_gb_params *p, const double *gb_radius, const double *vj,
                  const double *terms123, int nthreads, pdo_energies *e, double *force, double *born_out);

/* --- LCPO surface area (PD src/mmlib/forcefields/lcpo.cpp:640-961) --- */
int pdo_lcpo_forces(const pdo_system *s, double list_cutoff, const double *lcpo_radius, const double *P /*n*4*/,
                    const double *sigma, const int *use, int nthreads, pdo_energies *e, double *force, double *sasa);

/* --- integrators (PD src/mmlib/protocols/md.cpp) --- */
/* PD velocity Verlet as written (md.cpp:805-855): half kick, kinetic energy,
 * second half kick, drift with t*(v+dv), final kick.  Returns kinetic energy (J). */
double pdo_vv_step(int natom, double *pos, double *vel, const double *force, const double *mass, double dt);
/* PD Langevin (md.cpp:923-1063) for one step with caller-supplied unit
 * normals noise[natom*6] ordered (n1x,n2y,n2x,n1z,n1y,n2z) per atom as PD
 * draws them; first_step / last_step mirror the Step>0 / Step<Steps-1 guards. */
double pdo_langevin_step(int natom, double *pos, double *vel, const double *force, const double *mass, double dt,
                         double gamma, double T, const double *noise, int first_step, int last_step);
/* Langevin coefficients (c0, c1, c2, varv, varr, crv), md.cpp:966-1003 */
void pdo_langevin_coeffs(double gamma, double dt, double out[6]);

/* --- bonded terms used to keep the MD step physical (PD src/mmlib/forcefields/ffbonded.cpp) --- */
int pdo_bonded(int natom, const double *pos, int nbond, const int *bidx, const double *bpar, int nangle,
               const int *aidx, const double *apar, int ntors, const int *tidx, const double *tpar, int nimpr,
               const int *iidx, const double *ipar, double *energy, double *force);

#ifdef __cplusplus
}
#endif
#endif
