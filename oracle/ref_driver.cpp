// Fixture driver linked against the PD reference library (oracle/_ref/libmmlib.a).
//
// Test infrastructure only: it builds the synthetic systems with PD's own
// builders and parameter files, evaluates PD's own FP64 forcefield components
// on them, and writes everything (system description + reference energies,
// forces, Born radii, per-atom SASA, neighbour-list checksums, scalar pair-law
// scans) to a small tagged binary container that tests/golden/make_golden.py
// turns into .npz fixtures.
//
// Usage: ref_driver <water|peptide|solvated> <out.bin> [key=value ...]
//
// PD entry points exercised (paths inside the PD project):
//   Forcefield::calcForces            src/mmlib/forcefields/forcefield.cpp:237-264
//   FF_NonBonded (T_fast2 kernel)     src/mmlib/forcefields/nonbonded.cpp:559-910
//   FF_NonBonded::calc_LJ_Coulomb_Force src/mmlib/forcefields/nonbonded.cpp:400-534
//   FF_GeneralizedBorn_Still (fast)   src/mmlib/forcefields/gbff.cpp:1466-1835
//   FF_SASA_LCPO::calcLCPOSasaForces  src/mmlib/forcefields/lcpo.cpp:640-961
//   NeighbourList::calcNewList        src/mmlib/workspace/neighbourlist.cpp:222-439
//   NewProtein / setResiduePhiPsi     src/mmlib/system/genpolymer.cpp:284-298
//
// Access to the components' internal per-atom tables (Born radii, Vj, LCPO
// parameters) is obtained by compiling this one file with the access
// specifiers opened; class layouts are unchanged.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <map>
#include <set>
#include <sstream>
#include <ctime>

#define private public
#define protected public
#include "system/system.h"
#include "system/molecule.h"
#include "system/genpolymer.h"
#include "forcefields/ffparam.h"
#include "forcefields/forcefield.h"
#include "forcefields/ffbonded.h"
#include "forcefields/nonbonded.h"
#include "forcefields/gbff.h"
#include "forcefields/lcpo.h"
#include "workspace/workspace.h"
#include "workspace/space.h"
#include "workspace/neighbourlist.h"
#include "workspace/bondorder.h"
#include "protocols/md.h"
#include "protocols/minimise.h"
#undef private
#undef protected

using namespace Physics;

// ---------------------------------------------------------------------------
// tagged container writer: [u32 namelen][name][char dtype][u32 ndim][u64 dims][raw]
// ---------------------------------------------------------------------------
static FILE *g_out = NULL;
static void stage(const char *what) { fprintf(stderr, "[%8.2f s] %s\n", (double)clock() / CLOCKS_PER_SEC, what); }

static void put_array(const std::string &name, char dtype, const std::vector<unsigned long long> &dims,
                      const void *data, size_t elsize) {
    unsigned int nl = (unsigned int)name.size();
    fwrite(&nl, 4, 1, g_out);
    fwrite(name.data(), 1, nl, g_out);
    fwrite(&dtype, 1, 1, g_out);
    unsigned int nd = (unsigned int)dims.size();
    fwrite(&nd, 4, 1, g_out);
    size_t count = 1;
    for (size_t k = 0; k < dims.size(); k++) {
        unsigned long long d = dims[k];
        fwrite(&d, 8, 1, g_out);
        count *= (size_t)d;
    }
    if (count) fwrite(data, elsize, count, g_out);
}
static void put_f64(const std::string &n, const std::vector<double> &v, size_t cols = 1) {
    std::vector<unsigned long long> d;
    if (cols == 1) d.push_back(v.size());
    else { d.push_back(v.size() / cols); d.push_back(cols); }
    put_array(n, 'd', d, v.empty() ? NULL : &v[0], 8);
}
static void put_i32(const std::string &n, const std::vector<int> &v, size_t cols = 1) {
    std::vector<unsigned long long> d;
    if (cols == 1) d.push_back(v.size());
    else { d.push_back(v.size() / cols); d.push_back(cols); }
    put_array(n, 'i', d, v.empty() ? NULL : &v[0], 4);
}
static void put_i64(const std::string &n, const std::vector<long long> &v) {
    std::vector<unsigned long long> d(1, v.size());
    put_array(n, 'q', d, v.empty() ? NULL : &v[0], 8);
}
static void put_scalar(const std::string &n, double x) { put_f64(n, std::vector<double>(1, x)); }

// ---------------------------------------------------------------------------
// options
// ---------------------------------------------------------------------------
static std::map<std::string, std::string> g_opt;
static double optd(const char *k, double dflt) {
    std::map<std::string, std::string>::iterator it = g_opt.find(k);
    return it == g_opt.end() ? dflt : atof(it->second.c_str());
}
static std::string opts(const char *k, const char *dflt) {
    std::map<std::string, std::string>::iterator it = g_opt.find(k);
    return it == g_opt.end() ? std::string(dflt) : it->second;
}

// ---------------------------------------------------------------------------
// seeded generator (xorshift64*), independent of libc rand()
// ---------------------------------------------------------------------------
struct Rng {
    unsigned long long s;
    explicit Rng(unsigned long long seed) : s(seed * 0x9E3779B97F4A7C15ULL + 0x1234567ULL) { if (!s) s = 1; next(); }
    unsigned long long next() {
        s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
        return s * 2685821657736338717ULL;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

static Maths::matrix3x3 random_rotation(Rng &rng) {
    // uniform random unit quaternion (Shoemake 1992)
    double u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
    double a = sqrt(1 - u1), b = sqrt(u1);
    double qw = a * sin(2 * M_PI * u2), qx = a * cos(2 * M_PI * u2);
    double qy = b * sin(2 * M_PI * u3), qz = b * cos(2 * M_PI * u3);
    Maths::matrix3x3 m;
    m.r[0][0] = 1 - 2 * (qy * qy + qz * qz); m.r[0][1] = 2 * (qx * qy - qz * qw); m.r[0][2] = 2 * (qx * qz + qy * qw);
    m.r[1][0] = 2 * (qx * qy + qz * qw); m.r[1][1] = 1 - 2 * (qx * qx + qz * qz); m.r[1][2] = 2 * (qy * qz - qx * qw);
    m.r[2][0] = 2 * (qx * qz - qy * qw); m.r[2][1] = 2 * (qy * qz + qx * qw); m.r[2][2] = 1 - 2 * (qx * qx + qy * qy);
    return m;
}

static const char *AA = "ACDEFGHIKLMNPQRSTVWY";

static std::string random_sequence(int nres, Rng &rng) {
    std::string s;
    for (int k = 0; k < nres; k++) s += AA[rng.next() % 20];
    return s;
}

// "*A-(CDE...)-Y*" : PD sequence string with terminal residues outside the brackets
static std::string pd_sequence_string(const std::string &s) {
    std::string out = "*";
    out += s[0];
    out += "-(";
    out += s.substr(1, s.size() - 2);
    out += ")-";
    out += s[s.size() - 1];
    out += "*";
    return out;
}

static double mol_rgyr(Molecule &m) {
    double cx = 0, cy = 0, cz = 0;
    size_t n = m.nAtoms();
    for (size_t i = 0; i < n; i++) { cx += m.atomxyz(i).x; cy += m.atomxyz(i).y; cz += m.atomxyz(i).z; }
    cx /= n; cy /= n; cz /= n;
    double s = 0;
    for (size_t i = 0; i < n; i++) {
        double dx = m.atomxyz(i).x - cx, dy = m.atomxyz(i).y - cy, dz = m.atomxyz(i).z - cz;
        s += dx * dx + dy * dy + dz * dz;
    }
    return sqrt(s / n);
}

// Clash count on a 3 A cell grid: pairs further apart than 1-4 along the
// covalent graph that are closer than 2.6 A (two heavy atoms) or 1.8 A (any
// pair with a hydrogen).
static int mol_clashes(Molecule &m) {
    size_t n = m.nAtoms();
    const double cell = 3.0;
    std::map<long long, std::vector<int> > grid;
    for (size_t i = 0; i < n; i++) {
        const Maths::dvector &p = m.atomxyz(i);
        long long cx = (long long)floor(p.x / cell), cy = (long long)floor(p.y / cell), cz = (long long)floor(p.z / cell);
        grid[(cx * 1000003LL + cy) * 1000003LL + cz].push_back((int)i);
    }
    int count = 0;
    for (size_t i = 0; i < n; i++) {
        const Particle &ai = m.getAtom(i);
        const Maths::dvector &pi = m.atomxyz(i);
        long long cx = (long long)floor(pi.x / cell), cy = (long long)floor(pi.y / cell), cz = (long long)floor(pi.z / cell);
        bool hi = ai.Z == 1;
        for (int a = -1; a <= 1; a++) for (int b = -1; b <= 1; b++) for (int c = -1; c <= 1; c++) {
            std::map<long long, std::vector<int> >::iterator it = grid.find(((cx + a) * 1000003LL + (cy + b)) * 1000003LL + (cz + c));
            if (it == grid.end()) continue;
            for (size_t k = 0; k < it->second.size(); k++) {
                int j = it->second[k];
                if (j <= (int)i) continue;
                bool bonded = false;
                for (size_t q = 0; q < ai.cov12atom.size() && !bonded; q++) bonded = ai.cov12atom[q].i == j;
                for (size_t q = 0; q < ai.cov13atom.size() && !bonded; q++) bonded = ai.cov13atom[q].i == j;
                for (size_t q = 0; q < ai.cov14atom.size() && !bonded; q++) bonded = ai.cov14atom[q].i == j;
                if (bonded) continue;
                bool hj = m.getAtom(j).Z == 1;
                double lim = (hi || hj) ? 1.8 : 2.6;
                const Maths::dvector &pj = m.atomxyz(j);
                double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                if (dx * dx + dy * dy + dz * dz < lim * lim) count++;
            }
        }
    }
    return count;
}

// Compaction: seeded random phi/psi moves through PD's own torsion setter,
// accepted when the radius of gyration does not grow and no clash appears.
static void compact(Molecule &m, int moves, Rng &rng) {
    // each move picks one residue and tries `trials` random (phi, psi) pairs,
    // keeping the clash-free one with the smallest radius of gyration if it
    // does not grow
    int nres = (int)m.nResidues();
    int trials = (int)optd("trials", 12);
    double rg = mol_rgyr(m);
    int clashes = mol_clashes(m);
    fprintf(stderr, "compact: start Rg %.2f A, %d clashes\n", rg, clashes);
    size_t n = m.nAtoms();
    std::vector<Maths::dvector> save(n), best(n);
    int accepted = 0;
    for (int mv = 0; mv < moves; mv++) {
        int ir = 1 + (int)(rng.next() % (unsigned long long)(nres - 2));
        double phi, psi;
        m.calcResiduePhiPsi(ir, phi, psi);
        for (size_t i = 0; i < n; i++) save[i] = m.atomxyz(i);
        double brg = rg;
        int bcl = clashes;
        bool found = false;
        for (int t = 0; t < trials; t++) {
            double nphi = rng.uniform(-M_PI, M_PI);
            double npsi = rng.uniform(-M_PI, M_PI);
            m.setResiduePhiPsi(ir, nphi, npsi);
            double nrg = mol_rgyr(m);
            int ncl = (nrg < brg || clashes > 0) ? mol_clashes(m) : 1 << 30;
            if ((ncl < bcl) || (ncl == bcl && nrg < brg)) {
                brg = nrg; bcl = ncl; found = true;
                for (size_t i = 0; i < n; i++) best[i] = m.atomxyz(i);
            }
            for (size_t i = 0; i < n; i++) m.atomxyz(i) = save[i];
        }
        if (found) {
            for (size_t i = 0; i < n; i++) m.atomxyz(i) = best[i];
            rg = brg; clashes = bcl; accepted++;
        }
    }
    fprintf(stderr, "compact: %d/%d accepted, Rg %.2f A, %d clashes\n", accepted, moves, rg, clashes);
}

static void round_to_f32(WorkSpace &ws) {
    for (size_t i = 0; i < ws.nAtoms(); i++) {
        Maths::dvector &p = ws.cur.atom[i].p;
        p.x = (double)(float)p.x; p.y = (double)(float)p.y; p.z = (double)(float)p.z;
    }
}

// ---------------------------------------------------------------------------
// export helpers
// ---------------------------------------------------------------------------
static void export_system(WorkSpace &ws, const double box[3]) {
    size_t n = ws.nAtoms();
    std::vector<double> pos(3 * n), q(n), rad(n), eps(n), mass(n);
    std::vector<int> Z(n), ft(n), ir(n);
    for (size_t i = 0; i < n; i++) {
        pos[3 * i] = ws.cur.atom[i].p.x; pos[3 * i + 1] = ws.cur.atom[i].p.y; pos[3 * i + 2] = ws.cur.atom[i].p.z;
        q[i] = ws.atom[i].charge; rad[i] = ws.atom[i].radius; eps[i] = ws.atom[i].epsilon;
        mass[i] = ws.atom[i].mass; Z[i] = ws.atom[i].Z; ft[i] = ws.atom[i].FFType; ir[i] = ws.atom[i].ir;
    }
    put_f64("pos", pos, 3); put_f64("charge", q); put_f64("radius", rad); put_f64("epsilon", eps);
    put_f64("mass", mass); put_i32("Z", Z); put_i32("fftype", ft); put_i32("ires", ir);
    put_f64("box", std::vector<double>(box, box + 3));
}

// exclusion / 1-4 table as the neighbour list sees it: (j, i, bondorder) for j<i, bondorder<=3
// covalent 1-2 / 1-3 partners with the equilibrium distances FF_Bonded::setup
// stores in them (ffbonded.cpp:149,303); valid only after bonded setup
static void export_covalent(WorkSpace &ws) {
    size_t n = ws.nAtoms();
    std::vector<int> c12, c13; std::vector<double> d12, d13;
    for (size_t i = 0; i < n; i++) {
        for (size_t k = 0; k < ws.atom[i].cov12atom.size(); k++) {
            c12.push_back((int)i); c12.push_back(ws.atom[i].cov12atom[k].i); d12.push_back(ws.atom[i].cov12atom[k].d);
        }
        for (size_t k = 0; k < ws.atom[i].cov13atom.size(); k++) {
            c13.push_back((int)i); c13.push_back(ws.atom[i].cov13atom[k].i); d13.push_back(ws.atom[i].cov13atom[k].d);
        }
    }
    put_i32("cov12", c12, 2); put_f64("cov12d", d12); put_i32("cov13", c13, 2); put_f64("cov13d", d13);
}

static void export_exclusions(WorkSpace &ws) {
    const NeighbourData *nb = ws.nlist().getData();
    std::vector<int> ex;
    for (size_t i = 0; i < ws.nAtoms(); i++) {
        for (int k = 0; k < nb[i].n; k++) {
            unsigned int raw = (unsigned int)nb[i].i[k];
            int j = (int)(raw & 0x00FFFFFF);
            int bo = (int)((raw >> 24) & 7);
            if (j < (int)i && bo <= 3) { ex.push_back(j); ex.push_back((int)i); ex.push_back(bo); }
        }
    }
    put_i32("excl", ex, 3);
}

static void export_list_checksum(WorkSpace &ws, const std::string &tag) {
    const NeighbourData *nb = ws.nlist().getData();
    size_t n = ws.nAtoms();
    std::vector<int> cnt(n);
    std::vector<long long> s1(n), s2(n);
    for (size_t i = 0; i < n; i++) {
        int c = 0; long long a = 0, b = 0;
        for (int k = 0; k < nb[i].n; k++) {
            int j = (int)((unsigned int)nb[i].i[k] & 0x00FFFFFF);
            if (j >= (int)i) continue;
            c++; a += j; b += (long long)j * j;
        }
        cnt[i] = c; s1[i] = a; s2[i] = b;
    }
    put_i32(tag + "_n", cnt); put_i64(tag + "_sumj", s1); put_i64(tag + "_sumj2", s2);
}

static void export_result(WorkSpace &ws, const std::string &tag) {
    size_t n = ws.nAtoms();
    std::vector<double> f(3 * n);
    for (size_t i = 0; i < n; i++) {
        f[3 * i] = ws.cur.atom[i].f.x; f[3 * i + 1] = ws.cur.atom[i].f.y; f[3 * i + 2] = ws.cur.atom[i].f.z;
    }
    const Hamiltonian &e = ws.ene;
    double ene[8] = {e.epot, e.epot_vdw, e.epot_elec, e.epot_pol, e.epot_pol_self, e.epot_pol_cross, e.epot_surf, e.InternalVirial};
    put_f64(tag + "_ene", std::vector<double>(ene, ene + 8));
    put_f64(tag + "_f", f, 3);
}

static void configure_nb(FF_NonBonded &nb) {
    nb.Cutoff = optd("cutoff", 12); nb.InnerCutoff = optd("inner", 10);
    nb.VdwCutoff = optd("vdwcut", nb.Cutoff); nb.VdwInnerCutoff = optd("vdwinner", nb.InnerCutoff);
    std::string mode = opts("elec", "eswitch");
    nb.EnergySwitch = (mode == "eswitch");
    nb.ForceSwitch = (mode == "fswitch");
    nb.Dielectric = optd("dielectric", 1.0);
    nb.DoVdw = optd("dovdw", 1) != 0; nb.DoElec = optd("doelec", 1) != 0;
}

static void export_settings(const std::string &prefix, FF_NonBonded &nb) {
    put_scalar(prefix + "Cutoff", nb.Cutoff); put_scalar(prefix + "InnerCutoff", nb.InnerCutoff);
    put_scalar(prefix + "VdwCutoff", nb.VdwCutoff); put_scalar(prefix + "VdwInnerCutoff", nb.VdwInnerCutoff);
    put_scalar(prefix + "Vdw14Scaling", nb.Vdw14Scaling); put_scalar(prefix + "Elec14Scaling", nb.Elec14Scaling);
    put_scalar(prefix + "Dielectric", nb.Dielectric);
    put_scalar(prefix + "EnergySwitch", nb.EnergySwitch ? 1 : 0); put_scalar(prefix + "ForceSwitch", nb.ForceSwitch ? 1 : 0);
    put_scalar(prefix + "DoVdw", nb.DoVdw ? 1 : 0); put_scalar(prefix + "DoElec", nb.DoElec ? 1 : 0);
}

static void scan_pair_law(WorkSpace &ws) {
    // r-scan of the scalar pair law for every electrostatics mode
    const char *modes[3] = {"eswitch", "fswitch", "normal"};
    for (int m = 0; m < 3; m++) {
        FF_NonBonded nb(ws);
        nb.Cutoff = 12; nb.InnerCutoff = 9; nb.VdwCutoff = 12; nb.VdwInnerCutoff = 9;
        nb.EnergySwitch = (m == 0); nb.ForceSwitch = (m == 1);
        std::vector<double> out;
        for (double r = 2.5; r < nb.Cutoff; r += 0.025) {
            double vp, vf, ep, ef;
            nb.calc_LJ_Coulomb_Force(r, 1 / r, 3.0, 1.0 / (PhysicsConst::J2kcal * PhysicsConst::Na), 1, 1, vp, vf, ep, ef);
            out.push_back(r); out.push_back(vp); out.push_back(vf); out.push_back(ep); out.push_back(ef);
        }
        put_f64(std::string("scan_") + modes[m], out, 5);
    }
}

static void export_bonded_terms(FF_Bonded &b) {
    std::vector<int> bi, ai, ti, ii;
    std::vector<double> bp, ap, tp, ip;
    for (size_t k = 0; k < b.bond.size(); k++) {
        bi.push_back(b.bond[k].i); bi.push_back(b.bond[k].j);
        bp.push_back(b.bond[k].l); bp.push_back(b.bond[k].k);
    }
    for (size_t k = 0; k < b.angle.size(); k++) {
        ai.push_back(b.angle[k].i); ai.push_back(b.angle[k].a); ai.push_back(b.angle[k].j);
        ap.push_back(b.angle[k].theta0); ap.push_back(b.angle[k].k);
    }
    for (int pass = 0; pass < 2; pass++) {
        std::vector<Torsion> &T = pass == 0 ? b.torsion : b.improper;
        std::vector<int> &I = pass == 0 ? ti : ii;
        std::vector<double> &P = pass == 0 ? tp : ip;
        for (size_t k = 0; k < T.size(); k++) {
            I.push_back(T[k].i); I.push_back(T[k].a); I.push_back(T[k].b); I.push_back(T[k].j); I.push_back(T[k].terms);
            for (int t = 0; t < 4; t++) { P.push_back(T[k].Vn[t]); P.push_back(T[k].n[t]); P.push_back(T[k].gamma[t]); }
        }
    }
    put_i32("bond_idx", bi, 2); put_f64("bond_par", bp, 2);
    put_i32("angle_idx", ai, 3); put_f64("angle_par", ap, 2);
    put_i32("torsion_idx", ti, 5); put_f64("torsion_par", tp, 12);
    put_i32("improper_idx", ii, 5); put_f64("improper_par", ip, 12);
}

static void evaluate(Forcefield &ff, WorkSpace &ws) {
    ff.ensuresetup(ws);
    ws.nlist().calcNewList();
    ff.calcForces();
}

// ---------------------------------------------------------------------------
// systems
// ---------------------------------------------------------------------------
// Rotate a molecule about its centre so that its principal axes (largest
// spread first) lie along the cubic box's body diagonal, face diagonal and
// the remaining orthogonal direction; an elongated chain then fits a box
// shorter than its length without touching its periodic images.
static void align_to_box_diagonal(Molecule &m) {
    m.zeroCentreOfGeometry();
    size_t n = m.nAtoms();
    double c[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (size_t i = 0; i < n; i++) {
        double p[3] = {m.atomxyz(i).x, m.atomxyz(i).y, m.atomxyz(i).z};
        for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) c[a][b] += p[a] * p[b];
    }
    // Jacobi eigen-decomposition of the 3x3 covariance
    double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 50; sweep++) {
        for (int p = 0; p < 2; p++) for (int q = p + 1; q < 3; q++) {
            if (fabs(c[p][q]) < 1e-12) continue;
            double th = 0.5 * atan2(2 * c[p][q], c[q][q] - c[p][p]);
            double cs = cos(th), sn = sin(th);
            for (int k = 0; k < 3; k++) {
                double ckp = c[k][p], ckq = c[k][q];
                c[k][p] = cs * ckp - sn * ckq; c[k][q] = sn * ckp + cs * ckq;
            }
            for (int k = 0; k < 3; k++) {
                double cpk = c[p][k], cqk = c[q][k];
                c[p][k] = cs * cpk - sn * cqk; c[q][k] = sn * cpk + cs * cqk;
            }
            for (int k = 0; k < 3; k++) {
                double vkp = v[k][p], vkq = v[k][q];
                v[k][p] = cs * vkp - sn * vkq; v[k][q] = sn * vkp + cs * vkq;
            }
        }
    }
    int ord[3] = {0, 1, 2};
    for (int a = 0; a < 3; a++) for (int b = a + 1; b < 3; b++)
        if (c[ord[b]][ord[b]] > c[ord[a]][ord[a]]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
    const double s3 = 1 / sqrt(3.0), s2 = 1 / sqrt(2.0), s6 = 1 / sqrt(6.0);
    double target[3][3] = {{s3, s3, s3}, {s2, -s2, 0}, {s6, s6, -2 * s6}};
    for (size_t i = 0; i < n; i++) {
        double p[3] = {m.atomxyz(i).x, m.atomxyz(i).y, m.atomxyz(i).z};
        double np_[3] = {0, 0, 0};
        for (int k = 0; k < 3; k++) {
            double proj = p[0] * v[0][ord[k]] + p[1] * v[1][ord[k]] + p[2] * v[2][ord[k]];
            for (int a = 0; a < 3; a++) np_[a] += proj * target[k][a];
        }
        m.atomxyz(i).x = np_[0]; m.atomxyz(i).y = np_[1]; m.atomxyz(i).z = np_[2];
    }
}

static double min_image_contact(Molecule &m, double box) {
    // closest heavy-atom approach between the molecule and its periodic images
    double best = 1e30;
    size_t n = m.nAtoms();
    for (size_t i = 0; i < n; i++) {
        if (m.getAtom(i).Z == 1) continue;
        for (size_t j = i; j < n; j++) {
            if (m.getAtom(j).Z == 1) continue;
            for (int a = -1; a <= 1; a++) for (int b = -1; b <= 1; b++) for (int c = -1; c <= 1; c++) {
                if (!a && !b && !c) continue;
                double dx = m.atomxyz(j).x - m.atomxyz(i).x + a * box;
                double dy = m.atomxyz(j).y - m.atomxyz(i).y + b * box;
                double dz = m.atomxyz(j).z - m.atomxyz(i).z + c * box;
                double d2 = dx * dx + dy * dy + dz * dz;
                if (d2 < best) best = d2;
            }
        }
    }
    return sqrt(best);
}

static void add_waters_lattice(System &sim, FFParamSet &ffps, int nwat_max, double box, int per_side,
                               Rng &rng, double jitter, const Molecule *solute, double excl_dist) {
    Molecule water = NewMolecule(ffps, "TIP3");
    water.zeroCentreOfGeometry();
    double sp = box / per_side;
    int added = 0;
    for (int a = 0; a < per_side && added < nwat_max; a++)
        for (int b = 0; b < per_side && added < nwat_max; b++)
            for (int c = 0; c < per_side && added < nwat_max; c++) {
                Maths::dvector site((a + 0.5) * sp - box / 2 + rng.uniform(-jitter, jitter),
                                    (b + 0.5) * sp - box / 2 + rng.uniform(-jitter, jitter),
                                    (c + 0.5) * sp - box / 2 + rng.uniform(-jitter, jitter));
                Maths::matrix3x3 rot = random_rotation(rng);
                if (solute) {
                    bool clash = false;
                    double e2 = excl_dist * excl_dist;
                    for (size_t k = 0; k < solute->nAtoms() && !clash; k++) {
                        const Maths::dvector &p = solute->atomxyz(k);
                        double dx = p.x - site.x, dy = p.y - site.y, dz = p.z - site.z;
                        dx -= box * floor(dx / box + 0.5); dy -= box * floor(dy / box + 0.5); dz -= box * floor(dz / box + 0.5);
                        if (dx * dx + dy * dy + dz * dz < e2) clash = true;
                    }
                    if (clash) continue;
                }
                Molecule w(water);
                w.rotate(rot);
                w.move(site);
                sim.add(w);
                added++;
            }
    fprintf(stderr, "waters added: %d\n", added);
}

// Relieve builder clashes with PD's own conjugate-gradient minimiser (bonded
// terms + switched vacuum LJ and Coulomb, 10/8 A) on the bare peptide, then
// copy the minimised coordinates back into the molecule.
static void minimise_molecule(FFParamSet &ffps, Molecule &m, int minsteps) {
    if (minsteps <= 0) return;
    fprintf(stderr, "before minimisation: Rg %.2f A, clashes %d\n", mol_rgyr(m), mol_clashes(m));
    System tmp(ffps);
    tmp.add(m);
    WorkSpace ws(tmp);
    FF_Bonded mb(ws);
    FF_NonBonded mnb(ws);
    mnb.Cutoff = 10; mnb.InnerCutoff = 8; mnb.VdwCutoff = 10; mnb.VdwInnerCutoff = 8;
    mnb.EnergySwitch = true; mnb.ForceSwitch = false;
    Forcefield mff(ws);
    mff.add(mb);
    mff.add(mnb);
    Protocol::Minimisation mini(mff);
    mini.Algorithm = optd("mincg", 0) != 0 ? Protocol::Minimisation::ConjugateGradients : Protocol::Minimisation::SteepestDescent;
    mini.Steps = minsteps;
    mini.StepSize = optd("minstep", 2E5);
    mini.UpdateScr = 0;
    mini.UpdateTra = 0;
    mini.UpdateNList = 10;
    mini.OutputLevel = Verbosity::Silent;
    mini.run();
    for (size_t i = 0; i < m.nAtoms(); i++) m.atomxyz(i) = ws.cur.atom[i].p;
    fprintf(stderr, "minimised: Rg %.2f A, natoms %d\n", mol_rgyr(m), (int)m.nAtoms());
}

static Molecule build_peptide(FFParamSet &ffps, int nres, int moves, Rng &rng, std::string &seq) {
    seq = random_sequence(nres, rng);
    Molecule m = NewProtein(ffps, pd_sequence_string(seq));
    compact(m, moves, rng);
    minimise_molecule(ffps, m, (int)optd("minimise", 200));
    m.zeroCentreOfGeometry();
    return m;
}

int main(int argc, char **argv) {
    if (argc < 3) { fprintf(stderr, "usage: ref_driver <water|peptide|solvated> <out.bin> [k=v ...]\n"); return 2; }
    std::string kind = argv[1];
    for (int a = 3; a < argc; a++) {
        std::string kv = argv[a];
        size_t e = kv.find('=');
        if (e != std::string::npos) g_opt[kv.substr(0, e)] = kv.substr(e + 1);
    }
    unsigned long long seed = (unsigned long long)optd("seed", 1);
    Rng rng(seed);
    srand((unsigned)seed);

    g_out = fopen(argv[2], "wb");
    if (!g_out) { perror("open"); return 1; }

    FFParamSet ffps;
    double box[3] = {0, 0, 0};
    System sim(ffps);
    std::string seq;

    if (kind == "water") {
        ffps.readLib("tip3.ff");
        double L = optd("box", 27.5);
        int nwat = (int)optd("nwat", 667);
        int side = (int)ceil(pow((double)nwat, 1.0 / 3.0) - 1e-9);
        add_waters_lattice(sim, ffps, nwat, L, side, rng, optd("jitter", 0.2), NULL, 0);
        box[0] = box[1] = box[2] = L;
    } else if (kind == "peptide" || kind == "solvated") {
        ffps.readLib(opts("ff", "amber99aa.ff").c_str());
        if (kind == "solvated") ffps.readLib("tip3.ff");
        Molecule prot = build_peptide(ffps, (int)optd("nres", 20), (int)optd("moves", 500), rng, seq);
        sim.add(prot);
        if (kind == "solvated") {
            double L = optd("box", 62.0);
            align_to_box_diagonal(prot);
            sim.getMolecule(0) = prot;
            fprintf(stderr, "closest heavy-atom contact with a periodic image: %.2f A\n", min_image_contact(prot, L));
            int side = (int)optd("side", 20);
            add_waters_lattice(sim, ffps, 1 << 30, L, side, rng, optd("jitter", 0.2), &prot, optd("exclude", 2.8));
            box[0] = box[1] = box[2] = L;
        }
    } else {
        fprintf(stderr, "unknown kind %s\n", kind.c_str());
        return 2;
    }

    stage("system built");
    WorkSpace ws(sim);
    stage("workspace created");
    PeriodicBox *pbox = NULL;
    if (box[0] > 0) { pbox = new PeriodicBox(box[0], box[1], box[2]); ws.setSpace(pbox); }
    ws.nlist().setPadding(optd("padding", 2.0));
    stage("minimised");
    round_to_f32(ws);

    put_scalar("cfg_padding", optd("padding", 2.0));
    put_scalar("cfg_seed", (double)seed);
    if (!seq.empty()) {
        std::vector<int> s(seq.begin(), seq.end());
        put_i32("sequence", s);
    }
    export_system(ws, box);

    bool want_gb = optd("gb", kind == "peptide" ? 1 : 0) != 0;
    bool want_sasa = optd("sasa", kind == "peptide" ? 1 : 0) != 0;
    bool want_nb = optd("nb", 1) != 0;

    FF_Bonded bonds(ws);
    Forcefield ffb(ws);
    ffb.add(bonds);
    evaluate(ffb, ws);
    export_result(ws, "bonded");
    export_bonded_terms(bonds);
    export_covalent(ws);

    // keep component objects alive across cases (the list cutoff is the max of all requests)
    FF_GeneralizedBorn_Still gb(ws);
    FF_SASA_LCPO sasa(ws);
    FF_NonBonded nb(ws);

    if (want_gb) {
        gb.Cutoff = optd("gbcutoff", 12); gb.InnerCutoff = optd("gbinner", 9);
        gb.VdwCutoff = optd("gbvdwcut", gb.Cutoff); gb.VdwInnerCutoff = optd("gbvdwinner", gb.InnerCutoff);
        gb.GbsaStillCutoff = optd("gbsastill", 10);
        gb.FastMode = true;
        Forcefield ff(ws);
        ff.add(gb);
        evaluate(ff, ws);
        export_result(ws, "gb");
        export_settings("gb_", gb);
        put_scalar("gb_GbsaStillCutoff", gb.GbsaStillCutoff);
        put_scalar("gb_DielectricSolvent", gb.DielectricSolvent);
        put_scalar("gb_DielectricSolute", gb.DielectricSolute);
        put_scalar("gb_ExpApproxThreshold", gb.ExpApproxThreshold);
        put_scalar("gb_DielectricOffset", gb.DielectricOffset);
        put_scalar("gb_BornRadiusOffset", gb.BornRadiusOffset);
        double P[5] = {gb.P1, gb.P2, gb.P3, gb.P4, gb.P5};
        put_f64("gb_P", std::vector<double>(P, P + 5));
        size_t n = ws.nAtoms();
        std::vector<double> R(n), vj(n), t123(n), born(n);
        for (size_t i = 0; i < n; i++) {
            R[i] = gb.GBtype[ws.atom[i].FFType].radius;
            vj[i] = gb.GB_atom_param_still[i].Vj;
            t123[i] = gb.GB_atom_param_still[i].terms123;
            born[i] = gb.GB_atom_param[i].bornradius;
        }
        put_f64("gb_radius", R); put_f64("gb_vj", vj); put_f64("gb_terms123", t123); put_f64("gb_born", born);
        // FastMode = false: FF_NonBonded::calcForces + calcBornForces (gbff.cpp:185-197, 1189-1437)
        gb.FastMode = false;
        {
            Forcefield ff2(ws);
            ff2.add(gb);
            evaluate(ff2, ws);
            export_result(ws, "gbslow");
        }
        // calcEnergies (gbff.cpp:178-183): Born radii, FF_NonBonded::calcEnergies, calcBornEnergy
        {
            Forcefield ff3(ws);
            ff3.add(gb);
            ff3.ensuresetup(ws);
            ws.nlist().calcNewList();
            ff3.calcEnergies();
            const Hamiltonian &e = ws.ene;
            double ene[8] = {e.epot, e.epot_vdw, e.epot_elec, e.epot_pol, e.epot_pol_self, e.epot_pol_cross,
                             e.epot_surf, e.InternalVirial};
            put_f64("gbene_ene", std::vector<double>(ene, ene + 8));
        }
        gb.FastMode = true;
    }
    if (want_sasa) {
        sasa.GlobalASP = optd("asp", 0.005);
        sasa.UpdateSasa = 1;
        Forcefield ff(ws);
        ff.add(sasa);
        evaluate(ff, ws);
        export_result(ws, "sasa");
        size_t n = ws.nAtoms();
        std::vector<double> P(4 * n), r(n), sig(n), sa(n);
        std::vector<int> use(n);
        for (size_t i = 0; i < n; i++) {
            P[4 * i] = sasa.SASAatom[i].P1; P[4 * i + 1] = sasa.SASAatom[i].P2;
            P[4 * i + 2] = sasa.SASAatom[i].P3; P[4 * i + 3] = sasa.SASAatom[i].P4;
            r[i] = sasa.SASAatom[i].radius; sig[i] = sasa.SASAatom[i].sigma;
            use[i] = sasa.SASAatom[i].use; sa[i] = sasa.SASAatom[i].SASA;
        }
        put_f64("lcpo_P", P, 4); put_f64("lcpo_radius", r); put_f64("lcpo_sigma", sig);
        put_i32("lcpo_use", use); put_f64("lcpo_sasa", sa);
        put_scalar("lcpo_GlobalASP", sasa.GlobalASP);
    }
    if (want_nb) {
        configure_nb(nb);
        Forcefield ff(ws);
        ff.add(nb);
        evaluate(ff, ws);
        export_result(ws, "nb");
        export_settings("nb_", nb);
    }
    // list radius = max of all requested cutoffs + padding
    put_scalar("cfg_list_cutoff", ws.nlist().Cutoff);
    export_list_checksum(ws, "nl");
    // bonded partners are always closer than 7 A: make sure the list reaches them
    if (ws.nlist().Cutoff < 7.0) { ws.nlist().requestCutoff(7.0); ws.nlist().calcNewList(); }
    export_exclusions(ws);
    if (optd("scan", 0) != 0) scan_pair_law(ws);

    fclose(g_out);
    fprintf(stderr, "natoms=%d written %s\n", (int)ws.nAtoms(), argv[2]);
    return 0;
}
