// ff_gpu.h — PD forcefield components evaluated by libpdgpu on the GPU.
//
// What a PD maintainer adds under src/mods/pdgpu/ (with pdgpu.i): drop-in
// subclasses of PD's FF_NonBonded and FF_GeneralizedBorn_Still that keep every
// public attribute and PD's setup(), and replace the pair loops
// (nonbonded.cpp:559-910; gbff.cpp:432-483, 1466-1835) by the C ABI of
// include/pdgpu.h.  PD's setup() still reads the parameter file (types,
// radii, GB fixed terms); these classes copy the per-atom results to the
// device and add energies and forces into the WorkSpace as PD's own
// components do (forcefield.cpp:237-264).  The GB300 context follows the
// WorkSpace's atom order, so positions and forces cross the boundary in PD's
// own SnapShotAtom layout (72-byte stride).
//
// FF_SASA_LCPO keeps its per-atom LCPO table private (lcpo.h:119-122), so
// FF_SASA_LCPO_GPU is a ForcefieldBase of its own with FF_SASA_LCPO's public
// attributes: its setup() rebuilds the table from the WorkSpace and the
// parameter set's LCPOSASAPARAMETERS (and optional ASP) sections as
// FF_SASA_LCPO::setup does (lcpo.cpp:33-127, 224-305, 310-390), with no edit to
// PD's headers.
#ifndef PDGPU_PD_PLUGIN_FF_GPU_H
#define PDGPU_PD_PLUGIN_FF_GPU_H

#include <limits>
#include <vector>

#include "forcefields/ffparam.h"
#include "forcefields/gbff.h"
#include "forcefields/nonbonded.h"
#include "maths/maths.h"
#include "tools/stringtool.h"
#include "pdgpu.h"
#include "workspace/bondorder.h"
#include "workspace/neighbourlist.h"
#include "workspace/space.h"
#include "workspace/workspace.h"

namespace Physics {

namespace pdgpu_plugin {

// A WorkSpace's per-atom arrays and bonded-pair classes in the C ABI's layout.
struct SystemArrays {
  int n;
  double box[3];
  std::vector<double> charge, radius, epsilon, mass;
  std::vector<int> excl;  // (i, j, bond order 1..3) for the 1-2, 1-3 and 1-4 pairs

  void gather(WorkSpace& ws) {
    n = ws.nAtoms();
    charge.resize(n);
    radius.resize(n);
    epsilon.resize(n);
    mass.resize(n);
    for (int i = 0; i < n; i++) {
      charge[i] = ws.atom[i].charge;    // e
      radius[i] = ws.atom[i].radius;    // LJ Rmin/2 (A)
      epsilon[i] = ws.atom[i].epsilon;  // sqrt(J), PD's storage
      mass[i] = ws.atom[i].mass;        // kg
    }
    // bond orders as PD's neighbour list packs them (neighbourlist.cpp:398-408)
    const BondOrder& bo = ws.bondorder();
    excl.clear();
    for (int i = 0; i < n; i++) {
      const int jmax = i + bo.getMaxIndexDelta() < n - 1 ? i + bo.getMaxIndexDelta() : n - 1;
      for (int j = i + 1; j <= jmax; j++) {
        const int o = bo.getBondOrder(i, j);
        if (o >= 1 && o <= 3) {
          excl.push_back(i);
          excl.push_back(j);
          excl.push_back(o);
        }
      }
    }
    const std::vector<LongBondOrder>& far = bo.getOffDiagData();
    for (size_t k = 0; k < far.size(); k++)
      for (size_t p = 0; p < far[k].partner.size(); p++) {
        const int i = far[k].i, j = far[k].partner[p].j, o = far[k].partner[p].order;
        if (j > i && bo.isOffDiag(i, j) && o >= 1 && o <= 3) {
          excl.push_back(i);
          excl.push_back(j);
          excl.push_back(o);
        }
      }
    box[0] = box[1] = box[2] = 0.0;  // infinite space
    const PeriodicBox* pbox = dynamic_cast<const PeriodicBox*>(&ws.boundary());
    if (pbox) {
      Maths::dvector A, B, C;
      pbox->getBoxVectors(A, B, C);
      box[0] = A.x;
      box[1] = B.y;
      box[2] = C.z;
    }
  }

  void fill(pdgpu_system_desc& d) {
    d.nsystems = 1;
    d.natoms = &n;
    d.box = box;
    d.charge = &charge[0];
    d.radius = &radius[0];
    d.epsilon = &epsilon[0];
    d.mass = &mass[0];
    d.nexcl = (int)(excl.size() / 3);
    d.excl = excl.empty() ? 0 : &excl[0];
  }
};

inline void check(int status) {
  if (status != PDGPU_OK) throw ProcedureException(pdgpu_error_string(status));
}

// the device list's skin (PD keeps NeighbourListBase::Padding protected, so the
// components carry their own copy, default PD's 0.5 A, neighbourlist.cpp:35)
inline pdgpu_list_params list_params(double padding) {
  pdgpu_list_params lp;
  lp.Padding = padding;
  lp.check_skin = 1;
  return lp;
}

}  // namespace pdgpu_plugin

// FF_NonBonded on the GPU: LJ + Coulomb with PD's switches.
class FF_NonBonded_GPU : public FF_NonBonded {
 public:
  FF_NonBonded_GPU(WorkSpace& ws) : FF_NonBonded(ws), ListPadding(0.5), ctx(0) {}
  // a copy sets up its own device context on first use
  FF_NonBonded_GPU(const FF_NonBonded_GPU& other) : FF_NonBonded(other), ListPadding(other.ListPadding), ctx(0) {}
  virtual FF_NonBonded_GPU* clone() const { return new FF_NonBonded_GPU(*this); }
  virtual ~FF_NonBonded_GPU() {
    if (ctx) pdgpu_destroy(ctx);
  }

  double ListPadding;  // skin of the device list (A); set it like the WorkSpace list's Padding

 protected:
  pdgpu_ctx* ctx;

  pdgpu_nb_params nb_params() const {
    pdgpu_nb_params p;
    p.Cutoff = Cutoff;
    p.InnerCutoff = InnerCutoff;
    p.VdwCutoff = VdwCutoff;
    p.VdwInnerCutoff = VdwInnerCutoff;
    p.Vdw14Scaling = Vdw14Scaling;
    p.Elec14Scaling = Elec14Scaling;
    p.Dielectric = Dielectric;
    p.EnergySwitch = EnergySwitch ? 1 : 0;
    p.ForceSwitch = ForceSwitch ? 1 : 0;
    p.DoVdw = DoVdw ? 1 : 0;
    p.DoElec = DoElec ? 1 : 0;
    return p;
  }

  virtual void setup() {
    FF_NonBonded::setup();  // 1-4 scalings from the parameter set, basis vectors
    WorkSpace& ws = getWSpace();
    pdgpu_plugin::SystemArrays a;
    a.gather(ws);
    pdgpu_system_desc d = pdgpu_system_desc();
    a.fill(d);
    if (ctx) pdgpu_destroy(ctx);
    int st = PDGPU_OK;
    ctx = pdgpu_create(0, &d, &st);
    if (!ctx) pdgpu_plugin::check(st);
    const pdgpu_nb_params p = nb_params();
    pdgpu_plugin::check(pdgpu_set_nb_params(ctx, &p));
    const pdgpu_list_params lp = pdgpu_plugin::list_params(ListPadding);
    pdgpu_plugin::check(pdgpu_set_list_params(ctx, &lp));
  }

  void evaluate(bool forces) {
    WorkSpace& ws = getWSpace();
    pdgpu_plugin::check(pdgpu_set_positions(ctx, &ws.cur.atom[0].p.x, sizeof(SnapShotAtom)));
    pdgpu_energies e;
    const int st = pdgpu_compute(ctx, PDGPU_NB, &e, forces ? &ws.cur.atom[0].f.x : 0, sizeof(SnapShotAtom));
    if (st == PDGPU_ERR_NAN) {  // ProtocolBase::assertStability turns a NaN epot into an exception
      ws.ene.epot = std::numeric_limits<double>::quiet_NaN();
      return;
    }
    pdgpu_plugin::check(st);
    // VdwCor (nonbonded.cpp:862-874): PD's pair loop adds, for every atom i, the
    // analytic integral of the attractive LJ term from VdwCorCutoff to infinity,
    // an energy without force
    double cor = 0.0;
    if (VdwCor) {
      const double r2 = VdwCorRadius * VdwCorRadius;
      cor = ws.nAtoms() * (-0.5 * VdwCorDensity * VdwCorEpsilon / (PhysicsConst::J2kcal * PhysicsConst::Na) *
                           (8.0 / 3.0) * Maths::MathConst::PI * r2 * r2 * r2 /
                           (VdwCorCutoff * VdwCorCutoff * VdwCorCutoff));
    }
    // PD overwrites epot_vdw / epot_elec and adds to epot (nonbonded.cpp:681-682, 826, 871)
    ws.ene.epot += e.vdw + cor + e.elec;
    ws.ene.epot_vdw = e.vdw + cor;
    ws.ene.epot_vdw_att += cor;
    ws.ene.epot_elec = e.elec;
    ws.ene.InternalVirial += e.virial;
    epot_vdw = e.vdw + cor;
    epot_elec = e.elec;
    epot = e.vdw + cor + e.elec;
  }

  virtual void calcForces() { evaluate(true); }
  virtual void calcEnergies() { evaluate(false); }
};

// FF_GeneralizedBorn_Still on the GPU (FastMode): Born radii, the GB cross term
// fused with vacuum LJ + Coulomb, self energies and the chain rule.
class FF_GeneralizedBorn_Still_GPU : public FF_GeneralizedBorn_Still {
 public:
  FF_GeneralizedBorn_Still_GPU(WorkSpace& ws) : FF_GeneralizedBorn_Still(ws), ListPadding(0.5), ctx(0) {}
  FF_GeneralizedBorn_Still_GPU(const FF_GeneralizedBorn_Still_GPU& other)
      : FF_GeneralizedBorn_Still(other), ListPadding(other.ListPadding), ctx(0) {}
  virtual FF_GeneralizedBorn_Still_GPU* clone() const { return new FF_GeneralizedBorn_Still_GPU(*this); }
  virtual ~FF_GeneralizedBorn_Still_GPU() {
    if (ctx) pdgpu_destroy(ctx);
  }

  double ListPadding;  // skin of the device list (A); set it like the WorkSpace list's Padding

 protected:
  pdgpu_ctx* ctx;

  virtual void setup() {
    FF_GeneralizedBorn_Still::setup();  // GB types, Vj and terms123 (gbff.cpp:57-104, 324-398)
    WorkSpace& ws = getWSpace();
    pdgpu_plugin::SystemArrays a;
    a.gather(ws);
    const int n = a.n;
    std::vector<double> R(n), vj(n), t(n);
    for (int i = 0; i < n; i++) {
      R[i] = GBtype[ws.atom[i].FFType].radius;  // raw type radius, as PD's CCF uses it
      vj[i] = GB_atom_param_still[i].Vj;
      t[i] = GB_atom_param_still[i].terms123;
    }
    pdgpu_system_desc d = pdgpu_system_desc();
    a.fill(d);
    d.gb_radius = &R[0];
    d.gb_vj = &vj[0];
    d.gb_terms123 = &t[0];
    if (ctx) pdgpu_destroy(ctx);
    int st = PDGPU_OK;
    ctx = pdgpu_create(0, &d, &st);
    if (!ctx) pdgpu_plugin::check(st);
    pdgpu_gb_params p;
    p.Cutoff = Cutoff;
    p.InnerCutoff = InnerCutoff;
    p.VdwCutoff = VdwCutoff;
    p.VdwInnerCutoff = VdwInnerCutoff;
    p.Vdw14Scaling = Vdw14Scaling;
    p.Elec14Scaling = Elec14Scaling;
    p.DielectricSolute = DielectricSolute;
    p.DielectricSolvent = DielectricSolvent;
    p.GbsaStillCutoff = GbsaStillCutoff;
    p.ExpApproxThreshold = ExpApproxThreshold;
    p.BornRadiusOffset = BornRadiusOffset;
    p.P4 = P4;
    p.P5 = P5;
    pdgpu_plugin::check(pdgpu_set_gb_params(ctx, &p));
    // FastMode off / calcEnergies run the vacuum part with this object's own
    // FF_NonBonded settings (gbff.cpp:178-197)
    pdgpu_nb_params vac;
    vac.Cutoff = Cutoff;
    vac.InnerCutoff = InnerCutoff;
    vac.VdwCutoff = VdwCutoff;
    vac.VdwInnerCutoff = VdwInnerCutoff;
    vac.Vdw14Scaling = Vdw14Scaling;
    vac.Elec14Scaling = Elec14Scaling;
    vac.Dielectric = Dielectric;
    vac.EnergySwitch = EnergySwitch ? 1 : 0;
    vac.ForceSwitch = ForceSwitch ? 1 : 0;
    vac.DoVdw = DoVdw ? 1 : 0;
    vac.DoElec = DoElec ? 1 : 0;
    pdgpu_plugin::check(pdgpu_set_gb_mode(ctx, FastMode ? 1 : 0, &vac));
    // the same settings as this context's FF_NonBonded part: calcEnergies runs
    // FF_NonBonded::calcEnergies with them (gbff.cpp:178-183)
    pdgpu_plugin::check(pdgpu_set_nb_params(ctx, &vac));
    const pdgpu_list_params lp = pdgpu_plugin::list_params(ListPadding);
    pdgpu_plugin::check(pdgpu_set_list_params(ctx, &lp));
  }

  void evaluate(unsigned what, bool forces) {
    WorkSpace& ws = getWSpace();
    pdgpu_plugin::check(pdgpu_set_positions(ctx, &ws.cur.atom[0].p.x, sizeof(SnapShotAtom)));
    pdgpu_energies e;
    const int st = pdgpu_compute(ctx, what, &e, forces ? &ws.cur.atom[0].f.x : 0, sizeof(SnapShotAtom));
    if (st == PDGPU_ERR_NAN) {
      ws.ene.epot = std::numeric_limits<double>::quiet_NaN();
      return;
    }
    pdgpu_plugin::check(st);
    ws.ene.epot += e.vdw + e.elec + e.pol;
    ws.ene.epot_vdw = e.vdw;
    ws.ene.epot_elec = e.elec;
    ws.ene.epot_pol += e.pol;
    ws.ene.epot_pol_self += e.pol_self;
    ws.ene.epot_pol_cross += e.pol_cross;
    epot_vdw = e.vdw;
    epot_elec = e.elec;
    epot_pol = e.pol;
    epot_pol_self = e.pol_self;
    epot_pol_cross = e.pol_cross;
    epot = e.vdw + e.elec + e.pol;
  }

  virtual void calcForces() { evaluate(PDGPU_GB, true); }
  // PD's calcEnergies (gbff.cpp:178-183): FF_NonBonded::calcEnergies with this
  // object's settings — whose kernel also adds its forces and virial
  // (nonbonded.cpp:1154-1206) — then calcBornEnergy without the exp threshold,
  // which adds the GB energy to epot only (gbff.cpp:537-596)
  virtual void calcEnergies() {
    WorkSpace& ws = getWSpace();
    pdgpu_plugin::check(pdgpu_set_positions(ctx, &ws.cur.atom[0].p.x, sizeof(SnapShotAtom)));
    pdgpu_energies en, eg;
    int st = pdgpu_compute(ctx, PDGPU_NB, &en, &ws.cur.atom[0].f.x, sizeof(SnapShotAtom));
    if (st == PDGPU_OK) st = pdgpu_compute(ctx, PDGPU_GB | PDGPU_PD_ENERGIES, &eg, 0, sizeof(SnapShotAtom));
    if (st == PDGPU_ERR_NAN) {
      ws.ene.epot = std::numeric_limits<double>::quiet_NaN();
      return;
    }
    pdgpu_plugin::check(st);
    ws.ene.epot += en.vdw + en.elec + eg.pol;
    ws.ene.epot_vdw = en.vdw;
    ws.ene.epot_elec = en.elec;
    ws.ene.InternalVirial += en.virial;
    epot_vdw = en.vdw;
    epot_elec = en.elec;
    epot_pol = eg.pol;
    epot_pol_self = eg.pol_self;
    epot_pol_cross = eg.pol_cross;
    epot = en.vdw + en.elec + eg.pol;
  }
};

// FF_SASA_LCPO on the GPU: LCPO surface area and its forces (lcpo.cpp:640-961),
// recalculated every UpdateSasa steps and reused in between (lcpo.cpp:193-206).
class FF_SASA_LCPO_GPU : public ForcefieldBase {
 public:
  FF_SASA_LCPO_GPU(WorkSpace& ws) : ForcefieldBase(ws), ListPadding(0.5), ctx(0), cached(false), cache_surf(0.0) {
    name = "LCPO SASA (GPU)";
    settodefault();
  }
  FF_SASA_LCPO_GPU(const FF_SASA_LCPO_GPU& other)
      : ForcefieldBase(other), ASPsection_name(other.ASPsection_name), GlobalASP(other.GlobalASP),
        UpdateSasa(other.UpdateSasa), ListPadding(other.ListPadding), ctx(0), cached(false), cache_surf(0.0) {}
  virtual FF_SASA_LCPO_GPU* clone() const { return new FF_SASA_LCPO_GPU(*this); }
  virtual ~FF_SASA_LCPO_GPU() {
    if (ctx) pdgpu_destroy(ctx);
  }

  // FF_SASA_LCPO's public attributes and defaults (lcpo.h:61-72)
  std::string ASPsection_name;
  double GlobalASP;
  int UpdateSasa;
  double ListPadding;  // skin of the device list (A)

  virtual void settodefault() {
    ASPsection_name = "";
    GlobalASP = 0.0;
    UpdateSasa = 5;
  }

 protected:
  struct SasaType {
    int attype, neighbors;
    double radius, P[4], sigma;
  };
  pdgpu_ctx* ctx;
  std::vector<double> radius, P, sigma;  // per atom: radius + 1.4, P1..P4, sigma (PD's units)
  std::vector<int> use;
  std::vector<double> cache_f, sasa;     // forces (N) and per-atom SASA of the last recalculation
  bool cached;
  double cache_surf;

  // the LCPOSASAPARAMETERS section: LCPOSASATYPE <atom type> <heavy neighbours
  // or -1> <radius> <P1> <P2> <P3> <P4> (lcpo.cpp:310-390)
  void read_types(std::vector<SasaType>& types) {
    WorkSpace& ws = getWSpace();
    Section section;
    if (ws.ffps().getSection("LCPOSASAPARAMETERS", section) != 0)
      throw ProcedureException("Error reading Solvation parameters");
    for (size_t l = 0; l < section.sectionline.size(); l++) {
      std::string line = section.sectionline[l];
      removecomments(line, "#\12\15");
      std::vector<std::string> tok = chopstr(line, " \12\15\t");
      if (tok.empty()) continue;
      SasaType t;
      if (!cmpstring(tok[0], "LCPOSASATYPE") || tok.size() < 8 || (t.attype = ws.ffps().findAtomType(tok[1])) < 0 ||
          str2int(tok[2], t.neighbors) != 0 || str2double(tok[3], t.radius) != 0 || str2double(tok[4], t.P[0]) != 0 ||
          str2double(tok[5], t.P[1]) != 0 || str2double(tok[6], t.P[2]) != 0 || str2double(tok[7], t.P[3]) != 0)
        throw ProcedureException("Error reading Solvation parameters");
      t.sigma = 0.0;
      types.push_back(t);
    }
  }

  // an ASP section: SOLVATIONTYPE <atom type> <value>, sigma = value kcal2J Na as
  // PD reads it (lcpo.cpp:224-305)
  void read_asp(std::vector<SasaType>& types) {
    WorkSpace& ws = getWSpace();
    Section section;
    if (ws.ffps().getSection(ASPsection_name, section) != 0)
      throw ProcedureException("Error reading Solvation parameters");
    for (size_t l = 0; l < section.sectionline.size(); l++) {
      std::string line = section.sectionline[l];
      removecomments(line, "#\12\15");
      std::vector<std::string> tok = chopstr(line, " \12\15\t");
      if (tok.empty()) continue;
      int attype;
      double value;
      if (!cmpstring(tok[0], "SOLVATIONTYPE") || tok.size() < 3 || (attype = ws.ffps().findAtomType(tok[1])) < 0 ||
          str2double(tok[2], value) != 0)
        throw ProcedureException("Error reading Solvation parameters");
      bool found = false;
      for (size_t j = 0; j < types.size(); j++)
        if (types[j].attype == attype) {
          types[j].sigma = value * PhysicsConst::kcal2J * PhysicsConst::Na;
          found = true;
        }
      if (!found) throw ProcedureException("Error reading Solvation parameters");
    }
  }

  virtual void setup() {
    WorkSpace& ws = getWSpace();
    ws.nlist().requestCutoff(7.0);  // as FF_SASA_LCPO::setup (lcpo.cpp:37)
    std::vector<SasaType> types;
    read_types(types);
    if (!cmpstring(ASPsection_name, "")) read_asp(types);
    else
      for (size_t j = 0; j < types.size(); j++) types[j].sigma = GlobalASP / PhysicsConst::Na / PhysicsConst::J2kcal;
    const int n = ws.nAtoms();
    radius.assign(n, 0.0);
    P.assign(4 * (size_t)n, 0.0);
    sigma.assign(n, 0.0);
    use.assign(n, 0);
    for (int i = 0; i < n; i++) {
      // the first type of the atom's force-field type whose heavy-neighbour count
      // matches (or is -1) (lcpo.cpp:67-106)
      int heavy = 0;
      for (size_t j = 0; j < ws.atom[i].cov12atom.size(); j++)
        if (ws.atom[ws.atom[i].cov12atom[j].i].Z != 1) heavy++;
      size_t j = 0;
      for (; j < types.size(); j++)
        if (types[j].attype == ws.atom[i].FFType && (types[j].neighbors < 0 || types[j].neighbors == heavy)) break;
      if (j >= types.size()) throw ProcedureException("Error reading Solvation parameters");
      radius[i] = types[j].radius + 1.4;
      for (int c = 0; c < 4; c++) P[4 * (size_t)i + c] = types[j].P[c];
      sigma[i] = types[j].sigma;
      use[i] = ws.atom[i].Z == 1 ? 0 : 1;
    }
    pdgpu_plugin::SystemArrays a;
    a.gather(ws);
    pdgpu_system_desc d = pdgpu_system_desc();
    a.fill(d);
    d.lcpo_radius = &radius[0];
    d.lcpo_p = &P[0];
    d.lcpo_sigma = &sigma[0];
    d.lcpo_use = &use[0];
    if (ctx) pdgpu_destroy(ctx);
    int st = PDGPU_OK;
    ctx = pdgpu_create(0, &d, &st);
    if (!ctx) pdgpu_plugin::check(st);
    const pdgpu_list_params lp = pdgpu_plugin::list_params(ListPadding);
    pdgpu_plugin::check(pdgpu_set_list_params(ctx, &lp));
    cached = false;
  }

  // a full recalculation into the cache (forces in N, energy in J, per-atom SASA)
  void recalc(bool forces) {
    WorkSpace& ws = getWSpace();
    const int n = ws.nAtoms();
    pdgpu_plugin::check(pdgpu_set_positions(ctx, &ws.cur.atom[0].p.x, sizeof(SnapShotAtom)));
    pdgpu_energies e;
    cache_f.assign(3 * (size_t)n, 0.0);
    pdgpu_plugin::check(pdgpu_compute(ctx, PDGPU_SA, &e, forces ? &cache_f[0] : 0, 24));
    sasa.assign(n, 0.0);
    pdgpu_plugin::check(pdgpu_get_sasa(ctx, &sasa[0]));
    cache_surf = e.surf;
    cached = forces;
  }

  void distribute(bool forces) {
    WorkSpace& ws = getWSpace();
    const int n = ws.nAtoms();
    for (int i = 0; i < n; i++) {
      ws.atom[i].epot += sasa[i] * sigma[i];
      if (forces) {
        ws.cur.atom[i].f.x += cache_f[3 * (size_t)i];
        ws.cur.atom[i].f.y += cache_f[3 * (size_t)i + 1];
        ws.cur.atom[i].f.z += cache_f[3 * (size_t)i + 2];
      }
    }
    ws.ene.epot += cache_surf;
    ws.ene.epot_surf += cache_surf;
    epot = cache_surf;
  }

  virtual void calcForces() {
    if (!cached || getWSpace().Step % UpdateSasa == 0) recalc(true);
    distribute(true);
  }
  virtual void calcEnergies() {
    recalc(false);
    distribute(false);
  }
};

}  // namespace Physics

#endif
