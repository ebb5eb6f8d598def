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
// FF_SASA_LCPO keeps its per-atom LCPO parameters private (lcpo.h:119-122);
// a GPU LCPO component needs them protected (a one-line change in lcpo.h) and
// then passes SASAatom[i].{radius, P1..P4, sigma} the same way.
#ifndef PDGPU_PD_PLUGIN_FF_GPU_H
#define PDGPU_PD_PLUGIN_FF_GPU_H

#include <limits>
#include <vector>

#include "forcefields/gbff.h"
#include "forcefields/nonbonded.h"
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
    // PD overwrites epot_vdw / epot_elec and adds to epot (nonbonded.cpp:681-682, 905)
    ws.ene.epot += e.vdw + e.elec;
    ws.ene.epot_vdw = e.vdw;
    ws.ene.epot_elec = e.elec;
    ws.ene.InternalVirial += e.virial;
    epot_vdw = e.vdw;
    epot_elec = e.elec;
    epot = e.vdw + e.elec;
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
  // PD's calcEnergies: calcBornEnergy without the exp threshold plus FF_NonBonded's
  // energies with this object's settings (gbff.cpp:178-183)
  virtual void calcEnergies() { evaluate(PDGPU_GB | PDGPU_PD_ENERGIES, false); }
};

}  // namespace Physics

#endif
