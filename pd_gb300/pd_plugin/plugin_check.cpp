// The PD components of ff_gpu.h run inside PD against PD's own components on
// one WorkSpace (test program; built by `make -C oracle plugin-check`).
//
// A peptide built by PD (NewProtein, PD's parameter files) is evaluated by two
// Forcefield containers (forcefield.cpp:237-264): PD's FF_Bonded +
// FF_GeneralizedBorn_Still + FF_SASA_LCPO, and FF_Bonded + the GPU components;
// then FF_Bonded + FF_NonBonded (with VdwCor) against FF_Bonded +
// FF_NonBonded_GPU.  Every Hamiltonian field the components write and every
// atom's force must agree, for calcForces and calcEnergies.  Linked against
// the oracle-backed test double of the C ABI (oracle/pdgpu_abi_double.c) it
// checks the components' marshalling on a machine without a GPU; linked
// against libpdgpu it runs the same comparison on the GPU.
//
// Usage: plugin_check [sequence]   (exit 0 when everything agrees)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ff_gpu.h"
#include "forcefields/ffbonded.h"
#include "forcefields/forcefield.h"
#include "forcefields/lcpo.h"
#include "system/genpolymer.h"
#include "system/system.h"

using namespace Physics;

namespace {

struct Result {
  std::vector<double> ene;  // epot, vdw, elec, pol, pol_self, pol_cross, surf, virial, vdw_att
  std::vector<double> f;    // forces, N
};

Result evaluate(Forcefield& ff, WorkSpace& ws, bool forces) {
  ff.setup();   // every component, in add order (forcefield.cpp:179-186)
  ws.nlist().calcNewList();
  if (forces) ff.calcForces();
  else ff.calcEnergies();
  Result r;
  const Hamiltonian& e = ws.ene;
  const double v[9] = {e.epot, e.epot_vdw, e.epot_elec, e.epot_pol, e.epot_pol_self, e.epot_pol_cross,
                       e.epot_surf, e.InternalVirial, e.epot_vdw_att};
  r.ene.assign(v, v + 9);
  for (size_t i = 0; i < ws.nAtoms(); i++) {
    r.f.push_back(ws.cur.atom[i].f.x);
    r.f.push_back(ws.cur.atom[i].f.y);
    r.f.push_back(ws.cur.atom[i].f.z);
  }
  return r;
}

int compare(const char* what, const Result& pd, const Result& gpu, double etol, double ftol) {
  static const char* names[9] = {"epot", "vdw", "elec", "pol", "pol_self", "pol_cross", "surf", "virial", "vdw_att"};
  int bad = 0;
  for (int k = 0; k < 9; k++) {
    const double a = pd.ene[k], b = gpu.ene[k];
    const double err = std::fabs(a - b) / std::max(std::fabs(a), 1e-30);
    const bool ok = (a == 0.0 && b == 0.0) || err <= etol;
    if (!ok) {
      std::printf("  %s %s: PD %.12e  GPU component %.12e  (rel %.2e)\n", what, names[k], a, b, err);
      bad++;
    }
  }
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < pd.f.size(); i++) {
    num += (gpu.f[i] - pd.f[i]) * (gpu.f[i] - pd.f[i]);
    den += pd.f[i] * pd.f[i];
  }
  const double rms = den > 0 ? std::sqrt(num / den) : std::sqrt(num);
  if (rms > ftol) {
    std::printf("  %s forces: relative RMS %.2e\n", what, rms);
    bad++;
  }
  std::printf("%s: %s (force rel RMS %.2e)\n", what, bad ? "MISMATCH" : "agree", rms);
  return bad;
}

std::string sequence_string(const std::string& s) {
  return "*" + s.substr(0, 1) + "-(" + s.substr(1, s.size() - 2) + ")-" + s.substr(s.size() - 1) + "*";
}

}  // namespace

int main(int argc, char** argv) {
  // tolerances: 1e-9 with the FP64 test double; the GPU's FP32 pair math with
  // 64-bit fixed-point sums meets 1e-6 (energies) and 1e-5 (forces)
  const double etol = argc > 2 ? std::atof(argv[2]) : 1e-9, ftol = argc > 3 ? std::atof(argv[3]) : 1e-9;
  const std::string seq = argc > 1 ? argv[1] : "MKTAYIAKQRQISFVKSHFSRQLEERLGLIEVQG";
  FFParamSet ffps;
  ffps.readLib("amber99aa.ff");
  Molecule m = NewProtein(ffps, sequence_string(seq));
  System sim(ffps);
  sim.add(m);
  WorkSpace ws(sim);
  ws.nlist().setPadding(0.5);
  int bad = 0;

  // GB/SA: PD's components against the GPU ones
  {
    FF_Bonded b1(ws), b2(ws);
    FF_GeneralizedBorn_Still gb1(ws);
    FF_GeneralizedBorn_Still_GPU gb2(ws);
    FF_SASA_LCPO sa1(ws);
    FF_SASA_LCPO_GPU sa2(ws);
    FF_GeneralizedBorn_Still* gbs[2] = {&gb1, &gb2};
    for (int k = 0; k < 2; k++) {
      gbs[k]->Cutoff = 12.0;
      gbs[k]->InnerCutoff = 9.0;
      gbs[k]->VdwCutoff = 12.0;
      gbs[k]->VdwInnerCutoff = 9.0;
      gbs[k]->GbsaStillCutoff = 10.0;
    }
    gb2.ListPadding = 0.5;
    sa1.GlobalASP = sa2.GlobalASP = 0.005;
    sa1.UpdateSasa = sa2.UpdateSasa = 1;
    Forcefield pd(ws), gpu(ws);
    pd.add(b1);   // bonded first: GB's setup reads the covalent distances it sets up
    pd.add(gb1);
    pd.add(sa1);
    gpu.add(b2);
    gpu.add(gb2);
    gpu.add(sa2);
    const Result r1 = evaluate(pd, ws, true), r2 = evaluate(gpu, ws, true);
    bad += compare("GB/SA calcForces", r1, r2, etol, ftol);
    const Result e1 = evaluate(pd, ws, false), e2 = evaluate(gpu, ws, false);
    bad += compare("GB/SA calcEnergies", e1, e2, etol, ftol);
  }
  // LJ + Coulomb (force switch) with the long-range VdwCor term
  {
    FF_Bonded b1(ws), b2(ws);
    FF_NonBonded nb1(ws);
    FF_NonBonded_GPU nb2(ws);
    FF_NonBonded* nbs[2] = {&nb1, &nb2};
    for (int k = 0; k < 2; k++) {
      nbs[k]->Cutoff = 12.0;
      nbs[k]->InnerCutoff = 10.0;
      nbs[k]->VdwCutoff = 12.0;
      nbs[k]->VdwInnerCutoff = 10.0;
      nbs[k]->ForceSwitch = true;
      nbs[k]->EnergySwitch = false;
      nbs[k]->VdwCor = true;
      nbs[k]->VdwCorDensity = 0.0334;
      nbs[k]->VdwCorEpsilon = 0.152;
      nbs[k]->VdwCorRadius = 1.77;
      nbs[k]->VdwCorCutoff = 12.0;
    }
    Forcefield pd(ws), gpu(ws);
    pd.add(b1);
    pd.add(nb1);
    gpu.add(b2);
    gpu.add(nb2);
    const Result r1 = evaluate(pd, ws, true), r2 = evaluate(gpu, ws, true);
    bad += compare("NB calcForces", r1, r2, etol, ftol);
  }
  if (bad) std::printf("pdgpu PD components: %d mismatches\n", bad);
  else std::printf("pdgpu PD components match PD\n");
  return bad ? 1 : 0;
}
