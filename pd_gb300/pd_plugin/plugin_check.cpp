// Link check of the PD components in ff_gpu.h: built against PD's headers and
// libmmlib.a (the oracle's out-of-tree build of the PD sources) and libpdgpu,
// so every PD virtual the components override or call, and every C ABI entry
// point they use, must resolve.  The program only reports that it linked; it
// creates no WorkSpace and touches no GPU.
#include <cstdio>

#include "ff_gpu.h"

// referenced (never called) so the components' vtables and bodies are emitted
Physics::ForcefieldBase* pdgpu_plugin_components(WorkSpace& ws, int which) {
  if (which == 0) return new Physics::FF_NonBonded_GPU(ws);
  return new Physics::FF_GeneralizedBorn_Still_GPU(ws);
}

int main(int argc, char**) {
  if (argc > 99) return pdgpu_plugin_components(*(WorkSpace*)0, argc) != 0;
  std::printf("pdgpu PD components linked\n");
  return 0;
}
