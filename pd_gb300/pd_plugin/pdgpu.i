// SWIG interface of the PD components in ff_gpu.h (src/mods/pdgpu/pdgpu.i in a
// PD tree), following PD's module pattern (src/mods/example/example.i): the
// components take PD's WorkSpace and join a Forcefield with ff.add(...).
%module pdgpu
%{
#include "ff_gpu.h"
%}
%import "pd.i"
%include "ff_gpu.h"
