"""pd_gb300 — GB300-native nonbonded / Generalised-Born / LCPO path for PD.

The compute path is libpdgpu.so (hand-written CUDA for sm_103a behind the C ABI
in include/pdgpu.h).  This package holds its build step, its ctypes binding and
a Python mirror of PD's forcefield interface (WorkSpace, Forcefield, FF_*).
"""
from .ffi import PDGPUError  # noqa: F401
from .forcefield import (FF_Bonded_GPU, FF_GeneralizedBorn_Still_GPU, FF_NonBonded_GPU,  # noqa: F401
                         FF_SASA_LCPO_GPU, Forcefield, ForcefieldBase)
from .workspace import Hamiltonian, SystemImage, WorkSpace, load_workload  # noqa: F401

__all__ = ["FF_Bonded_GPU", "FF_GeneralizedBorn_Still_GPU", "FF_NonBonded_GPU", "FF_SASA_LCPO_GPU", "Forcefield",
           "ForcefieldBase", "Hamiltonian", "SystemImage", "WorkSpace", "load_workload", "PDGPUError"]
