"""ctypes binding to libpdgpu.so (include/pdgpu.h).

The library is built in-tree (pd_gb300/_build/libpdgpu.so) by pd_gb300.build.
There is no fallback: if the library cannot be loaded, every entry point raises.
"""
import ctypes
import os

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

OK = 0
ERRORS = {
    -1: "invalid argument", -2: "CUDA runtime error", -3: "LCPO overlap list or tile list overflow",
    -4: "fixed-point accumulator overflow", -5: "NaN energy or force", -6: "device wait timed out",
    -7: "unsupported option", -8: "stale neighbour list", -9: "call sequence error",
    -10: "beyond what the allocation-free entry point holds (static scratch or list arrays)",
}
ERR_STALE_LIST = -8
ERR_CAPACITY = -10
NB, GB, SA, BONDED, ENERGY, PD_ENERGIES = 1, 2, 4, 8, 0x100, 0x200


class PDGPUError(RuntimeError):
    """Raised for a non-zero pdgpu status (PD raises ProcedureException / RuntimeError)."""

    def __init__(self, status, where=""):
        self.status = status
        super().__init__("%s: pdgpu status %d (%s)" % (where, status, ERRORS.get(status, "unknown")))


class Energies(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("epot", "vdw", "elec", "pol", "pol_self", "pol_cross", "surf",
                                                "virial", "bond", "angle", "torsion", "improper")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SystemDesc(ctypes.Structure):
    _fields_ = [("nsystems", ctypes.c_int), ("natoms", _ip), ("box", _dp), ("charge", _dp), ("radius", _dp),
                ("epsilon", _dp), ("mass", _dp), ("gb_radius", _dp), ("gb_vj", _dp), ("gb_terms123", _dp),
                ("lcpo_radius", _dp), ("lcpo_p", _dp), ("lcpo_sigma", _dp), ("lcpo_use", _ip),
                ("nexcl", ctypes.c_int), ("excl", _ip),
                ("nbond", ctypes.c_int), ("bond_idx", _ip), ("bond_par", _dp),
                ("nangle", ctypes.c_int), ("angle_idx", _ip), ("angle_par", _dp),
                ("ntors", ctypes.c_int), ("tors_idx", _ip), ("tors_par", _dp),
                ("nimpr", ctypes.c_int), ("impr_idx", _ip), ("impr_par", _dp)]


class NBParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("Cutoff", "InnerCutoff", "VdwCutoff", "VdwInnerCutoff",
                                                "Vdw14Scaling", "Elec14Scaling", "Dielectric")] + \
               [(k, ctypes.c_int) for k in ("EnergySwitch", "ForceSwitch", "DoVdw", "DoElec")]


class GBParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "Cutoff", "InnerCutoff", "VdwCutoff", "VdwInnerCutoff", "Vdw14Scaling", "Elec14Scaling",
        "DielectricSolute", "DielectricSolvent", "GbsaStillCutoff", "ExpApproxThreshold", "BornRadiusOffset",
        "P4", "P5")]


class ListParams(ctypes.Structure):
    _fields_ = [("Padding", ctypes.c_double), ("check_skin", ctypes.c_int)]


class MDParams(ctypes.Structure):
    _fields_ = [("Integrator", ctypes.c_int), ("Timestep", ctypes.c_double), ("FricCoeff", ctypes.c_double),
                ("UpdateNList", ctypes.c_int), ("UpdateSasa", ctypes.c_int), ("what", ctypes.c_uint),
                ("seed", ctypes.c_ulonglong), ("use_graph", ctypes.c_int)]


class ParamGrads(ctypes.Structure):
    """pdgpu_param_grads: host (pdgpu_param_grad) or device (…_device) pointers, NULL = skip."""
    _fields_ = [(n, ctypes.c_void_p) for n in ("charge", "radius", "epsilon", "gb_radius", "gb_vj", "gb_terms123")]


# every symbol include/pdgpu.h declares, with its ctypes signature
SIGNATURES = {
    "pdgpu_create": ([ctypes.c_int, ctypes.POINTER(SystemDesc), _ip], ctypes.c_void_p),
    "pdgpu_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "pdgpu_error_string": ([ctypes.c_int], ctypes.c_char_p),
    "pdgpu_set_nb_params": ([ctypes.c_void_p, ctypes.POINTER(NBParams)], ctypes.c_int),
    "pdgpu_set_gb_params": ([ctypes.c_void_p, ctypes.POINTER(GBParams)], ctypes.c_int),
    "pdgpu_set_list_params": ([ctypes.c_void_p, ctypes.POINTER(ListParams)], ctypes.c_int),
    "pdgpu_set_gb_mode": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(NBParams)], ctypes.c_int),
    "pdgpu_update_params": ([ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    "pdgpu_update_params_device": ([ctypes.c_void_p] + [ctypes.c_void_p] * 6, ctypes.c_int),
    "pdgpu_nb_energy_full": ([ctypes.c_void_p, ctypes.POINTER(Energies)], ctypes.c_int),
    "pdgpu_nb_energy_update": ([ctypes.c_void_p, ctypes.POINTER(Energies), _ip], ctypes.c_int),
    "pdgpu_param_grad": ([ctypes.c_void_p, ctypes.c_uint, ctypes.POINTER(Energies), ctypes.POINTER(ParamGrads)],
                         ctypes.c_int),
    "pdgpu_param_grad_device": ([ctypes.c_void_p, ctypes.c_uint, ctypes.POINTER(ParamGrads)], ctypes.c_int),
    "pdgpu_param_grad_device_noalloc": ([ctypes.c_void_p, ctypes.c_uint, ctypes.POINTER(ParamGrads)], ctypes.c_int),
    "pdgpu_set_positions": ([ctypes.c_void_p, _dp, ctypes.c_size_t], ctypes.c_int),
    "pdgpu_set_positions_device": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pdgpu_get_positions": ([ctypes.c_void_p, _dp, ctypes.c_size_t], ctypes.c_int),
    "pdgpu_set_positions_async": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "pdgpu_get_positions_async": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "pdgpu_rebuild_list": ([ctypes.c_void_p], ctypes.c_int),
    "pdgpu_compute": ([ctypes.c_void_p, ctypes.c_uint, ctypes.POINTER(Energies), _dp, ctypes.c_size_t],
                      ctypes.c_int),
    "pdgpu_compute_device": ([ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p], ctypes.c_int),
    "pdgpu_get_energies": ([ctypes.c_void_p, ctypes.POINTER(Energies)], ctypes.c_int),
    "pdgpu_get_born_radii": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "pdgpu_get_sasa": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "pdgpu_list_stats": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                          ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "pdgpu_list_tiles": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_longlong,
                          ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                          ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "pdgpu_list_slots": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "pdgpu_stream": ([ctypes.c_void_p], ctypes.c_void_p),
    "pdgpu_md_setup": ([ctypes.c_void_p, ctypes.POINTER(MDParams), _dp], ctypes.c_int),
    "pdgpu_set_velocities": ([ctypes.c_void_p, _dp, ctypes.c_size_t], ctypes.c_int),
    "pdgpu_get_velocities": ([ctypes.c_void_p, _dp, ctypes.c_size_t], ctypes.c_int),
    "pdgpu_md_run": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "pdgpu_get_kinetic": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "pdgpu_get_kinetic_async": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "pdgpu_remd_exchange": ([ctypes.c_void_p, ctypes.c_int, _ip, _dp], ctypes.c_int),
    "pdgpu_md_autotune": ([ctypes.c_void_p, ctypes.c_int, _ip, _ip], ctypes.c_int),
    "pdgpu_remd_set_modes": ([ctypes.c_void_p, _ip], ctypes.c_int),
    "pdgpu_md_checkpoint": ([ctypes.c_void_p], ctypes.c_int),
    "pdgpu_md_set_trajectory": ([ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int], ctypes.c_int),
    "pdgpu_md_trajectory_frames": ([ctypes.c_void_p], ctypes.c_longlong),
    "pdgpu_md_rescue": ([ctypes.c_void_p, ctypes.c_ulonglong, _ip, _ip], ctypes.c_int),
    "pdgpu_set_launch_shape": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "pdgpu_get_launch_shape": ([ctypes.c_void_p, _ip], ctypes.c_int),
    "pdgpu_set_work_items": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "pdgpu_get_work_items": ([ctypes.c_void_p, _ip], ctypes.c_int),
    "pdgpu_set_nb_groups": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "pdgpu_get_nb_groups": ([ctypes.c_void_p, _ip, ctypes.POINTER(ctypes.c_longlong),
                             ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "pdgpu_md_enqueue": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "pdgpu_synchronize": ([ctypes.c_void_p], ctypes.c_int),
    "pdgpu_kernel_launches": ([ctypes.c_void_p], ctypes.c_longlong),
    "pdgpu_time_kernel": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp], ctypes.c_int),
    "pdgpu_pair_census": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "pdgpu_fp32_peak": ([ctypes.c_int, _dp, _dp], ctypes.c_int),
    "pdgpu_device_allocations": ([ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
                                 ctypes.c_int),
    "pdgpu_host_alloc": ([ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "pdgpu_host_free": ([ctypes.c_void_p], ctypes.c_int),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libpdgpu.so (building it first if allowed).  Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libpdgpu.so is not built (%s); run pd_gb300.build.build()" % path)
        _build.build()
    try:
        L = ctypes.CDLL(path)
    except OSError:
        if not build_if_missing:
            raise
        # a library built for another machine (e.g. another CPU architecture): rebuild here
        _build.build(force=True)
        L = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def fp32_peak(device=0):
    """Measured FP32 FMA throughput (TFLOP/s, FFMA and packed FFMA2; pdgpu_fp32_peak)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    check(load().pdgpu_fp32_peak(int(device), ctypes.byref(a), ctypes.byref(b)), "pdgpu_fp32_peak")
    return {"ffma_tflops": a.value, "ffma2_tflops": b.value}


def device_allocations():
    """(cudaMalloc calls the library made so far, device bytes it holds now)."""
    n, b = ctypes.c_longlong(), ctypes.c_longlong()
    check(load().pdgpu_device_allocations(ctypes.byref(n), ctypes.byref(b)), "pdgpu_device_allocations")
    return n.value, b.value


def host_array(shape):
    """A float64 numpy array in page-locked host memory from pdgpu_host_alloc
    (ordinary memory when the runtime cannot provide it).  The memory is freed
    by pdgpu_host_free once the array and every view of it are gone."""
    import weakref

    import numpy as np
    count = int(np.prod(shape))
    L = load()
    ptr = ctypes.c_void_p()
    if L.pdgpu_host_alloc(8 * count, ctypes.byref(ptr)) != OK:
        return np.zeros(shape)
    buf = (ctypes.c_double * count).from_address(ptr.value)
    weakref.finalize(buf, L.pdgpu_host_free, ctypes.c_void_p(ptr.value))
    arr = np.frombuffer(buf, dtype=np.float64).reshape(shape)   # keeps buf (and the memory) alive
    arr[...] = 0.0
    return arr


def check(status, where):
    if status != OK:
        raise PDGPUError(status, where)
    return status
