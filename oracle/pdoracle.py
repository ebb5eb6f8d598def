"""ctypes binding to the FP64 C restatement in ``oracle/pdoracle.c``.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg as the checker.  The product never imports
this module.  Units are PD's (Angstrom, J, N, sqrt(J) epsilons).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_build", "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class System(ctypes.Structure):
    _fields_ = [("natom", ctypes.c_int), ("pos", _dp), ("charge", _dp), ("radius", _dp), ("epsilon", _dp),
                ("nexcl", ctypes.c_int), ("excl", _ip), ("box", ctypes.c_double * 3)]


class NBParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("Cutoff", "InnerCutoff", "VdwCutoff", "VdwInnerCutoff",
                                                "Vdw14Scaling", "Elec14Scaling", "Dielectric")] + \
               [(k, ctypes.c_int) for k in ("EnergySwitch", "ForceSwitch", "DoVdw", "DoElec", "VdwCor")] + \
               [(k, ctypes.c_double) for k in ("VdwCorDensity", "VdwCorEpsilon", "VdwCorRadius", "VdwCorCutoff",
                                                "ListCutoff")]


class GBParams(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "Cutoff", "InnerCutoff", "VdwCutoff", "VdwInnerCutoff", "Vdw14Scaling", "Elec14Scaling",
        "DielectricSolute", "DielectricSolvent", "GbsaStillCutoff", "ExpApproxThreshold", "DielectricOffset",
        "BornRadiusOffset", "P1", "P2", "P3", "P4", "P5", "ListCutoff")] + [("FastMode", ctypes.c_int)]


class NList(ctypes.Structure):
    _fields_ = [("natom", ctypes.c_int), ("start", ctypes.c_void_p), ("j", ctypes.c_void_p),
                ("shift", ctypes.c_void_p)]


class Energies(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("epot", "vdw", "elec", "pol", "pol_self", "pol_cross", "surf",
                                                "virial")]

    def as_array(self):
        return np.array([self.epot, self.vdw, self.elec, self.pol, self.pol_self, self.pol_cross, self.surf,
                         self.virial])


_lib = None


def build():
    """Compile liboracle.so from oracle/pdoracle.c (gcc, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        try:
            L = ctypes.CDLL(LIB_PATH)
        except OSError:
            # built for another CPU architecture: rebuild from source here
            os.remove(LIB_PATH)
            build()
            L = ctypes.CDLL(LIB_PATH)
        L.pdo_nonbonded.argtypes = [ctypes.POINTER(System), ctypes.POINTER(NBParams), ctypes.c_int,
                                    ctypes.POINTER(Energies), _dp]
        L.pdo_list_checksums.argtypes = [ctypes.POINTER(System), ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]
        L.pdo_pair_law.argtypes = [ctypes.POINTER(NBParams)] + [ctypes.c_double] * 5 + [_dp] * 4
        L.pdo_gb_fixed_terms.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _dp, ctypes.c_int, _ip, _dp,
                                         ctypes.POINTER(GBParams), _dp, _dp]
        L.pdo_gb_born_radii.argtypes = [ctypes.POINTER(System), ctypes.POINTER(GBParams), _dp, _dp, _dp,
                                        ctypes.c_int, _dp]
        L.pdo_gb_forces.argtypes = [ctypes.POINTER(System), ctypes.POINTER(GBParams), _dp, _dp, _dp, ctypes.c_int,
                                    ctypes.POINTER(Energies), _dp, _dp]
        L.pdo_lcpo_forces.argtypes = [ctypes.POINTER(System), ctypes.c_double, _dp, _dp, _dp, _ip, ctypes.c_int,
                                      ctypes.POINTER(Energies), _dp, _dp]
        L.pdo_vv_step.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_double]
        L.pdo_vv_step.restype = ctypes.c_double
        L.pdo_langevin_step.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, _dp, ctypes.c_int, ctypes.c_int]
        L.pdo_langevin_step.restype = ctypes.c_double
        L.pdo_langevin_coeffs.argtypes = [ctypes.c_double, ctypes.c_double, _dp]
        L.pdo_bonded.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _dp, ctypes.c_int, _ip, _dp, ctypes.c_int,
                                 _ip, _dp, ctypes.c_int, _ip, _dp, _dp, _dp]
        L.pdo_list_build.argtypes = [ctypes.POINTER(System), ctypes.c_double, ctypes.c_int, ctypes.POINTER(NList)]
        L.pdo_list_free.argtypes = [ctypes.POINTER(NList)]
        L.pdo_nonbonded_list.argtypes = [ctypes.POINTER(System), ctypes.POINTER(NList), ctypes.POINTER(NBParams),
                                         ctypes.c_int, ctypes.POINTER(Energies), _dp]
        L.pdo_econv_joule.restype = ctypes.c_double
        L.pdo_halfeconv.restype = ctypes.c_double
        _lib = L
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _pd(a):
    return a.ctypes.data_as(_dp)


def _pi(a):
    return a.ctypes.data_as(_ip)


class OracleSystem:
    """Keeps the numpy buffers alive for the ctypes System record."""

    def __init__(self, pos, charge, radius, epsilon, excl, box=(0.0, 0.0, 0.0)):
        self.pos = _d(pos).reshape(-1, 3)
        self.charge = _d(charge)
        self.radius = _d(radius)
        self.epsilon = _d(epsilon)
        self.excl = _i(excl).reshape(-1, 3)
        self.rec = System(len(self.pos), _pd(self.pos), _pd(self.charge), _pd(self.radius), _pd(self.epsilon),
                          len(self.excl), _pi(self.excl), (ctypes.c_double * 3)(*box))

    @property
    def natom(self):
        return len(self.pos)


def nb_params(**kw):
    d = dict(Cutoff=12.0, InnerCutoff=10.0, VdwCutoff=None, VdwInnerCutoff=None, Vdw14Scaling=1.0,
             Elec14Scaling=1.0, Dielectric=1.0, EnergySwitch=1, ForceSwitch=0, DoVdw=1, DoElec=1, VdwCor=0,
             VdwCorDensity=0.0, VdwCorEpsilon=0.0, VdwCorRadius=0.0, VdwCorCutoff=0.0, ListCutoff=None)
    d.update(kw)
    if d["VdwCutoff"] is None:
        d["VdwCutoff"] = d["Cutoff"]
    if d["VdwInnerCutoff"] is None:
        d["VdwInnerCutoff"] = d["InnerCutoff"]
    if d["ListCutoff"] is None:
        d["ListCutoff"] = max(d["Cutoff"], d["VdwCutoff"]) + 2.0
    return NBParams(**{k: d[k] for k, _ in NBParams._fields_})


def gb_params(**kw):
    d = dict(Cutoff=12.0, InnerCutoff=9.0, VdwCutoff=None, VdwInnerCutoff=None, Vdw14Scaling=0.5,
             Elec14Scaling=0.83333, DielectricSolute=1.0, DielectricSolvent=80.0, GbsaStillCutoff=10.0,
             ExpApproxThreshold=-4.0, DielectricOffset=-0.09, BornRadiusOffset=0.0, P1=0.073, P2=0.921,
             P3=6.211, P4=15.236, P5=1.254, ListCutoff=None, FastMode=1)
    d.update(kw)
    if d["VdwCutoff"] is None:
        d["VdwCutoff"] = d["Cutoff"]
    if d["VdwInnerCutoff"] is None:
        d["VdwInnerCutoff"] = d["InnerCutoff"]
    if d["ListCutoff"] is None:
        d["ListCutoff"] = max(d["Cutoff"], d["VdwCutoff"]) + 2.0
    return GBParams(**{k: d[k] for k, _ in GBParams._fields_})


def nonbonded(sys_, params, nthreads=1):
    e = Energies()
    f = np.zeros((sys_.natom, 3))
    lib().pdo_nonbonded(ctypes.byref(sys_.rec), ctypes.byref(params), nthreads, ctypes.byref(e), _pd(f))
    return e.as_array(), f


class StoredList:
    """A PD-style half list kept between rebuilds (freed with the object)."""

    def __init__(self, sys_, list_cutoff, nthreads=1):
        self.rec = NList()
        lib().pdo_list_build(ctypes.byref(sys_.rec), list_cutoff, nthreads, ctypes.byref(self.rec))

    def __del__(self):
        try:
            lib().pdo_list_free(ctypes.byref(self.rec))
        except Exception:
            pass


def nonbonded_list(sys_, nlist, params, nthreads=1):
    e = Energies()
    f = np.zeros((sys_.natom, 3))
    lib().pdo_nonbonded_list(ctypes.byref(sys_.rec), ctypes.byref(nlist.rec), ctypes.byref(params), nthreads,
                             ctypes.byref(e), _pd(f))
    return e.as_array(), f


def list_checksums(sys_, list_cutoff):
    n = sys_.natom
    c = np.zeros(n, np.int32)
    s1 = np.zeros(n, np.int64)
    s2 = np.zeros(n, np.int64)
    lib().pdo_list_checksums(ctypes.byref(sys_.rec), list_cutoff, c.ctypes.data, s1.ctypes.data, s2.ctypes.data)
    return c, s1, s2


def pair_law(params, r, radiusij, epsilon, qi, qj):
    out = [ctypes.c_double() for _ in range(4)]
    lib().pdo_pair_law(ctypes.byref(params), r, radiusij, epsilon, qi, qj, *[ctypes.byref(o) for o in out])
    return [o.value for o in out]


def gb_fixed_terms(gb_radius, cov12, d12, cov13, d13, params):
    n = len(gb_radius)
    R = _d(gb_radius)
    c12, c13 = _i(cov12).reshape(-1, 2), _i(cov13).reshape(-1, 2)
    e12, e13 = _d(d12), _d(d13)
    vj = np.zeros(n)
    t = np.zeros(n)
    lib().pdo_gb_fixed_terms(n, _pd(R), len(c12), _pi(c12), _pd(e12), len(c13), _pi(c13), _pd(e13),
                             ctypes.byref(params), _pd(vj), _pd(t))
    return vj, t


def gb_born_radii(sys_, params, gb_radius, vj, terms123, nthreads=1):
    born = np.zeros(sys_.natom)
    R, V, T = _d(gb_radius), _d(vj), _d(terms123)
    lib().pdo_gb_born_radii(ctypes.byref(sys_.rec), ctypes.byref(params), _pd(R), _pd(V), _pd(T), nthreads,
                            _pd(born))
    return born


def gb_forces(sys_, params, gb_radius, vj, terms123, nthreads=1):
    e = Energies()
    f = np.zeros((sys_.natom, 3))
    born = np.zeros(sys_.natom)
    R, V, T = _d(gb_radius), _d(vj), _d(terms123)
    lib().pdo_gb_forces(ctypes.byref(sys_.rec), ctypes.byref(params), _pd(R), _pd(V), _pd(T), nthreads,
                        ctypes.byref(e), _pd(f), _pd(born))
    return e.as_array(), f, born


def lcpo_forces(sys_, list_cutoff, lcpo_radius, lcpo_P, sigma, use, nthreads=1):
    e = Energies()
    f = np.zeros((sys_.natom, 3))
    sa = np.zeros(sys_.natom)
    R, P, S, U = _d(lcpo_radius), _d(lcpo_P), _d(sigma), _i(use)
    lib().pdo_lcpo_forces(ctypes.byref(sys_.rec), list_cutoff, _pd(R), _pd(P), _pd(S), _pi(U), nthreads,
                          ctypes.byref(e), _pd(f), _pd(sa))
    return e.as_array(), f, sa


def bonded(pos, bond_idx, bond_par, angle_idx, angle_par, tors_idx, tors_par, impr_idx, impr_par):
    pos = _d(pos)
    n = len(pos)
    f = np.zeros((n, 3))
    ene = np.zeros(4)
    arrs = [(_i(bond_idx), _d(bond_par)), (_i(angle_idx), _d(angle_par)), (_i(tors_idx), _d(tors_par)),
            (_i(impr_idx), _d(impr_par))]
    args = []
    for idx, par in arrs:
        args += [len(idx), _pi(idx), _pd(par)]
    lib().pdo_bonded(n, _pd(pos), *args, _pd(ene), _pd(f))
    return ene, f


def langevin_coeffs(gamma, dt):
    out = np.zeros(6)
    lib().pdo_langevin_coeffs(gamma, dt, _pd(out))
    return out


def vv_step(pos, vel, force, mass, dt):
    pos, vel = _d(pos).copy(), _d(vel).copy()
    ek = lib().pdo_vv_step(len(mass), _pd(pos), _pd(vel), _pd(_d(force)), _pd(_d(mass)), dt)
    return pos, vel, ek


def langevin_step(pos, vel, force, mass, dt, gamma, T, noise, first_step=False, last_step=False):
    pos, vel = _d(pos).copy(), _d(vel).copy()
    nz = _d(noise)
    ek = lib().pdo_langevin_step(len(mass), _pd(pos), _pd(vel), _pd(_d(force)), _pd(_d(mass)), dt, gamma, T,
                                 _pd(nz), int(first_step), int(last_step))
    return pos, vel, ek
