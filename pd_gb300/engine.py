"""Python handle on one libpdgpu context (the C ABI in include/pdgpu.h)."""
import ctypes

import numpy as np

from . import ffi

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _pd(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _pi(a):
    return None if a is None else a.ctypes.data_as(_ip)


class DeviceContext:
    """Owns a pdgpu context for a SystemImage; every call raises PDGPUError on failure."""

    def __init__(self, image, device=0):
        self.lib = ffi.load()
        self.image = image
        im = image
        self._keep = []

        def keep(a, dtype):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dtype)
            self._keep.append(a)
            return a

        d = ffi.SystemDesc()
        d.nsystems = im.nsystems
        d.natoms = _pi(keep(im.natoms, np.int32))
        d.box = _pd(keep(im.box, np.float64))
        d.charge = _pd(keep(im.charge, np.float64))
        d.radius = _pd(keep(im.radius, np.float64))
        d.epsilon = _pd(keep(im.epsilon, np.float64))
        d.mass = _pd(keep(im.mass, np.float64))
        if im.has_gb:
            d.gb_radius = _pd(keep(im.gb_radius, np.float64))
            d.gb_vj = _pd(keep(im.gb_vj, np.float64))
            d.gb_terms123 = _pd(keep(im.gb_terms123, np.float64))
        if im.has_sa:
            d.lcpo_radius = _pd(keep(im.lcpo_radius, np.float64))
            d.lcpo_p = _pd(keep(im.lcpo_p, np.float64))
            d.lcpo_sigma = _pd(keep(im.lcpo_sigma, np.float64))
            d.lcpo_use = _pi(keep(im.lcpo_use, np.int32))
        ex = keep(im.excl, np.int32)
        d.nexcl = len(ex)
        d.excl = _pi(ex)
        for name, (idx, par) in (("bond", im.bonds), ("angle", im.angles), ("tors", im.torsions),
                                 ("impr", im.impropers)):
            i = keep(idx, np.int32)
            p = keep(par, np.float64)
            setattr(d, "n" + name, len(i))
            setattr(d, name + "_idx", _pi(i) if len(i) else None)
            setattr(d, name + "_par", _pd(p) if len(i) else None)
        st = ctypes.c_int(0)
        h = self.lib.pdgpu_create(int(device), ctypes.byref(d), ctypes.byref(st))
        if not h:
            raise ffi.PDGPUError(st.value, "pdgpu_create")
        self.h = ctypes.c_void_p(h)
        self.natom = im.natom
        self.nsystems = im.nsystems

    def close(self):
        if getattr(self, "h", None):
            self.lib.pdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- parameters --------------------------------------------------------
    def set_nb(self, **kw):
        p = ffi.NBParams(**kw)
        ffi.check(self.lib.pdgpu_set_nb_params(self.h, ctypes.byref(p)), "pdgpu_set_nb_params")

    def set_gb(self, **kw):
        p = ffi.GBParams(**kw)
        ffi.check(self.lib.pdgpu_set_gb_params(self.h, ctypes.byref(p)), "pdgpu_set_gb_params")

    def set_gb_mode(self, fast_mode, **vacuum):
        """FastMode of the GB component; vacuum: the GB object's FF_NonBonded settings (PD names)."""
        p = ffi.NBParams(**vacuum) if vacuum else None
        ffi.check(self.lib.pdgpu_set_gb_mode(self.h, int(bool(fast_mode)), ctypes.byref(p) if p else None),
                  "pdgpu_set_gb_mode")

    def set_list(self, padding, check_skin=True):
        p = ffi.ListParams(float(padding), int(check_skin))
        ffi.check(self.lib.pdgpu_set_list_params(self.h, ctypes.byref(p)), "pdgpu_set_list_params")

    def update_params(self, charge=None, radius=None, epsilon=None, gb_radius=None, gb_vj=None, gb_terms123=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in
                (charge, radius, epsilon, gb_radius, gb_vj, gb_terms123)]
        ffi.check(self.lib.pdgpu_update_params(self.h, *[_pd(a) for a in arrs]), "pdgpu_update_params")

    def update_params_device(self, charge=0, radius=0, epsilon=0, gb_radius=0, gb_vj=0, gb_terms123=0):
        """Device pointers (int addresses, 0 = keep) of per-atom FP64 parameter arrays."""
        ptrs = [ctypes.c_void_p(p or None) for p in (charge, radius, epsilon, gb_radius, gb_vj, gb_terms123)]
        ffi.check(self.lib.pdgpu_update_params_device(self.h, *ptrs), "pdgpu_update_params_device")

    def nb_energy_full(self):
        """FF_NonBonded energies of every system; they and the positions become the reference."""
        E = (ffi.Energies * self.nsystems)()
        ffi.check(self.lib.pdgpu_nb_energy_full(self.h, E), "pdgpu_nb_energy_full")
        return [e.as_dict() for e in E]

    def nb_energy_update(self):
        """Energies after the atoms that moved since the reference (partial recalculation)."""
        E = (ffi.Energies * self.nsystems)()
        n = ctypes.c_int()
        ffi.check(self.lib.pdgpu_nb_energy_update(self.h, E, ctypes.byref(n)), "pdgpu_nb_energy_update")
        return [e.as_dict() for e in E], n.value

    def param_grad(self, what):
        """Energies of every system and dE/dp per atom (J per parameter unit) for the
        per-atom parameter arrays: dict charge, radius, epsilon, gb_radius, gb_vj, gb_terms123."""
        names = ("charge", "radius", "epsilon", "gb_radius", "gb_vj", "gb_terms123")
        out = {n: np.zeros(self.natom) for n in names}
        g = ffi.ParamGrads(*[out[n].ctypes.data for n in names])
        E = (ffi.Energies * self.nsystems)()
        ffi.check(self.lib.pdgpu_param_grad(self.h, what, E, ctypes.byref(g)), "pdgpu_param_grad")
        return [e.as_dict() for e in E], out

    def param_grad_device(self, what, ptrs):
        """Queue dE/dp into device arrays: ptrs maps the pdgpu_param_grads field names to addresses."""
        names = ("charge", "radius", "epsilon", "gb_radius", "gb_vj", "gb_terms123")
        g = ffi.ParamGrads(*[ptrs.get(n) or None for n in names])
        ffi.check(self.lib.pdgpu_param_grad_device(self.h, what, ctypes.byref(g)), "pdgpu_param_grad_device")

    # -- state / evaluation ------------------------------------------------
    def set_positions(self, pos, stride=24):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        ffi.check(self.lib.pdgpu_set_positions(self.h, _pd(pos), stride), "pdgpu_set_positions")

    def set_positions_device(self, ptr):
        ffi.check(self.lib.pdgpu_set_positions_device(self.h, ctypes.c_void_p(ptr)), "pdgpu_set_positions_device")

    def get_positions(self, out=None):
        """Positions (A) of every atom; `out`, if given, is a C-contiguous float64
        (natom, 3) array filled in place (a page-locked one takes the direct DMA path)."""
        if out is None:
            out = np.zeros((self.natom, 3))
        elif out.dtype != np.float64 or out.shape != (self.natom, 3) or not out.flags.c_contiguous:
            raise ValueError("get_positions: out must be a C-contiguous float64 array of shape (%d, 3)" % self.natom)
        ffi.check(self.lib.pdgpu_get_positions(self.h, _pd(out), 24), "pdgpu_get_positions")
        return out

    def rebuild_list(self):
        ffi.check(self.lib.pdgpu_rebuild_list(self.h), "pdgpu_rebuild_list")

    def compute(self, what, forces=None):
        """Energies (list of dicts, one per system, J) and forces ADDED into `forces` (N)."""
        E = (ffi.Energies * self.nsystems)()
        fp = None
        if forces is not None:
            assert forces.dtype == np.float64 and forces.flags.c_contiguous and forces.shape == (self.natom, 3)
            fp = _pd(forces)
        ffi.check(self.lib.pdgpu_compute(self.h, what, E, fp, 24), "pdgpu_compute")
        return [e.as_dict() for e in E]

    def compute_device(self, what, dptr=None):
        ffi.check(self.lib.pdgpu_compute_device(self.h, what, None if dptr is None else ctypes.c_void_p(dptr)),
                  "pdgpu_compute_device")

    def energies(self):
        E = (ffi.Energies * self.nsystems)()
        ffi.check(self.lib.pdgpu_get_energies(self.h, E), "pdgpu_get_energies")
        return [e.as_dict() for e in E]

    def born_radii(self):
        out = np.zeros(self.natom)
        ffi.check(self.lib.pdgpu_get_born_radii(self.h, _pd(out)), "pdgpu_get_born_radii")
        return out

    def sasa(self):
        out = np.zeros(self.natom)
        ffi.check(self.lib.pdgpu_get_sasa(self.h, _pd(out)), "pdgpu_get_sasa")
        return out

    def list_stats(self):
        a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        ffi.check(self.lib.pdgpu_list_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
                  "pdgpu_list_stats")
        return {"tiles": a.value, "masked_tiles": b.value, "slots": c.value}

    def list_tiles(self):
        """The tile list as an (ntiles, 3) array of (bi, bj, flags), the tile
        capacity and the bytes of the arrays sized by the list."""
        n, cap, nbytes = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        ffi.check(self.lib.pdgpu_list_tiles(self.h, None, 0, ctypes.byref(n), ctypes.byref(cap),
                                            ctypes.byref(nbytes)), "pdgpu_list_tiles")
        out = np.zeros((n.value, 3), dtype=np.int32)
        if n.value:
            ffi.check(self.lib.pdgpu_list_tiles(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n.value,
                                                ctypes.byref(n), None, None), "pdgpu_list_tiles")
        return out, cap.value, nbytes.value

    def list_slots(self):
        """The atom held by each sorted slot of the current list (-1: padding)."""
        n = self.list_stats()["slots"]
        out = np.zeros(n, dtype=np.int32)
        ffi.check(self.lib.pdgpu_list_slots(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))),
                  "pdgpu_list_slots")
        return out

    def pair_census(self):
        """Pairs of the current list by the branch the pair kernels take
        (pdgpu_pair_census): NB in cutoff, GB in cutoff, GB term on, Born sums,
        Born close contacts."""
        out = (ctypes.c_longlong * 5)()
        ffi.check(self.lib.pdgpu_pair_census(self.h, out), "pdgpu_pair_census")
        return dict(zip(("nb", "gb", "gb_term", "born", "born_contact"), (int(x) for x in out)))

    def stream(self):
        return self.lib.pdgpu_stream(self.h)

    # -- dynamics ----------------------------------------------------------
    def md_setup(self, temps, integrator=1, timestep=2e-15, fric=1e13, update_nlist=10, update_sasa=5, what=0,
                 seed=1, use_graph=True):
        p = ffi.MDParams(int(integrator), float(timestep), float(fric), int(update_nlist), int(update_sasa),
                         int(what), int(seed), int(bool(use_graph)))
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(temps, np.float64), (self.nsystems,)))
        ffi.check(self.lib.pdgpu_md_setup(self.h, ctypes.byref(p), _pd(t)), "pdgpu_md_setup")

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, np.float64)
        ffi.check(self.lib.pdgpu_set_velocities(self.h, _pd(v), 24), "pdgpu_set_velocities")

    def get_velocities(self):
        out = np.zeros((self.natom, 3))
        ffi.check(self.lib.pdgpu_get_velocities(self.h, _pd(out), 24), "pdgpu_get_velocities")
        return out

    def md_run(self, nsteps, energy_on_last=False):
        ffi.check(self.lib.pdgpu_md_run(self.h, int(nsteps), int(bool(energy_on_last))), "pdgpu_md_run")

    def md_enqueue(self, nsteps, energy_on_last=False):
        ffi.check(self.lib.pdgpu_md_enqueue(self.h, int(nsteps), int(bool(energy_on_last))), "pdgpu_md_enqueue")

    def synchronize(self):
        ffi.check(self.lib.pdgpu_synchronize(self.h), "pdgpu_synchronize")

    KERNELS = {"nb": 0, "gb_born": 1, "gb_pair": 2, "gb_chain": 3, "lcpo": 4, "integrate": 5, "list": 6, "pack": 7,
               "bonded": 8}

    def time_kernel(self, name, reps=10, flush_l2=True):
        ms = ctypes.c_double()
        ffi.check(self.lib.pdgpu_time_kernel(self.h, self.KERNELS[name], int(reps), int(bool(flush_l2)),
                                             ctypes.byref(ms)), "pdgpu_time_kernel")
        return ms.value

    def kernel_launches(self):
        return int(self.lib.pdgpu_kernel_launches(self.h))

    def kinetic(self):
        out = np.zeros(self.nsystems)
        ffi.check(self.lib.pdgpu_get_kinetic(self.h, _pd(out)), "pdgpu_get_kinetic")
        return out

    # asynchronous host copies: `buf` page-locked (ffi.host_array), packed, left
    # untouched until synchronize() returns
    def _host_buf(self, buf, shape, what):
        if buf.dtype != np.float64 or buf.shape != shape or not buf.flags.c_contiguous:
            raise ValueError("%s: a C-contiguous float64 array of shape %s" % (what, shape))
        return _pd(buf)

    def set_positions_async(self, buf):
        ffi.check(self.lib.pdgpu_set_positions_async(self.h, self._host_buf(buf, (self.natom, 3), "set_positions_async")),
                  "pdgpu_set_positions_async")

    def get_positions_async(self, buf):
        ffi.check(self.lib.pdgpu_get_positions_async(self.h, self._host_buf(buf, (self.natom, 3), "get_positions_async")),
                  "pdgpu_get_positions_async")

    def kinetic_async(self, buf):
        ffi.check(self.lib.pdgpu_get_kinetic_async(self.h, self._host_buf(buf, (self.nsystems,), "kinetic_async")),
                  "pdgpu_get_kinetic_async")

    def remd_exchange(self, parity):
        acc = np.zeros(max(self.nsystems - 1, 1), np.int32)
        temps = np.zeros(self.nsystems)
        ffi.check(self.lib.pdgpu_remd_exchange(self.h, int(parity), _pi(acc), _pd(temps)), "pdgpu_remd_exchange")
        return acc[:self.nsystems - 1], temps

    def remd_set_modes(self, modes):
        """Exchange mode of each rung's lower replica: 0 Swap, 1 Downward, 2 Upward."""
        m = np.ascontiguousarray(np.broadcast_to(np.asarray(modes, np.int32), (self.nsystems,)))
        ffi.check(self.lib.pdgpu_remd_set_modes(self.h, _pi(m)), "pdgpu_remd_set_modes")

    def md_set_trajectory(self, every, nslots=16):
        """Frames every `every` steps into a page-locked ring of nslots frames (returned,
        shape (nslots, natom, 3)); every = 0 switches it off."""
        if every <= 0:
            ffi.check(self.lib.pdgpu_md_set_trajectory(self.h, 0, None, 0), "pdgpu_md_set_trajectory")
            self._traj_ring = None
            return None
        # page-locked through the library (pdgpu_host_alloc), so the copies stay
        # asynchronous; kept alive with the context
        ring = self._traj_ring = ffi.host_array((nslots, self.natom, 3))
        ffi.check(self.lib.pdgpu_md_set_trajectory(self.h, int(every), _pd(ring), int(nslots)),
                  "pdgpu_md_set_trajectory")
        return ring

    def md_trajectory_frames(self):
        return int(self.lib.pdgpu_md_trajectory_frames(self.h))

    def md_checkpoint(self):
        ffi.check(self.lib.pdgpu_md_checkpoint(self.h), "pdgpu_md_checkpoint")

    def md_rescue(self, seed):
        """Systems with non-finite state back to the checkpoint with fresh velocities;
        returns the per-system flags of the rescued ones."""
        flags = np.zeros(self.nsystems, np.int32)
        n = ctypes.c_int()
        ffi.check(self.lib.pdgpu_md_rescue(self.h, ctypes.c_ulonglong(seed), _pi(flags), ctypes.byref(n)),
                  "pdgpu_md_rescue")
        return flags.astype(bool)

    def autotune(self, trial_steps=20):
        a, b = ctypes.c_int(), ctypes.c_int()
        ffi.check(self.lib.pdgpu_md_autotune(self.h, int(trial_steps), ctypes.byref(a), ctypes.byref(b)),
                  "pdgpu_md_autotune")
        return {"UpdateNList": a.value, "ctas_per_sm": b.value, "gb_tiles_per_item": self.work_items(),
                "nb_groups": self.nb_groups()[0]}

    def set_launch_shape(self, ctas_per_sm):
        ffi.check(self.lib.pdgpu_set_launch_shape(self.h, int(ctas_per_sm)), "pdgpu_set_launch_shape")

    def launch_shape(self):
        a = ctypes.c_int()
        ffi.check(self.lib.pdgpu_get_launch_shape(self.h, ctypes.byref(a)), "pdgpu_get_launch_shape")
        return a.value

    def set_work_items(self, tiles_per_item):
        """GB work-item size: 1 single tiles, 2 tile pairs (rewritten at the next list build)."""
        ffi.check(self.lib.pdgpu_set_work_items(self.h, int(tiles_per_item)), "pdgpu_set_work_items")

    def work_items(self):
        a = ctypes.c_int()
        ffi.check(self.lib.pdgpu_get_work_items(self.h, ctypes.byref(a)), "pdgpu_get_work_items")
        return a.value

    def set_nb_groups(self, on):
        """LJ/Coulomb j-atom groups on or off (rewritten at the next list build)."""
        ffi.check(self.lib.pdgpu_set_nb_groups(self.h, int(bool(on))), "pdgpu_set_nb_groups")

    def nb_groups(self):
        """(setting, groups, tiles left on the tile path) of the last list build."""
        a, g, r = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
        ffi.check(self.lib.pdgpu_get_nb_groups(self.h, ctypes.byref(a), ctypes.byref(g), ctypes.byref(r)),
                  "pdgpu_get_nb_groups")
        return bool(a.value), g.value, r.value
