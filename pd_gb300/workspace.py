"""System description and simulation state, mirroring PD's WorkSpace.

PD keeps per-atom parameters in ``WorkSpace::atom`` (Particle, PD
src/mmlib/system/fundamentals.h:106-197), coordinates / forces / velocities in
``WorkSpace::cur`` (SnapShot, src/mmlib/workspace/snapshot.h:33-39) and energies
in ``WorkSpace::ene`` (Hamiltonian, src/mmlib/workspace/hamiltonian.h:40-107).
This module keeps the same names and PD's units (Angstrom, J, N, kg, m/s,
sqrt(J) epsilons) so a PD user finds the familiar fields.

A ``SystemImage`` holds the static description of one or more systems (a
batch); a ``WorkSpace`` adds the state and owns the device context.
"""
import copy
import os

import numpy as np

# AMBER99 1-4 scalings (param/amber99aa.ff:29-30), used when an image does not carry its own
_DEFAULT_SCALING14 = (0.5, 0.83333)


class Hamiltonian:
    """PD's energy record (hamiltonian.h:43-66); energies in J per molecule."""

    FIELDS = ("etot", "epot", "ekin", "epot_vdw", "epot_elec", "epot_bond", "epot_angle", "epot_torsion",
              "epot_surf", "epot_pol", "epot_pol_cross", "epot_pol_self", "InternalVirial", "epot_vdw_att",
              "epot_vdw_rep")

    def __init__(self):
        self.zero()

    def zero(self):
        for k in self.FIELDS:
            setattr(self, k, 0.0)

    def as_dict(self):
        return {k: getattr(self, k) for k in self.FIELDS}


class SystemImage:
    """Static description of one or more independent systems, concatenated."""

    def __init__(self, natoms, box, charge, radius, epsilon, mass, excl, gb_radius=None, gb_vj=None,
                 gb_terms123=None, lcpo_radius=None, lcpo_p=None, lcpo_sigma=None, lcpo_use=None, bonds=None,
                 angles=None, torsions=None, impropers=None, pos=None, scaling14=_DEFAULT_SCALING14,
                 gb_P=(0.073, 0.921, 6.211, 15.236, 1.254)):
        self.natoms = np.asarray(natoms, dtype=np.int32).reshape(-1)
        self.nsystems = len(self.natoms)
        self.box = np.asarray(box, dtype=np.float64).reshape(self.nsystems, 3)
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        self.charge, self.radius, self.epsilon, self.mass = f(charge), f(radius), f(epsilon), f(mass)
        self.excl = np.ascontiguousarray(excl, dtype=np.int32).reshape(-1, 3)
        self.gb_radius, self.gb_vj, self.gb_terms123 = f(gb_radius), f(gb_vj), f(gb_terms123)
        self.lcpo_radius, self.lcpo_sigma = f(lcpo_radius), f(lcpo_sigma)
        self.lcpo_p = None if lcpo_p is None else np.ascontiguousarray(lcpo_p, dtype=np.float64).reshape(-1, 4)
        self.lcpo_use = None if lcpo_use is None else np.ascontiguousarray(lcpo_use, dtype=np.int32)
        z2 = (np.zeros((0, 2), np.int32), np.zeros((0, 2)))
        z5 = (np.zeros((0, 5), np.int32), np.zeros((0, 12)))
        norm = lambda t, z: z if t is None else (np.ascontiguousarray(t[0], np.int32), np.ascontiguousarray(t[1], np.float64))
        self.bonds = norm(bonds, z2)
        self.angles = norm(angles, (np.zeros((0, 3), np.int32), np.zeros((0, 2))))
        self.torsions = norm(torsions, z5)
        self.impropers = norm(impropers, z5)
        self.pos = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.scaling14 = tuple(float(x) for x in scaling14)
        self.gb_P = tuple(float(x) for x in gb_P)

    @property
    def natom(self):
        return int(self.natoms.sum())

    @property
    def offsets(self):
        return np.concatenate([[0], np.cumsum(self.natoms)]).astype(np.int64)

    @property
    def periodic(self):
        return bool(np.all(self.box > 0))

    @property
    def has_gb(self):
        return self.gb_vj is not None

    @property
    def has_sa(self):
        return self.lcpo_p is not None

    # -- loaders -----------------------------------------------------------
    @classmethod
    def from_npz(cls, path):
        d = np.load(path, allow_pickle=False)
        if "class_table" in d:
            return cls._from_compact(d)
        return cls._from_fixture(d)

    @classmethod
    def _from_fixture(cls, d):
        n = len(d["pos"])
        g = lambda k: d[k] if k in d else None
        s14 = _DEFAULT_SCALING14
        for pre in ("gb_", "nb_"):
            if pre + "Vdw14Scaling" in d:
                s14 = (float(d[pre + "Vdw14Scaling"][0]), float(d[pre + "Elec14Scaling"][0]))
                break
        return cls([n], d["box"], d["charge"], d["radius"], d["epsilon"], d["mass"], d["excl"],
                   gb_radius=g("gb_radius"), gb_vj=g("gb_vj"), gb_terms123=g("gb_terms123"),
                   lcpo_radius=g("lcpo_radius"), lcpo_p=g("lcpo_P"), lcpo_sigma=g("lcpo_sigma"),
                   lcpo_use=g("lcpo_use"), bonds=(d["bond_idx"], d["bond_par"]),
                   angles=(d["angle_idx"], d["angle_par"]), torsions=(d["torsion_idx"], d["torsion_par"]),
                   impropers=(d["improper_idx"], d["improper_par"]), pos=d["pos"], scaling14=s14,
                   gb_P=tuple(d["gb_P"]) if "gb_P" in d else (0.073, 0.921, 6.211, 15.236, 1.254))

    @classmethod
    def _from_compact(cls, d):
        cols = [str(c) for c in d["class_cols"]]
        tab = d["class_table"][d["atom_class"].astype(np.int64)]
        col = lambda name: tab[:, cols.index(name)]
        n = len(d["pos"])
        natoms = d["system_natoms"] if "system_natoms" in d else [n]
        nsys = len(natoms)
        box = d["box"].reshape(-1, 3)
        if len(box) != nsys:
            box = np.repeat(box[:1], nsys, axis=0)
        ei = d["excl_i"] if "excl_i" in d else np.cumsum(d["excl_first_delta"].astype(np.int64)).astype(np.int32)
        excl = np.stack([ei, ei + d["excl_dj"], d["excl_bo"].astype(np.int32)], axis=1)
        has_gb = bool(np.any(col("gb_vj") != 0))
        has_sa = bool(np.any(col("lcpo_use") != 0))

        def bonded(k):
            par = d[k + "_partable"][d[k + "_parclass"].astype(np.int64)]
            if k + "_idx" in d:
                return d[k + "_idx"], par
            first = np.cumsum(d[k + "_first_delta"].astype(np.int64))
            cols = [first] + [first + d[k + "_rel"][:, c] for c in range(d[k + "_rel"].shape[1])]
            if k + "_terms" in d:
                cols.append(d[k + "_terms"].astype(np.int64))
            return np.stack(cols, axis=1).astype(np.int32), par

        return cls(natoms, box, col("charge"), col("radius"), col("epsilon"), col("mass"), excl,
                   gb_radius=col("gb_radius") if has_gb else None, gb_vj=col("gb_vj") if has_gb else None,
                   gb_terms123=col("gb_terms123") if has_gb else None,
                   lcpo_radius=col("lcpo_radius") if has_sa else None,
                   lcpo_p=np.stack([col("lcpo_P%d" % k) for k in range(1, 5)], axis=1) if has_sa else None,
                   lcpo_sigma=col("lcpo_sigma") if has_sa else None,
                   lcpo_use=col("lcpo_use").astype(np.int32) if has_sa else None,
                   bonds=bonded("bond"), angles=bonded("angle"), torsions=bonded("torsion"),
                   impropers=bonded("improper"), pos=d["pos"].astype(np.float64),
                   scaling14=tuple(d["scaling14"]) if "scaling14" in d else _DEFAULT_SCALING14,
                   gb_P=tuple(d["gb_P"]) if "gb_P" in d else (0.073, 0.921, 6.211, 15.236, 1.254))

    @classmethod
    def concat(cls, images):
        """Batch several images into one multi-system image (indices re-based)."""
        offs = np.cumsum([0] + [im.natom for im in images])
        cat = lambda name: None if getattr(images[0], name) is None else np.concatenate(
            [getattr(im, name) for im in images])

        def catidx(getter, width_idx):
            idx = np.concatenate([getter(im)[0] + np.where(np.arange(getter(im)[0].shape[1]) < width_idx, o, 0)
                                  for im, o in zip(images, offs)])
            par = np.concatenate([getter(im)[1] for im in images])
            return idx, par

        excl = np.concatenate([im.excl + np.array([o, o, 0]) for im, o in zip(images, offs)])
        return cls(np.concatenate([im.natoms for im in images]), np.concatenate([im.box for im in images]),
                   cat("charge"), cat("radius"), cat("epsilon"), cat("mass"), excl,
                   gb_radius=cat("gb_radius"), gb_vj=cat("gb_vj"), gb_terms123=cat("gb_terms123"),
                   lcpo_radius=cat("lcpo_radius"), lcpo_p=cat("lcpo_p"), lcpo_sigma=cat("lcpo_sigma"),
                   lcpo_use=cat("lcpo_use"), bonds=catidx(lambda im: im.bonds, 2),
                   angles=catidx(lambda im: im.angles, 3), torsions=catidx(lambda im: im.torsions, 4),
                   impropers=catidx(lambda im: im.impropers, 4),
                   pos=None if images[0].pos is None else np.concatenate([im.pos for im in images]),
                   scaling14=images[0].scaling14, gb_P=images[0].gb_P)

    def replicate(self, reps):
        """A periodic one-system image copied reps = (nx, ny, nz) times along its
        box axes, as one system in the enlarged box (same density, reps-fold atoms)."""
        if self.nsystems != 1 or not self.periodic or self.pos is None:
            raise ValueError("replicate: one periodic system with positions")
        L = self.box[0]
        copies = []
        for i in range(int(reps[0])):
            for j in range(int(reps[1])):
                for k in range(int(reps[2])):
                    c = copy.copy(self)
                    c.pos = self.pos + L * np.array([i, j, k], dtype=np.float64)
                    copies.append(c)
        out = SystemImage.concat(copies)
        out.natoms = np.array([out.natom], dtype=np.int32)
        out.nsystems = 1
        out.box = (L * np.asarray(reps, dtype=np.float64)).reshape(1, 3)
        return out

    def subset(self, k):
        """System k of a batch as its own image."""
        o = self.offsets
        a, b = int(o[k]), int(o[k + 1])
        sl = lambda x: None if x is None else x[a:b]
        m = (self.excl[:, 0] >= a) & (self.excl[:, 0] < b)

        def sub(t, width_idx):
            idx, par = t
            sel = (idx[:, 0] >= a) & (idx[:, 0] < b)
            i = idx[sel].copy()
            i[:, :width_idx] -= a
            return i, par[sel]

        return SystemImage([b - a], self.box[k:k + 1], sl(self.charge), sl(self.radius), sl(self.epsilon),
                           sl(self.mass), self.excl[m] - np.array([a, a, 0]), gb_radius=sl(self.gb_radius),
                           gb_vj=sl(self.gb_vj), gb_terms123=sl(self.gb_terms123),
                           lcpo_radius=sl(self.lcpo_radius), lcpo_p=sl(self.lcpo_p),
                           lcpo_sigma=sl(self.lcpo_sigma), lcpo_use=sl(self.lcpo_use), bonds=sub(self.bonds, 2),
                           angles=sub(self.angles, 3), torsions=sub(self.torsions, 4),
                           impropers=sub(self.impropers, 4), pos=sl(self.pos), scaling14=self.scaling14,
                           gb_P=self.gb_P)


WORKLOAD_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "workloads")


def load_workload(name):
    """Synthetic benchmark systems built by PD (see tests/golden/make_golden.py)."""
    return SystemImage.from_npz(os.path.join(WORKLOAD_DIR, name + ".npz"))


class SnapShot:
    """Coordinates (A), forces (N) and velocities (m/s): SnapShotAtom {p, f, v} as arrays."""

    def __init__(self, n):
        self.p = np.zeros((n, 3))
        self.f = np.zeros((n, 3))
        self.v = np.zeros((n, 3))


class WorkSpace:
    """Simulation state of a SystemImage plus its GPU context (created on first use)."""

    def __init__(self, image, device=0, positions=None):
        self.image = image
        self.device = device
        n = image.natom
        self.cur = SnapShot(n)
        if positions is not None:
            self.cur.p[:] = positions
        elif image.pos is not None:
            self.cur.p[:] = image.pos
        self.ene = Hamiltonian()
        self.Step = 0
        self.Padding = 0.5          # NeighbourListBase::Padding default (neighbourlist.cpp:35)
        self._ctx = None
        self._ctx_params = None
        self.per_system_energies = None

    def nAtoms(self):
        return self.image.natom

    def zeroForces(self):
        """WorkSpace::zeroForces (workspace.cpp:316-324): energies and forces to zero."""
        self.ene.zero()
        self.cur.f[:] = 0.0

    # -- device context ----------------------------------------------------
    def context(self):
        if self._ctx is None:
            from .engine import DeviceContext
            self._ctx = DeviceContext(self.image, self.device)
        return self._ctx

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None
