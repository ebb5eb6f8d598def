"""MolecularDynamics and batched REMD with PD's interface, run on the device.

Mirrors PD's ``MolecularDynamics`` protocol (PD src/mmlib/protocols/md.h,
md.cpp:174-283) and ``REX_Local`` (remd.cpp:65-215).  The whole step — list
refresh, forces, FP64 integrator — runs in libpdgpu, replayed from captured
CUDA graphs; the host only schedules and reads back on request.
"""
import numpy as np

from . import ffi
from .forcefield import FF_SASA_LCPO_GPU

KB = 1.38065E-23          # PhysicsConst::kB (forcefield.cpp:39)


def maxwell_boltzmann(masses, temp, seed, natom_per_system=None):
    """setInitialSpeeds (md.cpp:359-380): Gaussian velocities sqrt(kB T / m), then the
    kinetic energy of each system scaled to exactly 3/2 N kB T."""
    rng = np.random.default_rng(seed)
    m = np.asarray(masses, np.float64)
    v = rng.standard_normal((len(m), 3)) * np.sqrt(KB * 1.0 / m)[:, None]
    counts = [len(m)] if natom_per_system is None else list(natom_per_system)
    temps = np.broadcast_to(np.asarray(temp, np.float64), (len(counts),))
    o = 0
    for n, T in zip(counts, temps):
        sl = slice(o, o + n)
        ke = 0.5 * (m[sl, None] * v[sl] ** 2).sum()
        target = 1.5 * n * KB * T
        v[sl] *= np.sqrt(target / ke) if ke > 0 else 0.0
        o += n
    return v


class MolecularDynamics:
    """PD-style MD protocol over every system of a WorkSpace's batch."""

    VelocityVerlet = 0
    Langevin = 1

    def __init__(self, ff):
        self.ff = ff
        self.wspace = ff.wspace
        # md.cpp:60-86 defaults (Integrator Beeman is not provided; Langevin is the default here)
        self.Integrator = MolecularDynamics.Langevin
        self.Timestep = 1E-15
        self.RandVel = True
        self.FricCoeff = 10E12
        self.Steps = 0
        self.UpdateNList = 10
        self.Seed = 1
        self.UseGraph = True
        self.UpdateTra = 0          # frame every UpdateTra steps (md.cpp:277); 0 = none
        self.trajectory = None      # a writer with append(frames), e.g. trajectory.PDBTrajectory
        self._temp = np.array([300.0])
        self._setup_done = False
        self.Step = 0

    def setTargetTemp(self, T):
        self._temp = np.atleast_1d(np.asarray(T, np.float64))
        self._setup_done = False

    def _what(self):
        w = 0
        for c in self.ff.components:
            if c.Active:
                w |= c.flag
        return w

    def setup(self):
        ws = self.wspace
        ctx = self.ff._prepare()
        ctx.set_positions(ws.cur.p)
        sa = [c for c in self.ff.components if isinstance(c, FF_SASA_LCPO_GPU)]
        temps = np.broadcast_to(self._temp, (ws.image.nsystems,))
        ctx.md_setup(temps, integrator=self.Integrator, timestep=self.Timestep, fric=self.FricCoeff,
                     update_nlist=self.UpdateNList, update_sasa=sa[0].UpdateSasa if sa else 1, what=self._what(),
                     seed=self.Seed, use_graph=self.UseGraph)
        if self.RandVel:
            ws.cur.v[:] = maxwell_boltzmann(ws.image.mass, temps, self.Seed, ws.image.natoms)
        ctx.set_velocities(ws.cur.v)
        self._setup_done = True
        return ctx

    def run(self, steps=None, energies=True):
        """Run Steps (or `steps`) steps; positions, velocities and energies come back to the WorkSpace."""
        n = self.Steps if steps is None else steps
        ctx = self.setup() if not self._setup_done else self.wspace.context()
        ring = None
        if self.UpdateTra > 0 and self.trajectory is not None:
            # every frame of this run fits the ring: no slot is reused before it is written out
            ring = ctx.md_set_trajectory(self.UpdateTra, nslots=max(1, n // self.UpdateTra))
        ctx.md_run(n, energy_on_last=energies)
        if ring is not None:
            k = ctx.md_trajectory_frames()
            self.trajectory.append(ring[:k])
            ctx.md_set_trajectory(0)
        self.Step += n
        self.sync(ctx, energies)
        return n

    def sync(self, ctx=None, energies=True):
        ctx = ctx or self.wspace.context()
        ws = self.wspace
        ws.cur.p[:] = ctx.get_positions()
        ws.cur.v[:] = ctx.get_velocities()
        ke = ctx.kinetic()
        ws.ene.ekin = float(ke.sum())
        if energies:
            es = ctx.energies()
            ws.per_system_energies = es
            ws.ene.epot = float(sum(e["epot"] for e in es))
            ws.ene.epot_vdw = float(sum(e["vdw"] for e in es))
            ws.ene.epot_elec = float(sum(e["elec"] for e in es))
            ws.ene.epot_pol = float(sum(e["pol"] for e in es))
            ws.ene.epot_surf = float(sum(e["surf"] for e in es))
        ws.ene.etot = ws.ene.epot + ws.ene.ekin
        self.kinetic_per_system = ke

    def temperature(self):
        """calcKineticEnergy: T = 2 K / (3 N kB), per system."""
        n = self.wspace.image.natoms
        return 2.0 * self.kinetic_per_system / (3.0 * n * KB)


class REX_Local:
    """Replica exchange over the systems of a batch: system k starts at ladder rung k.

    Every ExchangeFreq steps all replicas advance together (one device launch
    sequence for the whole batch) and an alternating even/odd exchange sweep
    runs on the device (remd.cpp:178-215).
    """

    Swap, Downward, Upward = 0, 1, 2     # REX_Replica::ExchangeModeType (remd.h:49)

    def __init__(self, md, temps, exchange_mode=0):
        self.md = md
        self.temps = np.asarray(temps, np.float64)
        self.ExchangeFreq = 500
        self.Steps = 0            # number of exchange rounds
        self.accepted = None
        self.rescues = 0          # replicas rescued after an unstable round (remd.cpp:118-147)
        # per replica (rung), as addReplica(..., exmode) sets it; the lower replica's mode governs a pair
        self.ExchangeMode = np.broadcast_to(np.asarray(exchange_mode, np.int32), self.temps.shape).copy()
        self.md.setTargetTemp(self.temps)

    @staticmethod
    def geometric_ladder(tmin, tmax, n):
        return tmin * (tmax / tmin) ** (np.arange(n) / max(n - 1, 1))

    # -- checkpoints in PD's MIME snapshot format (remd.cpp:319-331) -------------
    def _rung_systems(self, ctx):
        """System index at each temperature rung (rung r holds PD's replica r)."""
        cur = getattr(self, "current_temps", None)
        if cur is None:
            return np.arange(len(self.temps))
        return np.array([int(np.argmin(np.abs(cur - T))) for T in self.temps])

    def writeCheckPointMIME(self, f):
        """printCheckPointMIME into an open text file (or path): one section
        ``remd<r>`` per replica r, the structure now at temperature rung r."""
        from . import checkpoint
        if isinstance(f, str):
            with open(f, "w") as fh:
                return self.writeCheckPointMIME(fh)
        ctx = self.md.wspace.context()
        pos, vel = ctx.get_positions(), ctx.get_velocities()
        es = getattr(self.md.wspace, "per_system_energies", None)
        off = self.md.wspace.image.offsets
        for r, k in enumerate(self._rung_systems(ctx)):
            sl = slice(int(off[k]), int(off[k + 1]))
            epot = es[k]["epot"] if es else 0.0
            checkpoint.write_snapshot(f, "remd%d" % r, pos[sl], vel[sl], None, epot)

    def printCheckPointMIME(self):
        import sys
        self.writeCheckPointMIME(sys.stdout)

    def readCheckPointMIME(self, filename):
        """readCheckPointMIME: replica r's structure (positions, velocities) goes to
        the system at rung r; every section must match that system's atom count."""
        from . import checkpoint
        with open(filename) as f:
            secs = checkpoint.read_snapshots(f)
        ctx = self.md.setup() if not self.md._setup_done else self.md.wspace.context()
        pos, vel = ctx.get_positions(), ctx.get_velocities()
        off = self.md.wspace.image.offsets
        for r, k in enumerate(self._rung_systems(ctx)):
            name = "remd%d" % r
            if name not in secs:
                raise KeyError("MIME snapshot '%s' not found in %s" % (name, filename))
            snap = secs[name]
            sl = slice(int(off[k]), int(off[k + 1]))
            if len(snap["pos"]) != sl.stop - sl.start:
                raise ValueError("%s holds %d atoms, replica %d has %d" % (name, len(snap["pos"]), r,
                                                                         sl.stop - sl.start))
            pos[sl] = snap["pos"]
            vel[sl] = snap["vel"]
        ctx.set_positions(pos)
        ctx.set_velocities(vel)
        self.md.sync(ctx, energies=False)

    def run(self, rounds=None):
        n = self.Steps if rounds is None else rounds
        ctx = self.md.setup() if not self.md._setup_done else self.md.wspace.context()
        acc = np.zeros(max(len(self.temps) - 1, 1))
        ctx.remd_set_modes(self.ExchangeMode)
        for r in range(n):
            ctx.md_checkpoint()
            try:
                ctx.md_run(self.ExchangeFreq, energy_on_last=True)
            except ffi.PDGPUError as e:
                # an unstable replica: back to its structure at the start of the
                # round with new velocities (PD: remd.run_core_failure), then the
                # energies for the exchange criterion.  A non-finite atom shows
                # as NaN, fixed-point overflow or a stale list.
                if e.status not in (-5, -4, -8):
                    raise
                bad = ctx.md_rescue(self.md.Seed * 7919 + r)
                if not bad.any():
                    raise
                self.rescues += int(bad.sum())
                ctx.md_run(1, energy_on_last=True)
            a, current = ctx.remd_exchange(r % 2)
            acc[:len(a)] += a
            self.current_temps = current
        self.accepted = acc[:len(self.temps) - 1]
        self.md.sync(ctx)
        return n
