"""Drop-in forcefield components with PD's interface, evaluated on the GPU.

Mirrors PD's ``ForcefieldBase`` / ``Forcefield`` container (PD
src/mmlib/forcefields/forcefield.h:110-336) and the public attributes of
``FF_NonBonded`` (nonbonded.h:62-231), ``FF_GeneralizedBorn_Still``
(gbff.h:123-203), ``FF_SASA_LCPO`` (lcpo.h:49-143) and ``FF_Bonded``
(ffbonded.h:120-216).  Components are added to a ``Forcefield`` in order and
their energies / forces are added into the WorkSpace exactly as PD's
``Forcefield::calcForces`` does (forcefield.cpp:237-264).  All arithmetic runs
in libpdgpu; there is no CPU path.
"""
import numpy as np

from . import ffi

_J2KCALMOL = 6.0221418E23 / 4184.0


class ForcefieldBase:
    name = "ForcefieldBase"
    flag = 0

    def __init__(self, wspace):
        self.wspace = wspace
        self.Active = True
        self.epot = 0.0
        self.needsetup = True

    def getWSpace(self):
        return self.wspace

    def calcCheckSum(self):
        return hash(tuple(sorted((k, v) for k, v in vars(self).items()
                                 if isinstance(v, (int, float, bool, str)) and k not in ("epot", "needsetup"))))

    def setup(self):
        self.needsetup = False

    def ensuresetup(self):
        cs = self.calcCheckSum()
        if self.needsetup or cs != getattr(self, "_checksum", None):
            self.setup()
            self._checksum = cs
            self.wspace._ctx_params = None

    def configure(self, ctx):
        """Push this component's parameters to the device context."""

    def distribute(self, e, energies_only=False):
        """Add this component's share of the energies (dict, J) into wspace.ene; PD field names.
        energies_only: the evaluation was Forcefield::calcEnergies."""

    def calcForces(self):
        ff = Forcefield(self.wspace)
        ff.add(self)
        ff.calcForces(zero=False)

    def calcEnergies(self):
        self.calcForces()

    def info(self):
        print(" --%s-- " % self.name)
        for k, v in sorted(vars(self).items()):
            if isinstance(v, (int, float, bool)) and not k.startswith("_"):
                print("  %-22s %s" % (k, v))

    def infoLineHeader(self):
        return ""

    def infoLine(self):
        return ""


class FF_NonBonded_GPU(ForcefieldBase):
    """LJ + Coulomb with PD's switching, FF_NonBonded semantics (nonbonded.cpp:559-910)."""

    name = "Non-Bonded Forcefield (GPU)"
    flag = ffi.NB

    def __init__(self, wspace):
        super().__init__(wspace)
        # FF_NonBonded::settodefault, nonbonded.cpp:985-1021
        self.DoVdw = True
        self.DoElec = True
        self.Cutoff = 15.0
        self.InnerCutoff = 12.0
        self.VdwCutoff = 15.0
        self.VdwInnerCutoff = 12.0
        self.AutoScaling14 = True
        self.Vdw14Scaling = 1.0
        self.Elec14Scaling = 1.0
        self.Dielectric = 1.0
        self.DDDielectric = False
        self.ForceSwitch = True
        self.EnergySwitch = False
        self.UsePartialRecalc = False   # calcEnergies after small moves (nonbonded.cpp:1154-1182)
        # long-range LJ correction, off by default (nonbonded.cpp:1009-1013)
        self.VdwCor = False
        self.VdwCorDensity = 0.0        # atoms per A^3
        self.VdwCorEpsilon = 0.0        # kcal/mol
        self.VdwCorRadius = 0.0         # A
        self.VdwCorCutoff = 0.0         # A
        self.epot_vdw = 0.0
        self.epot_elec = 0.0

    def setup(self):
        # nonbonded.cpp:1025-1053: 1-4 scalings come from the parameter set when AutoScaling14
        if self.AutoScaling14:
            self.Vdw14Scaling, self.Elec14Scaling = self.wspace.image.scaling14
        if self.DDDielectric:
            raise ffi.PDGPUError(-7, "DDDielectric is not selected by PD's force path (nonbonded.cpp:1222-1246)")
        self.needsetup = False

    def _nb_kwargs(self):
        return dict(Cutoff=float(self.Cutoff), InnerCutoff=float(self.InnerCutoff), VdwCutoff=float(self.VdwCutoff),
                    VdwInnerCutoff=float(self.VdwInnerCutoff), Vdw14Scaling=float(self.Vdw14Scaling),
                    Elec14Scaling=float(self.Elec14Scaling), Dielectric=float(self.Dielectric),
                    EnergySwitch=int(bool(self.EnergySwitch)), ForceSwitch=int(bool(self.ForceSwitch)),
                    DoVdw=int(bool(self.DoVdw)), DoElec=int(bool(self.DoElec)))

    def configure(self, ctx):
        ctx.set_nb(**self._nb_kwargs())

    def vdw_correction(self):
        """With VdwCor, PD's pair loop adds, for every atom i, the analytic integral of
        the attractive LJ term from VdwCorCutoff to infinity (nonbonded.cpp:862-874):
        -1/2 density eps (8/3) pi R^6 / Rc^3, an energy without force.  Total in J."""
        if not self.VdwCor:
            return 0.0
        r3 = self.VdwCorRadius ** 3
        per_atom = (-0.5 * self.VdwCorDensity * self.VdwCorEpsilon / _J2KCALMOL * (8.0 / 3.0) * np.pi * r3 * r3 /
                    self.VdwCorCutoff ** 3)
        return self.wspace.nAtoms() * per_atom

    def distribute(self, e, energies_only=False):
        ene = self.wspace.ene
        cor = self.vdw_correction()
        vdw = e["vdw"] + cor
        ene.epot += vdw + e["elec"]
        ene.epot_vdw = vdw               # PD overwrites these two (nonbonded.cpp:681-682)
        ene.epot_elec = e["elec"]
        ene.epot_vdw_att += cor
        ene.InternalVirial += e["virial"]
        self.epot_vdw, self.epot_elec = vdw, e["elec"]
        self.epot = vdw + e["elec"]

    def infoLineHeader(self):
        return "%8s%8s" % ("EVdw", "Ecoul")

    def infoLine(self):
        return "% 8.1f% 8.1f" % (self.epot_vdw * _J2KCALMOL, self.epot_elec * _J2KCALMOL)


class FF_GeneralizedBorn_Still_GPU(FF_NonBonded_GPU):
    """Still GB (gbff.cpp): FastMode (default) fuses GB with the vacuum LJ/Coulomb
    (calcForcesIncludingVacuo, :1466-1835); FastMode off runs FF_NonBonded's
    calcForces with this object's own settings plus calcBornForces (:1189-1437)."""

    name = "Generalised Born Still (GPU)"
    flag = ffi.GB

    def __init__(self, wspace):
        super().__init__(wspace)
        # gbff.cpp:33-55
        self.FastMode = True
        self.DielectricSolvent = 80.0
        self.DielectricSolute = 1.0
        self.GbsaStillCutoff = 10.0
        self.ExpApproxThreshold = -4.0
        self.DielectricOffset = -0.090
        self.BornRadiusOffset = 0.0
        self.ForceSwitch = False
        self.EnergySwitch = True
        self.P1, self.P2, self.P3, self.P4, self.P5 = 0.073, 0.921, 6.211, 15.236, 1.254
        self.epot_pol = self.epot_pol_self = self.epot_pol_cross = 0.0

    def setup(self):
        super().setup()
        im = self.wspace.image
        if not im.has_gb:
            raise ffi.PDGPUError(-1, "the system image carries no GB radii / Vj / terms123")
        # the parameter file's GENERALPARAMETERS override the constructor defaults (gbff.cpp:234-263)
        self.P1, self.P2, self.P3, self.P4, self.P5 = im.gb_P
        self.needsetup = False

    def configure(self, ctx):
        ctx.set_gb(Cutoff=float(self.Cutoff), InnerCutoff=float(self.InnerCutoff), VdwCutoff=float(self.VdwCutoff),
                   VdwInnerCutoff=float(self.VdwInnerCutoff), Vdw14Scaling=float(self.Vdw14Scaling),
                   Elec14Scaling=float(self.Elec14Scaling), DielectricSolute=float(self.DielectricSolute),
                   DielectricSolvent=float(self.DielectricSolvent), GbsaStillCutoff=float(self.GbsaStillCutoff),
                   ExpApproxThreshold=float(self.ExpApproxThreshold), BornRadiusOffset=float(self.BornRadiusOffset),
                   P4=float(self.P4), P5=float(self.P5))
        # this object's FF_NonBonded settings: the vacuum part when FastMode is off and in calcEnergies
        ctx.set_gb_mode(self.FastMode, Cutoff=float(self.Cutoff), InnerCutoff=float(self.InnerCutoff),
                        VdwCutoff=float(self.VdwCutoff), VdwInnerCutoff=float(self.VdwInnerCutoff),
                        Vdw14Scaling=float(self.Vdw14Scaling), Elec14Scaling=float(self.Elec14Scaling),
                        Dielectric=float(self.Dielectric), EnergySwitch=int(bool(self.EnergySwitch)),
                        ForceSwitch=int(bool(self.ForceSwitch)), DoVdw=int(bool(self.DoVdw)),
                        DoElec=int(bool(self.DoElec)))

    def distribute(self, e, energies_only=False):
        ene = self.wspace.ene
        # the vacuum part runs through FF_NonBonded (and its VdwCor) with FastMode off and
        # in calcEnergies (gbff.cpp:178-197); FastMode's fused loop has no correction
        cor = self.vdw_correction() if (energies_only or not self.FastMode) else 0.0
        vdw = e["vdw"] + cor
        ene.epot_vdw = vdw
        ene.epot_elec = e["elec"]
        ene.epot_vdw_att += cor
        ene.epot += vdw + e["elec"] + e["pol"]
        ene.epot_pol += e["pol"]
        ene.epot_pol_cross += e["pol_cross"]
        ene.epot_pol_self += e["pol_self"]
        self.epot_vdw, self.epot_elec = vdw, e["elec"]
        self.epot_pol, self.epot_pol_self, self.epot_pol_cross = e["pol"], e["pol_self"], e["pol_cross"]
        self.epot = vdw + e["elec"] + e["pol"]

    def infoLineHeader(self):
        return "\t%6s\t%6s\t%6s\t%6s\t%6s\t%7s" % ("EVdw", "Ecoul", "Eself", "Ecross", "Epol", "Epol+ES")

    def infoLine(self):
        k = _J2KCALMOL
        return "\t%6.1f\t%6.1f\t%6.1f\t%6.1f\t%6.1f\t%7.2f" % (
            self.epot_vdw * k, self.epot_elec * k, self.epot_pol_self * k, self.epot_pol_cross * k,
            self.epot_pol * k, (self.epot_pol + self.epot_elec) * k)


class FF_SASA_LCPO_GPU(ForcefieldBase):
    """LCPO surface area term (lcpo.cpp:640-961); forces recomputed every UpdateSasa steps."""

    name = "LCPO SASA (GPU)"
    flag = ffi.SA

    def __init__(self, wspace):
        super().__init__(wspace)
        self.ASPsection_name = ""
        self.GlobalASP = 0.0
        self.UpdateSasa = 5
        self.epot_cav = 0.0
        self.totalSASA = 0.0

    def setup(self):
        im = self.wspace.image
        if not im.has_sa:
            raise ffi.PDGPUError(-1, "the system image carries no LCPO parameters")
        if self.ASPsection_name:
            raise ffi.PDGPUError(-7, "per-type ASP sections are not supported; use GlobalASP")
        self.needsetup = False

    def sigma(self):
        # FF_SASA_LCPO::setup, lcpo.cpp:57-63: sigma = GlobalASP / Na / J2kcal (J / A^2)
        return np.full(self.wspace.nAtoms(), self.GlobalASP / 6.0221418E23 * 4184.0)

    def distribute(self, e, energies_only=False):
        ene = self.wspace.ene
        ene.epot += e["surf"]
        ene.epot_surf += e["surf"]
        self.epot_cav = self.epot = e["surf"]

    def infoLineHeader(self):
        return "\t%6s" % "Esurf"

    def infoLine(self):
        return "\t%6.1f" % (self.epot_cav * _J2KCALMOL)


class FF_Bonded_GPU(ForcefieldBase):
    """Bonds, angles, torsions, impropers (ffbonded.cpp:869-884)."""

    name = "Bonded Forcefield (GPU)"
    flag = ffi.BONDED

    def distribute(self, e, energies_only=False):
        ene = self.wspace.ene
        ene.epot_bond += e["bond"]
        ene.epot_angle += e["angle"]
        ene.epot_torsion += e["torsion"] + e["improper"]
        ene.epot += e["bond"] + e["angle"] + e["torsion"] + e["improper"]
        self.epot = e["bond"] + e["angle"] + e["torsion"] + e["improper"]


class Forcefield:
    """Container of components sharing one WorkSpace (forcefield.cpp:167-264).

    One GPU evaluation serves every added component: their flags are OR-ed into
    a single pdgpu_compute call and each component then takes its share of the
    energies, so the device works through one list build and one force pass.
    """

    def __init__(self, wspace):
        self.wspace = wspace
        self.components = []
        self.max_force = -1.0

    def add(self, component):
        if component.wspace is not self.wspace:
            raise RuntimeError("This forcefield was initialised with a different workspace")
        self.components.append(component)

    addWithOwnership = add

    def ensuresetup(self):
        for c in self.components:
            c.ensuresetup()

    def _prepare(self):
        ws = self.wspace
        self.ensuresetup()
        ctx = ws.context()
        key = tuple((type(c).__name__, c.calcCheckSum()) for c in self.components) + (ws.Padding,)
        if ws._ctx_params != key:
            for c in self.components:
                c.configure(ctx)
            ctx.set_list(ws.Padding)
            sa = [c for c in self.components if isinstance(c, FF_SASA_LCPO_GPU)]
            if sa:
                im = ws.image
                im_sigma = sa[0].sigma()
                if im.lcpo_sigma is None or not np.array_equal(im.lcpo_sigma, im_sigma):
                    # GlobalASP changed: the per-atom sigma is part of the static description
                    im.lcpo_sigma = im_sigma
                    ws.close()
                    ctx = ws.context()
                    for c in self.components:
                        c.configure(ctx)
                    ctx.set_list(ws.Padding)
            ws._ctx_params = key
        return ctx

    def calcForces(self, zero=True, energies_only=False):
        """Forcefield::calcForces: zero, evaluate every component, apply max_force, NaN check.
        energies_only: Forcefield::calcEnergies (no forces; a GB component forms its
        energies as FF_GeneralizedBorn_Still::calcEnergies does, gbff.cpp:178-183)."""
        ws = self.wspace
        if zero:
            ws.zeroForces()
        ctx = self._prepare()
        what = 0
        for c in self.components:
            if c.Active:
                what |= c.flag
        ctx.set_positions(ws.cur.p)
        if energies_only and (what & ffi.GB):
            what |= ffi.PD_ENERGIES
        energies = ctx.compute(what, None if energies_only else ws.cur.f)
        ws.per_system_energies = energies
        tot = {k: sum(e[k] for e in energies) for k in energies[0]}
        for c in self.components:
            if c.Active:
                c.distribute(tot, energies_only)
        if self.max_force > 0:
            mag = np.linalg.norm(ws.cur.f, axis=1)
            big = mag > self.max_force
            ws.cur.f[big] *= (self.max_force / mag[big])[:, None]
        if not (np.isfinite(ws.ene.epot_vdw) and np.isfinite(ws.ene.epot_elec)):
            ws.ene.epot = float("nan")

    def calcEnergies(self):
        """Forcefield::calcEnergies.  When FF_NonBonded with UsePartialRecalc is the
        only active component (PD's Monte Carlo set-up), energies after a move come
        from the pairs of the moved atoms only (pdgpu_nb_energy_update); the first
        call, and the first after a parameter or cutoff change, is a full one."""
        act = [c for c in self.components if c.Active]
        if len(act) == 1 and isinstance(act[0], FF_NonBonded_GPU) and act[0].UsePartialRecalc:
            ws = self.wspace
            ctx = self._prepare()
            ctx.set_positions(ws.cur.p)
            key = ws._ctx_params
            if getattr(self, "_mc_key", None) != key:
                energies = ctx.nb_energy_full()
                self._mc_key = key
            else:
                energies, _ = ctx.nb_energy_update()
            ws.zeroForces()
            ws.per_system_energies = energies
            act[0].distribute({k: sum(e[k] for e in energies) for k in energies[0]}, True)
            return
        self.calcForces(energies_only=True)

    def printEnergySummary(self):
        self.calcForces()
        k = _J2KCALMOL
        e = self.wspace.ene
        print(" -----------------------------------")
        for c in self.components:
            print(" %-28s %12.3f kcal/mol" % (c.name, c.epot * k))
        print(" Total energy: %10.3f kcal/mol" % (e.epot * k))

    def info(self):
        for c in self.components:
            c.info()
