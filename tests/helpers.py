"""Shared helpers: build oracle inputs from a golden fixture."""
import numpy as np

from oracle import pdoracle as O


def oracle_system(d):
    return O.OracleSystem(d["pos"], d["charge"], d["radius"], d["epsilon"], d["excl"], tuple(d["box"]))


def list_cutoff(d):
    return float(d["cfg_list_cutoff"][0]) + float(d["cfg_padding"][0])


def nb_params(d, tag="nb"):
    g = lambda k: float(d["%s_%s" % (tag, k)][0])
    return O.nb_params(Cutoff=g("Cutoff"), InnerCutoff=g("InnerCutoff"), VdwCutoff=g("VdwCutoff"),
                       VdwInnerCutoff=g("VdwInnerCutoff"), Vdw14Scaling=g("Vdw14Scaling"),
                       Elec14Scaling=g("Elec14Scaling"), Dielectric=g("Dielectric"),
                       EnergySwitch=int(g("EnergySwitch")), ForceSwitch=int(g("ForceSwitch")),
                       ListCutoff=list_cutoff(d))


def gb_params(d):
    g = lambda k: float(d["gb_%s" % k][0])
    P = d["gb_P"]
    return O.gb_params(Cutoff=g("Cutoff"), InnerCutoff=g("InnerCutoff"), VdwCutoff=g("VdwCutoff"),
                       VdwInnerCutoff=g("VdwInnerCutoff"), Vdw14Scaling=g("Vdw14Scaling"),
                       Elec14Scaling=g("Elec14Scaling"), DielectricSolute=g("DielectricSolute"),
                       DielectricSolvent=g("DielectricSolvent"), GbsaStillCutoff=g("GbsaStillCutoff"),
                       ExpApproxThreshold=g("ExpApproxThreshold"), DielectricOffset=g("DielectricOffset"),
                       BornRadiusOffset=g("BornRadiusOffset"), P1=P[0], P2=P[1], P3=P[2], P4=P[3], P5=P[4],
                       ListCutoff=list_cutoff(d))


def nb_kwargs(d, tag="nb"):
    """FF_NonBonded attribute values stored in a fixture."""
    g = lambda k: float(d["%s_%s" % (tag, k)][0])
    return dict(Cutoff=g("Cutoff"), InnerCutoff=g("InnerCutoff"), VdwCutoff=g("VdwCutoff"),
                VdwInnerCutoff=g("VdwInnerCutoff"), Vdw14Scaling=g("Vdw14Scaling"), Elec14Scaling=g("Elec14Scaling"),
                Dielectric=g("Dielectric"), EnergySwitch=int(g("EnergySwitch")), ForceSwitch=int(g("ForceSwitch")),
                DoVdw=1, DoElec=1)


def gb_kwargs(d):
    g = lambda k: float(d["gb_%s" % k][0])
    return dict(Cutoff=g("Cutoff"), InnerCutoff=g("InnerCutoff"), VdwCutoff=g("VdwCutoff"),
                VdwInnerCutoff=g("VdwInnerCutoff"), Vdw14Scaling=g("Vdw14Scaling"),
                Elec14Scaling=g("Elec14Scaling"), DielectricSolute=g("DielectricSolute"),
                DielectricSolvent=g("DielectricSolvent"), GbsaStillCutoff=g("GbsaStillCutoff"),
                ExpApproxThreshold=g("ExpApproxThreshold"), BornRadiusOffset=g("BornRadiusOffset"),
                P4=float(d["gb_P"][3]), P5=float(d["gb_P"][4]))


ENE_INDEX = {"epot": 0, "vdw": 1, "elec": 2, "pol": 3, "pol_self": 4, "pol_cross": 5, "surf": 6, "virial": 7}


def ref_energy(d, tag, key):
    return float(d["%s_ene" % tag][ENE_INDEX[key]])
