"""PD's side of the boundary on the GPU, by replay.

tests/golden/plugin_peptide.npz holds every call the PD components of
pd_gb300/pd_plugin/ff_gpu.h (FF_GeneralizedBorn_Still_GPU, FF_SASA_LCPO_GPU,
FF_NonBonded_GPU) made through the C ABI while they ran inside PD on a
PD-built peptide (tests/golden/make_plugin_golden.py): the system
descriptions they gathered from PD's WorkSpace, the parameters they set, the
positions, and each call's result from the FP64 test double, which
reproduces PD's own components to 1e-12 (plugin_check verifies that, and
tests/test_pd_plugin.py runs it).  Here the same calls go to the real
library; energies must agree to |dE|/|E| <= 1e-6 per component and forces to
relative RMS <= 1e-5, so the components on the GPU reproduce PD's.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms

pytestmark = pytest.mark.gpu

NB_KEYS = ("Cutoff", "InnerCutoff", "VdwCutoff", "VdwInnerCutoff", "Vdw14Scaling", "Elec14Scaling", "Dielectric",
           "EnergySwitch", "ForceSwitch", "DoVdw", "DoElec")
GB_KEYS = ("Cutoff", "InnerCutoff", "VdwCutoff", "VdwInnerCutoff", "Vdw14Scaling", "Elec14Scaling",
           "DielectricSolute", "DielectricSolvent", "GbsaStillCutoff", "ExpApproxThreshold", "BornRadiusOffset", "P4",
           "P5")
ENE = ("epot", "vdw", "elec", "pol", "pol_self", "pol_cross", "surf", "virial")


def _nb(v):
    return {k: (int(x) if k in ("EnergySwitch", "ForceSwitch", "DoVdw", "DoElec") else float(x))
            for k, x in zip(NB_KEYS, v)}


def _contexts(d):
    return sorted({int(k.split("_")[0][3:]) for k in d}, key=int)


def test_pd_components_calls_replayed_on_the_gpu():
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    d = dict(np.load(os.path.join(GOLDEN, "plugin_peptide.npz")))
    checked = 0
    for c in _contexts(d):
        g = lambda k: d.get("ctx%d_%s" % (c, k))
        n = len(g("charge"))
        excl = g("excl") if g("excl") is not None else np.zeros((0, 3), np.int32)
        im = SystemImage([n], g("box"), g("charge"), g("radius"), g("epsilon"), g("mass"), excl,
                         gb_radius=g("gb_radius"), gb_vj=g("gb_vj"), gb_terms123=g("gb_terms123"),
                         lcpo_radius=g("lcpo_radius"), lcpo_p=g("lcpo_p"), lcpo_sigma=g("lcpo_sigma"),
                         lcpo_use=g("lcpo_use"), pos=g("pos"))
        ctx = DeviceContext(im)
        lp = g("list_params")
        ctx.set_list(float(lp[0]), bool(lp[1]))
        if g("nb_params") is not None:
            ctx.set_nb(**_nb(g("nb_params")))
        if g("gb_params") is not None:
            ctx.set_gb(**{k: float(x) for k, x in zip(GB_KEYS, g("gb_params"))})
        if g("gb_fast") is not None:
            ctx.set_gb_mode(int(g("gb_fast")[0]), **_nb(g("gb_vacuum")))
        ctx.set_positions(g("pos"))
        k = 0
        while g("call%d_what" % k) is not None:
            what = int(g("call%d_what" % k)[0])
            ref_e, ref_f = g("call%d_ene" % k), g("call%d_f" % k)
            f = np.zeros((n, 3))
            e = ctx.compute(what, f)[0]
            for i, key in enumerate(ENE):
                if abs(ref_e[i]) > 0:
                    assert abs(e[key] - ref_e[i]) <= 1e-6 * abs(ref_e[i]) + (1e-5 * abs(ref_e[i]) if key == "virial"
                                                                            else 0.0), (c, k, what, key)
            assert rel_rms(f, ref_f) <= 1e-5, (c, k, what)
            checked += 1
            k += 1
        ctx.close()
    assert checked >= 6
