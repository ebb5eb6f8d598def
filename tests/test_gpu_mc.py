"""Monte Carlo energies: FF_NonBonded partial recalculation after small moves
(nonbonded.cpp:76-386, 1154-1182) against full evaluations and the oracle.

Update vs full evaluation: 1e-7 relative (both are FP64 pair sums entered into
2^-24 kcal/mol fixed point, the full one per tile, so they differ by that
rounding; water's electrostatics cancel about 5000-fold).  Against the oracle:
the 1e-6 energy bar of the parity tests."""
import numpy as np
import pytest

from conftest import rel_err
from helpers import nb_kwargs, nb_params, oracle_system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,tag", [("water_c1", "nb"), ("water_c1", "nbfswitch"), ("peptide30", "nb")])
def test_partial_update_matches_full_evaluation(goldens, name, tag):
    from oracle import pdoracle as O
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    d = goldens[name]
    ctx = DeviceContext(SystemImage._from_fixture(d))
    ctx.set_list(float(d["cfg_padding"][0]))
    ctx.set_nb(**nb_kwargs(d, tag))
    pos = d["pos"].copy()
    ctx.set_positions(pos)
    e0 = ctx.nb_energy_full()[0]
    ef = ctx.compute(ffi.NB)[0]
    assert e0["vdw"] == ef["vdw"] and e0["elec"] == ef["elec"]
    rng = np.random.default_rng(4)
    for move in range(3):
        moved = rng.choice(len(pos), 3 + move, replace=False)
        pos[moved] += rng.normal(0.0, 0.15, (len(moved), 3))
        ctx.set_positions(pos)
        e1, n = ctx.nb_energy_update()
        assert n == len(moved)
        full = ctx.compute(ffi.NB)[0]
        for k in ("vdw", "elec"):
            assert rel_err(e1[0][k], full[k]) <= 1e-7, (k, e1[0][k], full[k])
        ref, _ = O.nonbonded(O.OracleSystem(pos, d["charge"], d["radius"], d["epsilon"], d["excl"], tuple(d["box"])),
                             nb_params(d, tag))
        assert rel_err(e1[0]["epot"], ref[0]) <= 1e-6
    e2, n = ctx.nb_energy_update()
    assert n == 0 and e2[0]["epot"] == e1[0]["epot"]


def test_forcefield_calc_energies_uses_partial_recalc(goldens):
    from pd_gb300.forcefield import FF_NonBonded_GPU, Forcefield
    from pd_gb300.workspace import SystemImage, WorkSpace
    d = goldens["water_c1"]
    ws = WorkSpace(SystemImage._from_fixture(d))
    ws.Padding = 2.0
    ff = Forcefield(ws)
    nb = FF_NonBonded_GPU(ws)
    for k, v in nb_kwargs(d, "nb").items():
        setattr(nb, k, v)
    nb.AutoScaling14 = False
    nb.UsePartialRecalc = True
    ff.add(nb)
    ff.calcEnergies()
    e0 = ws.ene.epot
    ws.cur.p[10] += 0.1
    ff.calcEnergies()                    # partial
    e1 = ws.ene.epot
    nb.UsePartialRecalc = False
    ff.calcEnergies()                    # full evaluation of the same positions
    assert e1 != e0 and rel_err(e1, ws.ene.epot) <= 1e-7
