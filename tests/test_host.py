"""Host-side logic: workload images, batching, the PD-interface mirror (no GPU)."""
import numpy as np
import pytest

from conftest import golden


@pytest.mark.parametrize("name,natom,nsys", [("c1_water", 2001, 1), ("c2_solvated", 22489, 1),
                                             ("c3_gb256", 4235, 1), ("c4_remd64", 209991, 64)])
def test_workload_images_load(name, natom, nsys):
    from pd_gb300.workspace import load_workload
    im = load_workload(name)
    assert im.natom == natom and im.nsystems == nsys
    assert np.all(np.isfinite(im.pos)) and np.all(im.mass > 0)
    sys_of = np.repeat(np.arange(nsys), im.natoms)
    # bonded pairs and terms never cross systems and name valid atoms
    assert np.all(sys_of[im.excl[:, 0]] == sys_of[im.excl[:, 1]])
    for idx, par in (im.bonds, im.angles, im.torsions, im.impropers):
        ncol = {2: 2, 3: 3, 5: 4}[idx.shape[1]]
        assert idx.shape[0] == par.shape[0]
        if len(idx):
            assert idx[:, :ncol].min() >= 0 and idx[:, :ncol].max() < natom
            assert np.all(sys_of[idx[:, 0]][:, None] == sys_of[idx[:, :ncol]])
    if nsys == 64:
        assert 400 < im.natoms.min() and im.natoms.max() < 9000
        assert im.has_gb and im.has_sa and not im.periodic


def test_concat_and_subset_roundtrip():
    from pd_gb300.workspace import SystemImage
    a = SystemImage._from_fixture(golden("peptide30"))
    b = SystemImage._from_fixture(golden("peptide120"))
    cat = SystemImage.concat([a, b, a])
    assert cat.nsystems == 3 and cat.natom == 2 * a.natom + b.natom
    for k, ref in enumerate([a, b, a]):
        sub = cat.subset(k)
        assert np.array_equal(sub.pos, ref.pos) and np.array_equal(sub.excl, ref.excl)
        for t in ("bonds", "angles", "torsions", "impropers"):
            assert np.array_equal(getattr(sub, t)[0], getattr(ref, t)[0])
            assert np.array_equal(getattr(sub, t)[1], getattr(ref, t)[1])


def test_replicate_tiles_a_periodic_box():
    """SystemImage.replicate (the replicated C2 boxes of the list-scaling
    measurement): copies shifted by whole box edges, indices re-based, one
    system in the enlarged box."""
    from pd_gb300.workspace import SystemImage
    w = SystemImage._from_fixture(golden("water_c1"))
    r = w.replicate((2, 1, 3))
    n = w.natom
    assert r.nsystems == 1 and r.natom == 6 * n
    assert np.allclose(r.box[0], w.box[0] * np.array([2, 1, 3]))
    L = w.box[0]
    for c in range(6):
        i, k = divmod(c, 3)
        assert np.allclose(r.pos[c * n:(c + 1) * n] - w.pos, L * np.array([i, 0, k]))
    assert len(r.excl) == 6 * len(w.excl) and r.excl[:, :2].max() < 6 * n
    assert np.array_equal(r.excl[len(w.excl):2 * len(w.excl), :2], w.excl[:, :2] + n)
    assert np.array_equal(r.charge, np.tile(w.charge, 6))
    with pytest.raises(ValueError):
        SystemImage.concat([w, w]).replicate((2, 1, 1))


def test_forcefield_defaults_mirror_pd():
    """Constructor defaults of the components equal PD's (nonbonded.cpp:985-1021, gbff.cpp:33-55, lcpo.h)."""
    import pd_gb300 as pdg
    ws = pdg.WorkSpace(pdg.SystemImage._from_fixture(golden("peptide30")))
    nb = pdg.FF_NonBonded_GPU(ws)
    assert (nb.Cutoff, nb.InnerCutoff, nb.VdwCutoff, nb.VdwInnerCutoff) == (15, 12, 15, 12)
    assert nb.ForceSwitch and not nb.EnergySwitch and nb.AutoScaling14
    gb = pdg.FF_GeneralizedBorn_Still_GPU(ws)
    assert gb.EnergySwitch and not gb.ForceSwitch and gb.FastMode
    assert (gb.DielectricSolvent, gb.DielectricSolute, gb.GbsaStillCutoff, gb.ExpApproxThreshold) == (80, 1, 10, -4)
    sa = pdg.FF_SASA_LCPO_GPU(ws)
    assert sa.UpdateSasa == 5 and sa.GlobalASP == 0
    nb.setup()
    assert (nb.Vdw14Scaling, nb.Elec14Scaling) == (0.5, 0.83333)
    assert ws.Padding == 0.5


def test_vdw_correction_follows_pd():
    """FF_NonBonded's VdwCor (nonbonded.cpp:862-874): off by default; when on, every atom of
    the pair loop adds -1/2 rho eps/(J2kcal Na) (8/3) pi R^6 / Rc^3 to epot, epot_vdw and
    epot_vdw_att.  GB reaches it only through FF_NonBonded (FastMode off, calcEnergies)."""
    import pd_gb300 as pdg
    ws = pdg.WorkSpace(pdg.SystemImage._from_fixture(golden("peptide30")))
    nb = pdg.FF_NonBonded_GPU(ws)
    assert not nb.VdwCor and nb.vdw_correction() == 0.0
    nb.VdwCor, nb.VdwCorDensity, nb.VdwCorEpsilon, nb.VdwCorRadius, nb.VdwCorCutoff = True, 0.0334, 0.152, 1.7682, 12.0
    j2kcal, na = 1.0 / 4184.0, 6.0221418E23
    per_atom = (-0.5 * 0.0334 * 0.152 / (j2kcal * na) * (8.0 / 3.0) * np.pi * 1.7682 ** 2 * 1.7682 ** 2 *
                1.7682 ** 2 / 12.0 ** 3)
    assert nb.vdw_correction() == pytest.approx(ws.nAtoms() * per_atom, rel=1e-14)
    e = {"vdw": -1.0e-19, "elec": -2.0e-19, "virial": 0.0}
    ws.ene.zero()
    nb.distribute(e)
    cor = nb.vdw_correction()
    assert ws.ene.epot_vdw == pytest.approx(e["vdw"] + cor, rel=1e-14)
    assert ws.ene.epot == pytest.approx(e["vdw"] + cor + e["elec"], rel=1e-14)
    assert ws.ene.epot_vdw_att == pytest.approx(cor, rel=1e-14)
    gb = pdg.FF_GeneralizedBorn_Still_GPU(ws)
    gb.VdwCor, gb.VdwCorDensity, gb.VdwCorEpsilon, gb.VdwCorRadius, gb.VdwCorCutoff = True, 0.0334, 0.152, 1.7682, 12.0
    g = dict(e, pol=0.0, pol_cross=0.0, pol_self=0.0)
    ws.ene.zero()
    gb.distribute(g)                         # FastMode forces: the fused loop has no correction
    assert ws.ene.epot_vdw == e["vdw"]
    ws.ene.zero()
    gb.distribute(g, energies_only=True)     # calcEnergies goes through FF_NonBonded
    assert ws.ene.epot_vdw == pytest.approx(e["vdw"] + cor, rel=1e-14)


def test_maxwell_boltzmann_hits_target_temperature():
    from pd_gb300.md import KB, maxwell_boltzmann
    m = np.full(3000, 2e-26)
    v = maxwell_boltzmann(m, [300.0, 450.0], 1, [1000, 2000])
    for sl, T in ((slice(0, 1000), 300.0), (slice(1000, 3000), 450.0)):
        ke = 0.5 * (m[sl, None] * v[sl] ** 2).sum()
        assert abs(2 * ke / (3 * (sl.stop - sl.start) * KB) - T) < 1e-9 * T


def test_geometric_ladder():
    from pd_gb300.md import REX_Local
    t = REX_Local.geometric_ladder(300.0, 500.0, 64)
    assert t[0] == 300.0 and abs(t[-1] - 500.0) < 1e-9
    assert np.allclose(t[1:] / t[:-1], (500 / 300.) ** (1 / 63))
