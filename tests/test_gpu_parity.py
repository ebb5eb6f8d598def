"""CUDA path (through the C ABI) against the oracle and PD's own FP64 outputs.

Tolerances (FP32 pair math, 64-bit fixed-point accumulation vs FP64):
  energies  |dE| / |E| <= 1e-6
  forces    sqrt(mean |dF|^2) / sqrt(mean |F|^2) <= 1e-5
"""
import numpy as np
import pytest

from conftest import rel_err, rel_rms
from helpers import gb_kwargs, gb_params, list_cutoff, nb_kwargs, nb_params, oracle_system, ref_energy

pytestmark = pytest.mark.gpu

E_TOL = 1e-6
F_TOL = 1e-5


def make_ctx(d, padding=None):
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    im = SystemImage._from_fixture(d)
    ctx = DeviceContext(im)
    ctx.set_list(float(d["cfg_padding"][0]) if padding is None else padding)
    ctx.set_positions(d["pos"])
    return ctx


NB_CASES = [("water_c1", "nb"), ("water_c1", "nbfswitch"), ("water_c1", "nbnormal"), ("water_c1", "nbvdwsplit"),
            ("peptide30", "nb"), ("peptide30_ap", "nb"), ("peptide120", "nb")]


@pytest.mark.parametrize("name,tag", NB_CASES)
def test_nb_matches_pd(goldens, name, tag):
    from pd_gb300 import ffi
    d = goldens[name]
    ctx = make_ctx(d)
    ctx.set_nb(**nb_kwargs(d, tag))
    f = np.zeros((len(d["pos"]), 3))
    e = ctx.compute(ffi.NB, f)[0]
    ref_f = d[tag + "_f"]
    for k in ("vdw", "elec", "epot"):
        assert rel_err(e[k], ref_energy(d, tag, k)) <= E_TOL, (k, e[k], ref_energy(d, tag, k))
    assert rel_err(e["virial"], ref_energy(d, tag, "virial")) <= 1e-5
    assert rel_rms(f, ref_f) <= F_TOL


@pytest.mark.parametrize("name", ["peptide30", "peptide30_ap", "peptide120"])
def test_gb_matches_pd(goldens, name):
    from pd_gb300 import ffi
    d = goldens[name]
    ctx = make_ctx(d)
    ctx.set_gb(**gb_kwargs(d))
    f = np.zeros((len(d["pos"]), 3))
    e = ctx.compute(ffi.GB, f)[0]
    born = ctx.born_radii()
    assert np.max(np.abs(born / d["gb_born"] - 1)) < 1e-6
    for k in ("vdw", "elec", "pol", "pol_self", "pol_cross", "epot"):
        assert rel_err(e[k], ref_energy(d, "gb", k)) <= E_TOL, (k, e[k], ref_energy(d, "gb", k))
    assert rel_rms(f, d["gb_f"]) <= F_TOL


@pytest.mark.parametrize("name", ["peptide30_ap", "peptide120"])
def test_gb_work_item_sizes_agree(goldens, name):
    """Single tiles and tile pairs as GB work items (pdgpu_set_work_items) give
    the same energies and forces to FP32 rounding of the per-item sums, all
    PD's: the energy evaluation and the force-only evaluation the dynamics step
    runs (its own bodies for all-inside tile pairs)."""
    torch = pytest.importorskip("torch")
    from pd_gb300 import ffi
    d = goldens[name]
    n = len(d["pos"])
    out = {}
    for tiles in (1, 2):
        ctx = make_ctx(d)
        ctx.set_gb(**gb_kwargs(d))
        ctx.set_work_items(tiles)
        assert ctx.work_items() == tiles
        f = np.zeros((n, 3))
        e = ctx.compute(ffi.GB, f)[0]
        fd = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        ctx.compute_device(ffi.GB, fd.data_ptr())
        ctx.synchronize()
        out[tiles] = (e, f, fd.cpu().numpy())
        ctx.close()
    e1, f1, _ = out[1]
    for tiles in (1, 2):
        e, f, ff = out[tiles]
        assert rel_rms(f, f1) <= 1e-6 and rel_rms(ff, f1) <= 1e-6
        for k in ("vdw", "elec", "pol", "epot"):
            assert rel_err(e[k], e1[k]) <= 1e-7, (tiles, k, e1[k], e[k])
            assert rel_err(e[k], ref_energy(d, "gb", k)) <= E_TOL
        assert rel_rms(f, d["gb_f"]) <= F_TOL and rel_rms(ff, d["gb_f"]) <= F_TOL


@pytest.mark.parametrize("name,tag", [("peptide120", "nb"), ("peptide30_ap", "nb"), ("water_c1", "nb"),
                                      ("water_c1", "nbfswitch")])
def test_nb_groups_match_pd(goldens, name, tag):
    """LJ/Coulomb j-atom groups (pdgpu_set_nb_groups): the force-only kernel (the
    one dynamics runs) and the energy kernel, groups on and off, against PD's
    forces and energies and against each other."""
    torch = pytest.importorskip("torch")
    from pd_gb300 import ffi
    d = goldens[name]
    n = len(d["pos"])
    out = {}
    for on in (1, 0):
        ctx = make_ctx(d)
        ctx.set_nb(**nb_kwargs(d, tag))
        ctx.set_nb_groups(on)
        f = np.zeros((n, 3))
        e = ctx.compute(ffi.NB, f)[0]
        setting, ngroups, nrest = ctx.nb_groups()
        assert setting == bool(on)
        if on and name.startswith("peptide"):
            assert ngroups > 0 and nrest >= 0
        if not on:
            assert ngroups == 0
        fd = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        ctx.compute_device(ffi.NB, fd.data_ptr())
        ctx.synchronize()
        out[on] = (e, f, fd.cpu().numpy())
        ctx.close()
    ref_f = d[tag + "_f"]
    for on in (1, 0):
        e, f, ff = out[on]
        for k in ("vdw", "elec", "epot"):
            assert rel_err(e[k], ref_energy(d, tag, k)) <= E_TOL, (on, k, e[k], ref_energy(d, tag, k))
        assert rel_rms(f, ref_f) <= F_TOL
        assert rel_rms(ff, ref_f) <= F_TOL
    assert rel_rms(out[1][2], out[0][2]) <= 1e-6
    assert rel_rms(out[1][1], out[0][1]) <= 1e-6


def test_nb_groups_keep_the_displacement_check(goldens):
    """With the groups on, a move beyond half the skin is reported as a stale list
    even in open space where every block pair is a tile (the groups drop j atoms
    beyond the list radius); with them off such a list cannot go stale."""
    from pd_gb300 import ffi
    d = goldens["peptide30"]
    pos = np.array(d["pos"], dtype=np.float64)
    for on in (1, 0):
        ctx = make_ctx(d, padding=1.0)
        ctx.set_nb(**nb_kwargs(d, "nb"))
        ctx.set_nb_groups(on)
        ctx.compute(ffi.NB, np.zeros((len(pos), 3)))
        ntiles = ctx.list_stats()["tiles"]
        nb = (len(pos) + 31) // 32
        moved = pos.copy()
        moved[0] += np.array([0.8, 0.0, 0.0])
        ctx.set_positions(moved)
        if on:
            with pytest.raises(ffi.PDGPUError) as ex:
                ctx.compute(ffi.NB, np.zeros((len(pos), 3)))
            assert ex.value.status == ffi.ERR_STALE_LIST
        elif ntiles == nb * (nb + 1) // 2:
            ctx.compute(ffi.NB, np.zeros((len(pos), 3)))
        ctx.close()


@pytest.mark.parametrize("name", ["peptide30", "peptide120"])
def test_lcpo_matches_pd(goldens, name):
    from pd_gb300 import ffi
    d = goldens[name]
    ctx = make_ctx(d)
    ctx.set_gb(**gb_kwargs(d))   # list radius as in the fixture (GB + LCPO requests)
    f = np.zeros((len(d["pos"]), 3))
    e = ctx.compute(ffi.SA, f)[0]
    assert rel_err(e["surf"], ref_energy(d, "sasa", "surf")) <= E_TOL
    sa = ctx.sasa()
    assert np.max(np.abs(sa - d["lcpo_sasa"])) <= 1e-4 * max(1.0, np.max(d["lcpo_sasa"]))
    assert rel_rms(f, d["sasa_f"]) <= F_TOL


def _dense_lcpo_lattice(a=2.1, r=3.1, seed=4, n=10, gap=2e-3):
    """A jittered 10^3 lattice, 2.1 A apart, of atoms with LCPO radius 3.1 A:
    407 atoms overlap more than 80 others (up to 105; none beyond the 160
    candidates kept), so both an atom's own list and its partners' lists are
    cut at 80 as PD cuts them (lcpo.h:24).  Atoms are moved until no pair lies
    within `gap` of the overlap distance, where FP32 and FP64 could decide a
    pair differently."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    g = np.arange(n)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) * a
    pos = pos + rng.uniform(-0.15, 0.15, pos.shape)
    for _ in range(50):
        p = cKDTree(pos).query_pairs(2 * r + gap, output_type="ndarray")
        d = np.linalg.norm(pos[p[:, 0]] - pos[p[:, 1]], axis=1)
        bad = np.unique(p[np.abs(d - 2 * r) < gap][:, 1])
        if len(bad) == 0:
            return pos
        pos[bad] += rng.uniform(-0.15, 0.15, (len(bad), 3))
    raise RuntimeError("no lattice without near-boundary pairs")


def test_lcpo_cut_lists_match_oracle():
    """LCPO where lists are cut at 80 partners (PD's first 80 by atom index):
    the device against the oracle's FP64 restatement of lcpo.cpp on the same
    positions.  P2-P4 are positive here so no atom's SA is clamped at zero; a k
    counted past a cut list would move SA by ~1e-2 of it.  Tolerances: SA and
    the energy are sums of positive FP32 terms (1e-4 of the largest SA, 1e-5
    of the energy); the forces of the dense lattice are small differences of
    ~1e4 FP32 terms per atom (force relative RMS 1e-3)."""
    pytest.importorskip("scipy")
    from oracle import pdoracle as O
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    pos = _dense_lcpo_lattice()
    n = len(pos)
    P = np.array([0.5, 1e-3, 1e-3, 1e-5])
    sigma = 3.47e-23
    kw = dict(lcpo_radius=np.full(n, 3.1), lcpo_p=np.tile(P, (n, 1)), lcpo_sigma=np.full(n, sigma),
              lcpo_use=np.ones(n, np.int32))
    im = SystemImage([n], np.zeros(3), np.zeros(n), np.full(n, 1.5), np.zeros(n), np.full(n, 2e-26),
                     np.zeros((0, 3), np.int32), pos=pos, **kw)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_positions(pos)
    f = np.zeros((n, 3))
    e = ctx.compute(ffi.SA, f)[0]
    sa = ctx.sasa()
    ctx.close()
    s = O.OracleSystem(pos, np.zeros(n), np.full(n, 1.5), np.zeros(n), np.zeros((0, 3), np.int32))
    ref_e, ref_f, ref_sa = O.lcpo_forces(s, 2 * 3.1 + 2.0, np.full(n, 3.1), np.tile(P, (n, 1)), np.full(n, sigma),
                                         np.ones(n, np.int32))
    assert np.max(np.abs(sa - ref_sa)) <= 1e-4 * np.max(ref_sa)
    assert rel_err(e["surf"], ref_e[6]) <= 1e-5
    assert rel_rms(f, ref_f) <= 1e-3


@pytest.mark.parametrize("name", ["water_c1", "peptide30", "peptide120"])
def test_bonded_matches_pd(goldens, name):
    from pd_gb300 import ffi
    d = goldens[name]
    ctx = make_ctx(d)
    ctx.set_nb(**nb_kwargs(d, "nb"))
    f = np.zeros((len(d["pos"]), 3))
    e = ctx.compute(ffi.BONDED, f)[0]
    tot = e["bond"] + e["angle"] + e["torsion"] + e["improper"]
    kcal = 4184.0 / 6.0221418e23          # J per kcal/mol
    ref = ref_energy(d, "bonded", "epot")
    # near-equilibrium water has ~zero bonded energy and force: absolute floors of
    # 1e-4 kcal/mol and 1e-4 kcal/mol/A keep the relative criteria meaningful
    assert abs(tot - ref) <= E_TOL * abs(ref) + 1e-4 * kcal
    ref_f = d["bonded_f"]
    err = np.sqrt(((f - ref_f) ** 2).sum(1).mean())
    assert err <= F_TOL * np.sqrt((ref_f ** 2).sum(1).mean()) + 1e-4 * kcal * 1e10


def test_deterministic_and_forces_add(goldens):
    from pd_gb300 import ffi
    d = goldens["peptide120"]
    ctx = make_ctx(d)
    ctx.set_gb(**gb_kwargs(d))
    f1 = np.zeros((len(d["pos"]), 3))
    e1 = ctx.compute(ffi.GB | ffi.SA, f1)
    f2 = np.zeros((len(d["pos"]), 3))
    e2 = ctx.compute(ffi.GB | ffi.SA, f2)
    assert np.array_equal(f1, f2) and e1 == e2
    ctx.compute(ffi.GB | ffi.SA, f2)          # forces are ADDED, as PD components add into atom[i].f
    assert np.array_equal(f2, 2 * f1)


def test_batch_equals_separate_systems(goldens):
    """Several systems in one context give each system's own result (tiles never cross systems)."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    names = ["peptide30", "peptide120", "peptide30_ap"]
    ims = [SystemImage._from_fixture(goldens[n]) for n in names]
    batch = SystemImage.concat(ims)
    ctx = DeviceContext(batch)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(goldens["peptide30"]))
    ctx.set_positions(np.concatenate([goldens[n]["pos"] for n in names]))
    f = np.zeros((batch.natom, 3))
    eb = ctx.compute(ffi.GB, f)
    o = batch.offsets
    for k, n in enumerate(names):
        c1 = make_ctx(goldens[n])
        c1.set_gb(**gb_kwargs(goldens["peptide30"]))
        f1 = np.zeros((len(goldens[n]["pos"]), 3))
        e1 = c1.compute(ffi.GB, f1)[0]
        assert np.array_equal(f[o[k]:o[k + 1]], f1)
        assert eb[k] == e1


def test_stale_list_is_reported(goldens):
    from pd_gb300 import ffi
    d = goldens["water_c1"]
    ctx = make_ctx(d)
    ctx.set_nb(**nb_kwargs(d, "nb"))
    ctx.compute(ffi.NB)
    p = d["pos"].copy()
    p[0] += 1.5          # further than Padding/2 = 1 A
    ctx.set_positions(p)
    with pytest.raises(ffi.PDGPUError) as ei:
        ctx.compute(ffi.NB)
    assert ei.value.status == -8
    ctx.rebuild_list()
    ctx.compute(ffi.NB)


def test_nan_is_reported(goldens):
    from pd_gb300 import ffi
    d = goldens["peptide30"]
    ctx = make_ctx(d)
    ctx.set_nb(**nb_kwargs(d, "nb"))
    p = d["pos"].copy()
    p[5] = p[40]        # two non-bonded atoms on top of each other
    ctx.set_positions(p)
    ctx.rebuild_list()
    with pytest.raises(ffi.PDGPUError):
        ctx.compute(ffi.NB)


def test_forcefield_mirror_matches_pd(goldens):
    """PD-style use: WorkSpace + Forcefield.add(...) + calcForces, results in wspace.ene / cur.f."""
    import pd_gb300 as pdg
    d = goldens["peptide30"]
    ws = pdg.WorkSpace(pdg.SystemImage._from_fixture(d))
    ws.Padding = 2.0
    ff = pdg.Forcefield(ws)
    gb = pdg.FF_GeneralizedBorn_Still_GPU(ws)
    gb.Cutoff, gb.InnerCutoff = 12.0, 9.0
    gb.VdwCutoff, gb.VdwInnerCutoff = 12.0, 9.0
    sasa = pdg.FF_SASA_LCPO_GPU(ws)
    sasa.GlobalASP = 0.005
    ff.add(gb)
    ff.add(sasa)
    ff.calcForces()
    ref = ref_energy(d, "gb", "epot") + ref_energy(d, "sasa", "epot")
    assert rel_err(ws.ene.epot, ref) <= E_TOL
    assert rel_rms(ws.cur.f, d["gb_f"] + d["sasa_f"]) <= F_TOL
    assert rel_err(ws.ene.epot_pol, ref_energy(d, "gb", "pol")) <= E_TOL
    assert rel_err(ws.ene.epot_surf, ref_energy(d, "sasa", "surf")) <= E_TOL


@pytest.mark.parametrize("name", ["peptide30", "peptide30_ap", "peptide120"])
def test_gb_fastmode_off_matches_pd(goldens, name):
    """FastMode = false: FF_NonBonded::calcForces with the GB object's own settings
    plus calcBornForces (gbff.cpp:185-197, 1189-1437), against PD."""
    from pd_gb300 import ffi
    d = goldens[name]
    ctx = make_ctx(d)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_gb_mode(0, **nb_kwargs(d, "gb"))
    f = np.zeros((len(d["pos"]), 3))
    e = ctx.compute(ffi.GB, f)[0]
    ref = d["gbslow_ene"]
    assert rel_err(e["epot"], ref[0]) <= E_TOL and rel_err(e["vdw"], ref[1]) <= E_TOL
    assert rel_err(e["elec"], ref[2]) <= E_TOL
    assert rel_err(e["pol"], ref[0] - ref[1] - ref[2]) <= E_TOL     # PD keeps it in the component
    assert rel_rms(f, d["gbslow_f"]) <= F_TOL


@pytest.mark.parametrize("name", ["peptide30", "peptide120"])
def test_gb_pd_energies_match_calc_energies(goldens, name):
    """PDGPU_PD_ENERGIES: FF_GeneralizedBorn_Still::calcEnergies (calcBornEnergy,
    no ExpApproxThreshold, gbff.cpp:178-183, 537-596), with the GB object's
    default FF_NonBonded settings."""
    from pd_gb300 import ffi
    d = goldens[name]
    ctx = make_ctx(d)
    ctx.set_gb(**gb_kwargs(d))
    e = ctx.compute(ffi.GB | ffi.PD_ENERGIES)[0]
    ref = d["gbene_ene"]
    assert rel_err(e["epot"], ref[0]) <= E_TOL
    assert rel_err(e["vdw"], ref[1]) <= E_TOL and rel_err(e["elec"], ref[2]) <= E_TOL
    e_fast = ctx.compute(ffi.GB)[0]                  # the mode itself is unchanged
    assert rel_err(e_fast["epot"], d["gb_ene"][0]) <= E_TOL


def test_forcefield_mirror_gb_modes_match_pd(goldens):
    """PD-style use of the GB component: FastMode off through calcForces, and
    Forcefield.calcEnergies (FF_GeneralizedBorn_Still::calcEnergies)."""
    import pd_gb300 as pdg
    d = goldens["peptide30"]
    ws = pdg.WorkSpace(pdg.SystemImage._from_fixture(d))
    ws.Padding = 2.0
    ff = pdg.Forcefield(ws)
    gb = pdg.FF_GeneralizedBorn_Still_GPU(ws)
    gb.Cutoff, gb.InnerCutoff = 12.0, 9.0
    gb.VdwCutoff, gb.VdwInnerCutoff = 12.0, 9.0
    ff.add(gb)
    ff.calcEnergies()
    assert rel_err(ws.ene.epot, float(d["gbene_ene"][0])) <= E_TOL
    gb.FastMode = False
    ff.calcForces()
    assert rel_err(ws.ene.epot, float(d["gbslow_ene"][0])) <= E_TOL
    assert rel_rms(ws.cur.f, d["gbslow_f"]) <= F_TOL
