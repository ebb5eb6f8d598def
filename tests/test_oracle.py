"""The FP64 C restatement (oracle/) against PD's own outputs (tests/golden/)."""
import numpy as np
import pytest

from conftest import rel_err, rel_rms
from helpers import gb_params, list_cutoff, nb_params, oracle_system, ref_energy
from oracle import pdoracle as O

NB_TAGS = [("water_c1", "nb"), ("water_c1", "nbfswitch"), ("water_c1", "nbnormal"), ("water_c1", "nbvdwsplit"),
           ("peptide30", "nb"), ("peptide30_ap", "nb"), ("peptide120", "nb")]


@pytest.mark.parametrize("name,tag", NB_TAGS)
def test_nonbonded_matches_pd(goldens, name, tag):
    d = goldens[name]
    e, f = O.nonbonded(oracle_system(d), nb_params(d, tag))
    for i, k in enumerate(("epot", "vdw", "elec")):
        assert rel_err(e[i], ref_energy(d, tag, k)) < 1e-12
    assert rel_err(e[7], ref_energy(d, tag, "virial")) < 1e-12
    assert rel_rms(f, d[tag + "_f"]) < 1e-12


@pytest.mark.parametrize("name", ["water_c1", "peptide30", "peptide120"])
def test_list_checksums_match_pd(goldens, name):
    d = goldens[name]
    c, s1, s2 = O.list_checksums(oracle_system(d), list_cutoff(d))
    assert np.array_equal(c, d["nl_n"]) and np.array_equal(s1, d["nl_sumj"]) and np.array_equal(s2, d["nl_sumj2"])


@pytest.mark.parametrize("name", ["peptide30", "peptide30_ap", "peptide120"])
def test_gb_matches_pd(goldens, name):
    d = goldens[name]
    p = gb_params(d)
    vj, t = O.gb_fixed_terms(d["gb_radius"], d["cov12"], d["cov12d"], d["cov13"], d["cov13d"], p)
    assert np.max(np.abs(vj - d["gb_vj"])) <= 1e-12 * np.max(np.abs(d["gb_vj"]))
    assert np.max(np.abs(t - d["gb_terms123"])) <= 1e-12 * np.max(np.abs(d["gb_terms123"]))
    e, f, born = O.gb_forces(oracle_system(d), p, d["gb_radius"], d["gb_vj"], d["gb_terms123"])
    assert np.max(np.abs(born / d["gb_born"] - 1)) < 1e-12
    for i, k in enumerate(("epot", "vdw", "elec", "pol", "pol_self", "pol_cross")):
        assert rel_err(e[i], ref_energy(d, "gb", k)) < 1e-12, k
    assert rel_rms(f, d["gb_f"]) < 1e-12


@pytest.mark.parametrize("name", ["peptide30", "peptide120"])
def test_lcpo_matches_pd(goldens, name):
    d = goldens[name]
    e, f, sa = O.lcpo_forces(oracle_system(d), list_cutoff(d), d["lcpo_radius"], d["lcpo_P"], d["lcpo_sigma"],
                             d["lcpo_use"])
    assert rel_err(e[6], ref_energy(d, "sasa", "surf")) < 1e-12
    assert np.max(np.abs(sa - d["lcpo_sasa"])) < 1e-9
    assert rel_rms(f, d["sasa_f"]) < 1e-12


@pytest.mark.parametrize("name", ["water_c1", "peptide30", "peptide120"])
def test_bonded_matches_pd(goldens, name):
    d = goldens[name]
    ene, f = O.bonded(d["pos"], d["bond_idx"], d["bond_par"], d["angle_idx"], d["angle_par"], d["torsion_idx"],
                      d["torsion_par"], d["improper_idx"], d["improper_par"])
    assert rel_err(ene.sum(), ref_energy(d, "bonded", "epot")) < 1e-10
    assert rel_rms(f, d["bonded_f"]) < 1e-9


@pytest.mark.parametrize("mode", ["eswitch", "fswitch", "normal"])
def test_pair_law_scan(goldens, mode):
    """FF_NonBonded::calc_LJ_Coulomb_Force r-scan (nonbonded.cpp:400-534)."""
    scan = goldens["water_c1"]["scan_" + mode]
    p = O.nb_params(Cutoff=12, InnerCutoff=9, VdwCutoff=12, VdwInnerCutoff=9, EnergySwitch=int(mode == "eswitch"),
                    ForceSwitch=int(mode == "fswitch"))
    eps = 1.0 / (1 / 4184.0 * 6.0221418e23)
    for r, vp, vf, ep, ef in scan[::7]:
        got = O.pair_law(p, r, 3.0, eps, 1.0, 1.0)
        for g, ref in zip(got, (vp, vf, ep, ef)):
            assert abs(g - ref) <= 1e-12 * max(abs(ref), 1e-30) + 1e-300


def test_oracle_threads_agree(goldens):
    d = goldens["peptide120"]
    s = oracle_system(d)
    e1, f1, _ = O.gb_forces(s, gb_params(d), d["gb_radius"], d["gb_vj"], d["gb_terms123"], nthreads=1)
    e4, f4, _ = O.gb_forces(s, gb_params(d), d["gb_radius"], d["gb_vj"], d["gb_terms123"], nthreads=4)
    assert np.allclose(e1, e4, rtol=1e-12) and rel_rms(f4, f1) < 1e-12


def test_langevin_coefficients_branches():
    """Taylor branch (gamma*dt <= 0.05) and exponential branch agree near the switch point."""
    a = O.langevin_coeffs(1e13, 0.0499e-14)
    b = O.langevin_coeffs(1e13, 0.0501e-14)
    assert np.allclose(a[:3], b[:3], rtol=1e-2)


def test_stored_list_matches_direct_scan(goldens):
    """PD keeps the list between rebuilds (neighbourlist.cpp:336-439); evaluating a
    freshly built stored list equals the direct minimum-image scan."""
    d = goldens["water_c1"]
    s = oracle_system(d)
    p = nb_params(d)
    e1, f1 = O.nonbonded(s, p)
    L = O.StoredList(s, list_cutoff(d), 2)
    e2, f2 = O.nonbonded_list(s, L, p, 2)
    assert np.allclose(e1, e2, rtol=1e-11) and rel_rms(f2, f1) < 1e-12


@pytest.mark.parametrize("name", ["peptide30", "peptide30_ap", "peptide120"])
def test_gb_slow_mode_and_calc_energies_match_pd(goldens, name):
    """FastMode = false (FF_NonBonded::calcForces + calcBornForces, gbff.cpp:185-197,
    1189-1437) and calcEnergies (calcBornEnergy, no ExpApproxThreshold,
    gbff.cpp:178-183, 537-596) against PD's own outputs."""
    d = goldens[name]
    s = oracle_system(d)
    p = gb_params(d)
    p.FastMode = 0
    e, f, _ = O.gb_forces(s, p, d["gb_radius"], d["gb_vj"], d["gb_terms123"])
    en, fn = O.nonbonded(s, nb_params(d, "gb"))     # the GB object's own FF_NonBonded settings
    ref = d["gbslow_ene"]
    assert abs(e[0] + en[0] - ref[0]) <= 1e-12 * abs(ref[0])
    assert abs(en[1] - ref[1]) <= 1e-12 * abs(ref[1]) and abs(en[2] - ref[2]) <= 1e-12 * abs(ref[2])
    rf = d["gbslow_f"]
    assert np.sqrt(((f + fn - rf) ** 2).sum(1).mean() / (rf ** 2).sum(1).mean()) <= 1e-12
    p.ExpApproxThreshold = -1e300
    e2, _, _ = O.gb_forces(s, p, d["gb_radius"], d["gb_vj"], d["gb_terms123"])
    assert abs(e2[0] + en[0] - d["gbene_ene"][0]) <= 1e-12 * abs(d["gbene_ene"][0])


def _cfg_system(name):
    """A workload image (or one of its systems) with the PD outputs for it."""
    import hashlib

    from conftest import golden
    from pd_gb300.workspace import load_workload
    d = golden(name)
    im = load_workload(str(d["image"]))
    k = int(d["system"][0])
    sub = im if k < 0 else im.subset(k)
    h = hashlib.sha256(np.ascontiguousarray(sub.pos, dtype=np.float32).tobytes()).hexdigest()
    assert h == str(d["pos_sha256"])
    s = O.OracleSystem(sub.pos, sub.charge, sub.radius, sub.epsilon, sub.excl, tuple(sub.box[0]))
    return d, sub, s


def test_oracle_matches_pd_on_the_solvated_workload():
    """The 22,489-atom periodic C2 box (solute + water): PD's forces are stored as
    float32 (relative rounding 6e-8), energies in FP64."""
    d, sub, s = _cfg_system("cfg_c2")
    e, f = O.nonbonded(s, nb_params(d), nthreads=8)
    for i, k in enumerate(("epot", "vdw", "elec")):
        assert rel_err(e[i], ref_energy(d, "nb", k)) < 1e-12
    assert rel_rms(f, d["nb_f"]) < 1e-7


@pytest.mark.parametrize("name", ["cfg_c3", "cfg_c4_small", "cfg_c4_large"])
def test_oracle_matches_pd_on_the_gb_workloads(name):
    """Energies to 1e-11: over the 30 M pairs of the largest peptide the threaded
    oracle and PD's sequential loop sum in different orders."""
    d, sub, s = _cfg_system(name)
    e, f, born = O.gb_forces(s, gb_params(d), sub.gb_radius, sub.gb_vj, sub.gb_terms123, nthreads=8)
    assert np.max(np.abs(born / d["gb_born"] - 1)) < 1e-6
    for i, k in enumerate(("epot", "vdw", "elec", "pol", "pol_self", "pol_cross")):
        assert rel_err(e[i], ref_energy(d, "gb", k)) < 1e-11, k
    assert rel_rms(f, d["gb_f"]) < 1e-7
    e, f, sa = O.lcpo_forces(s, list_cutoff(d), sub.lcpo_radius, sub.lcpo_p, sub.lcpo_sigma, sub.lcpo_use,
                             nthreads=8)
    assert rel_err(e[6], ref_energy(d, "sasa", "surf")) < 1e-12
    assert np.max(np.abs(sa - d["lcpo_sasa"])) <= 1e-4
    assert rel_rms(f, d["sasa_f"]) < 1e-7


def test_dense_lcpo_lattice_cuts_lists_and_the_cut_matters():
    """The premise of the device test of cut LCPO lists (test_gpu_parity.py::
    test_lcpo_cut_lists_match_oracle): atoms beyond PD's 80 partners and none
    beyond the 160 candidates, no pair near the overlap distance, and the
    triple terms (the sums the cut decides) a large share of each SA."""
    pytest.importorskip("scipy")
    from scipy.spatial import cKDTree
    from test_gpu_parity import _dense_lcpo_lattice
    pos = _dense_lcpo_lattice()
    n = len(pos)
    p = cKDTree(pos).query_pairs(2 * 3.1, output_type="ndarray")
    count = np.bincount(p.ravel(), minlength=n)
    assert (count > 80).sum() > 300 and count.max() <= 160
    q = cKDTree(pos).query_pairs(2 * 3.1 + 2e-3, output_type="ndarray")
    d = np.linalg.norm(pos[q[:, 0]] - pos[q[:, 1]], axis=1)
    assert np.min(np.abs(d - 2 * 3.1)) >= 2e-3
    s = O.OracleSystem(pos, np.zeros(n), np.full(n, 1.5), np.zeros(n), np.zeros((0, 3), np.int32))
    radius, sigma, use = np.full(n, 3.1), np.full(n, 3.47e-23), np.ones(n, np.int32)
    _, _, sa = O.lcpo_forces(s, 8.2, radius, np.tile([0.5, 1e-3, 1e-3, 1e-5], (n, 1)), sigma, use)
    _, _, sa_pairs = O.lcpo_forces(s, 8.2, radius, np.tile([0.5, 1e-3, 0.0, 0.0], (n, 1)), sigma, use)
    assert np.all(sa > 0) and np.mean(sa - sa_pairs) > 0.3 * np.mean(sa)
