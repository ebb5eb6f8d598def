"""Device dynamics against the oracle's FP64 integrators (PD md.cpp) and REMD properties."""
import os

import numpy as np
import pytest

from conftest import rel_rms
from helpers import gb_kwargs, nb_kwargs, nb_params, oracle_system
from oracle import pdoracle as O

pytestmark = pytest.mark.gpu


def water_ctx(d, integrator, what, use_graph=True, temp=300.0):
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    ctx = DeviceContext(SystemImage._from_fixture(d))
    ctx.set_list(2.0)
    ctx.set_nb(**nb_kwargs(d, "nb"))
    ctx.set_positions(d["pos"])
    ctx.md_setup([temp], integrator=integrator, timestep=1e-15, fric=1e13, update_nlist=1, what=what,
                 seed=7, use_graph=use_graph)
    return ctx


def oracle_forces(d, pos):
    s = O.OracleSystem(pos, d["charge"], d["radius"], d["epsilon"], d["excl"], tuple(d["box"]))
    _, f = O.nonbonded(s, nb_params(d, "nb"))
    _, fb = O.bonded(pos, d["bond_idx"], d["bond_par"], d["angle_idx"], d["angle_par"], d["torsion_idx"],
                     d["torsion_par"], d["improper_idx"], d["improper_par"])
    return f + fb


def test_velocity_verlet_steps_match_oracle(goldens):
    from pd_gb300 import ffi
    from pd_gb300.md import maxwell_boltzmann
    d = goldens["water_c1"]
    v0 = maxwell_boltzmann(d["mass"], 300.0, 3)
    ctx = water_ctx(d, 0, ffi.NB | ffi.BONDED)
    ctx.set_velocities(v0)
    p, v = d["pos"].copy(), v0.copy()
    for step in range(3):
        ctx.md_run(1)
        f = oracle_forces(d, p)
        p, v, ek = O.vv_step(p, v, f, d["mass"], 1e-15)
    gp, gv = ctx.get_positions(), ctx.get_velocities()
    # FP32 forces (rel. RMS <= 1e-5) propagate into the displacement at that level
    assert rel_rms(gp - d["pos"], p - d["pos"]) < 1e-5
    assert rel_rms(gv, v) < 1e-5


def test_langevin_zero_temperature_matches_oracle(goldens):
    """T = 0 removes the noise: the deterministic part of PD's Langevin step must agree."""
    from pd_gb300 import ffi
    from pd_gb300.md import maxwell_boltzmann
    d = goldens["water_c1"]
    v0 = maxwell_boltzmann(d["mass"], 300.0, 5)
    ctx = water_ctx(d, 1, ffi.NB | ffi.BONDED, temp=0.0)
    ctx.set_velocities(v0)
    p, v = d["pos"].copy(), v0.copy()
    noise = np.zeros((len(p), 6))
    for step in range(3):
        ctx.md_run(1)
        f = oracle_forces(d, p)
        p, v, _ = O.langevin_step(p, v, f, d["mass"], 1e-15, 1e13, 0.0, noise, first_step=(step == 0))
    gp, gv = ctx.get_positions(), ctx.get_velocities()
    assert rel_rms(gp - d["pos"], p - d["pos"]) < 1e-5
    assert rel_rms(gv, v) < 1e-5


def test_graph_replay_is_bitwise_identical_to_direct_launches(goldens):
    from pd_gb300 import ffi
    d = goldens["water_c1"]
    out = []
    for g in (False, True):
        ctx = water_ctx(d, 1, ffi.NB | ffi.BONDED, use_graph=g)
        ctx.md_run(12, energy_on_last=True)
        out.append((ctx.get_positions(), ctx.get_velocities(), ctx.energies()[0]["epot"]))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_langevin_thermalises_gb_peptide(goldens):
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    d = goldens["peptide30"]
    im = SystemImage._from_fixture(d)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_positions(d["pos"])
    ctx.md_setup([300.0], integrator=1, timestep=1e-15, fric=5e13, update_nlist=10, update_sasa=5,
                 what=ffi.GB | ffi.SA | ffi.BONDED, seed=11)
    temps = []
    for _ in range(10):
        ctx.md_run(200)
        temps.append(2 * ctx.kinetic()[0] / (3 * im.natom * 1.38065e-23))
    T = np.mean(temps[3:])
    assert 250.0 < T < 350.0, temps


def test_langevin_temperature_matches_oracle_statistically(goldens):
    """PD's Langevin scheme (md.cpp:923-1063) at 2 fs and its default friction reads a
    kinetic temperature a few percent under the target on a flexible peptide (kinetic
    energy taken after the first kick, as PD's calcKineticEnergy does).  The device
    integrator must reproduce that stationary temperature, not just approach the
    target: both run 3,000 steps from the same start (different random streams) and
    their mean temperatures over the last 2,000 steps must agree within 4 combined
    standard errors."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    from helpers import gb_params
    d = goldens["peptide30"]
    im = SystemImage._from_fixture(d)
    n, kB, dt, gamma, T0 = im.natom, 1.38065e-23, 2e-15, 1e13, 300.0
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_positions(d["pos"])
    ctx.md_setup([T0], integrator=1, timestep=dt, fric=gamma, update_nlist=1, what=ffi.GB | ffi.BONDED, seed=3)
    gT = []
    for c in range(300):
        ctx.md_run(10)
        if c >= 100:
            gT.append(2 * ctx.kinetic()[0] / (3 * n * kB))
    ctx.close()
    gp = gb_params(d)
    bonded = (d["bond_idx"], d["bond_par"], d["angle_idx"], d["angle_par"], d["torsion_idx"], d["torsion_par"],
              d["improper_idx"], d["improper_par"])
    rng = np.random.default_rng(3)
    pos, vel = d["pos"].copy(), np.zeros_like(d["pos"])
    oT = []
    for step in range(3000):
        s = O.OracleSystem(pos, d["charge"], d["radius"], d["epsilon"], d["excl"], tuple(d["box"]))
        _, f, _ = O.gb_forces(s, gp, d["gb_radius"], d["gb_vj"], d["gb_terms123"], os.cpu_count() or 1)
        _, fb = O.bonded(pos, *bonded)
        pos, vel, ek = O.langevin_step(pos, vel, f + fb, d["mass"], dt, gamma, T0, rng.standard_normal((n, 6)),
                                       first_step=(step == 0))
        if step >= 1000 and step % 10 == 0:
            oT.append(2 * ek / (3 * n * kB))
    sem = lambda x: np.std(x) / np.sqrt(len(x) / 10.0)   # samples 10 steps apart are correlated
    gm, om = float(np.mean(gT)), float(np.mean(oT))
    assert abs(gm - om) <= 4.0 * np.hypot(sem(gT), sem(oT)), (gm, om)
    assert 0.85 * T0 < gm < 1.05 * T0, gm


def test_remd_exchange_swaps_temperatures_and_rescales(goldens):
    """Equal energies and temperatures always accept (delta = 0); swapped
    systems exchange target temperatures and velocities scale by sqrt(T'/T)."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    d = goldens["peptide30"]
    im = SystemImage.concat([SystemImage._from_fixture(d)] * 4)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_positions(np.concatenate([d["pos"]] * 4))
    ladder = np.array([300.0, 300.0, 400.0, 400.0])
    ctx.md_setup(ladder, integrator=1, timestep=1e-15, what=ffi.GB | ffi.BONDED, seed=3)
    ctx.md_run(1, energy_on_last=True)
    v_before = ctx.get_velocities()
    acc, temps = ctx.remd_exchange(0)       # rungs (0,1) and (2,3): equal T => delta = 0 => accept
    assert acc[0] == 1 and acc[2] == 1
    assert np.allclose(temps, [300, 300, 400, 400])
    acc, temps = ctx.remd_exchange(1)       # rungs (1,2): 300 K <-> 400 K
    n = im.natoms[0]
    v_after = ctx.get_velocities()
    if acc[1]:
        lo, hi = 0, 3   # after the first sweep rung 1 holds system 0, rung 2 holds system 3
        assert np.isclose(temps[lo], 400.0) and np.isclose(temps[hi], 300.0)
        assert np.allclose(v_after[lo * n:(lo + 1) * n], v_before[lo * n:(lo + 1) * n] * np.sqrt(400 / 300.))
    else:
        assert np.array_equal(v_after, v_before)


def _philox4x32(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11), the generator of the exchange draws."""
    M = 0xFFFFFFFF
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0, p1 = 0xD2511F53 * c0, 0xCD9E8D57 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & M, p1 & M, ((p0 >> 32) ^ c3 ^ k1) & M, p0 & M
        k0, k1 = (k0 + 0x9E3779B9) & M, (k1 + 0xBB67AE85) & M
    return c0, c1, c2, c3


def _exchange_uniform(seed, rnd, rung):
    """The uniform draw of rung `rung` in exchange round `rnd` (counter (round, rung, 7))."""
    x = _philox4x32((rnd & 0xFFFFFFFF, rnd >> 32, rung, 7),
                    ((seed & 0xFFFFFFFF) ^ 0x5BD1E995, seed >> 32))[0]
    return (x + 0.5) / 4294967296.0


def test_remd_metropolis_decision_matches_pd_criterion(goldens):
    """REX_Local::exchangeCriterion (remd.cpp:349-356): delta = (E_lo - E_hi)
    (1/kT_hi - 1/kT_lo), accept when delta <= 0 or exp(-delta) > u.  Four
    systems of unequal energy on a ladder chosen so the first sweep's rungs have
    delta = 0.3, 1.0 and 2.5, then 24 sweeps of alternating parity: every device
    decision, the temperatures and the velocity rescaling against the host's
    own evaluation of the criterion with the same Philox uniforms."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    kB = 1.38065E-23
    d = goldens["peptide30"]
    rng = np.random.default_rng(11)
    pos = [d["pos"] + rng.normal(0.0, 0.05, d["pos"].shape) for _ in range(4)]
    im = SystemImage.concat([SystemImage._from_fixture(d)] * 4)
    n = im.natoms[0]
    what = ffi.GB | ffi.BONDED

    def energies(ctx):
        return np.array([e["epot"] for e in ctx.compute(what)])

    probe = DeviceContext(im)
    probe.set_list(2.0)
    probe.set_gb(**gb_kwargs(d))
    probe.set_positions(np.concatenate(pos))
    E = energies(probe)
    probe.close()
    order = np.argsort(E)                     # rung r starts with the r-th lowest energy
    pos = [pos[i] for i in order]
    E = E[order]
    T = [300.0]
    for r, target in enumerate((0.3, 1.0, 2.5)):
        dE = E[r] - E[r + 1]                  # < 0: the lower rung holds the lower energy
        target = min(target, 0.5 * abs(dE) / (kB * T[r]))
        T.append(1.0 / (1.0 / T[r] - target * kB / abs(dE)))
    T = np.array(T)
    seed = 0x1234ABCD5678
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_positions(np.concatenate(pos))
    ctx.md_setup(T, integrator=0, timestep=1e-15, what=what, seed=seed)
    v0 = np.tile(np.arange(1.0, 4.0), (im.natom, 1))
    ctx.set_velocities(v0)
    Edev = energies(ctx)                      # the energies the exchange reads
    assert np.allclose(Edev, E, rtol=1e-12, atol=0)
    holder = list(range(4))                   # system at each rung
    temp = dict(zip(range(4), T))             # target temperature of each system
    vscale = np.ones(4)
    decided, draws_on = 0, 0
    for rnd in range(24):
        parity = rnd % 2
        acc, temps = ctx.remd_exchange(parity)
        for r in range(parity, 3, 2):
            lo, hi = holder[r], holder[r + 1]
            delta = (Edev[lo] - Edev[hi]) * (1.0 / (kB * T[r + 1]) - 1.0 / (kB * T[r]))
            u = _exchange_uniform(seed, rnd, r)
            want = delta <= 0 or np.exp(-delta) > u
            if delta > 0 and abs(np.exp(-delta) - u) < 1e-9:
                want = bool(acc[r])          # a draw within rounding of the boundary decides nothing
            assert bool(acc[r]) == want, (rnd, r, delta, u)
            decided += 1
            draws_on += int(delta > 0)
            if want:
                f = np.sqrt(T[r + 1] / T[r])
                holder[r], holder[r + 1] = hi, lo
                temp[lo], temp[hi] = T[r + 1], T[r]
                vscale[lo] *= f
                vscale[hi] /= f
        assert np.allclose(temps, [temp[s] for s in range(4)], rtol=0, atol=1e-12)
    v = ctx.get_velocities()
    for s in range(4):
        assert np.allclose(v[s * n:(s + 1) * n], v0[s * n:(s + 1) * n] * vscale[s], rtol=1e-12)
    assert draws_on >= 10 and decided == 36
    ctx.close()


def test_async_host_copies_match_synchronous_calls(goldens):
    """A dynamics loop through the asynchronous entry points (positions in,
    one step, kinetic energies and positions out, all queued in stream order
    into page-locked buffers, one wait at the end) gives bit for bit what the
    synchronous calls give step by step."""
    from pd_gb300 import ffi
    d = goldens["water_c1"]
    ref = water_ctx(d, 1, ffi.NB | ffi.BONDED)
    pos = d["pos"].copy()
    kes = []
    for _ in range(7):
        ref.set_positions(pos)
        ref.md_run(1)
        kes.append(ref.kinetic())
        pos = ref.get_positions()
    ref.close()
    ctx = water_ctx(d, 1, ffi.NB | ffi.BONDED)
    pos_h = ffi.host_array(d["pos"].shape)
    pos_h[...] = d["pos"]
    ke_h = [ffi.host_array((1,)) for _ in range(7)]
    for k in range(7):
        ctx.set_positions_async(pos_h)
        ctx.md_enqueue(1)
        ctx.kinetic_async(ke_h[k])
        ctx.get_positions_async(pos_h)
    ctx.synchronize()
    assert np.array_equal(pos_h, pos)
    for k in range(7):
        assert np.array_equal(ke_h[k], kes[k])
    ctx.close()


@pytest.mark.parametrize("use_graph", [False, True])
def test_list_rebuilds_follow_update_nlist(goldens, use_graph):
    """The list is rebuilt on the steps PD's ProtocolBase::refreshNeighborList
    rebuilds it (protocolbase.cpp:135-144: a call counter that starts at 0 and
    rebuilds when counter % UpdateNList == 0, one call per MD step, md.cpp:232),
    counted across md_run calls as PD's counter lives with the protocol.  A
    rebuild step launches the list build's kernels on top of a plain step's."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    d = goldens["water_c1"]
    ctx = DeviceContext(SystemImage._from_fixture(d))
    ctx.set_list(2.0)
    ctx.set_nb(**nb_kwargs(d, "nb"))
    ctx.set_positions(d["pos"])
    ctx.md_setup([300.0], integrator=1, timestep=1e-15, fric=1e13, update_nlist=3, what=ffi.NB | ffi.BONDED,
                 seed=7, use_graph=use_graph)
    counts = []
    for n in (2, 3, 2, 4):   # runs of different lengths: the cadence carries across them
        for _ in range(n):
            k1 = ctx.kernel_launches()
            ctx.md_enqueue(1)
            counts.append(ctx.kernel_launches() - k1)
        ctx.synchronize()
    plain = min(counts)
    rebuilt = [s for s, k in enumerate(counts) if k > plain]
    assert rebuilt == [s for s in range(len(counts)) if s % 3 == 0], counts
    ctx.close()


def test_md_is_deterministic(goldens):
    from pd_gb300 import ffi
    d = goldens["water_c1"]
    res = []
    for _ in range(2):
        ctx = water_ctx(d, 1, ffi.NB | ffi.BONDED)
        ctx.md_run(15)
        res.append(ctx.get_positions())
        ctx.close()
    assert np.array_equal(res[0], res[1])


def test_rex_checkpoint_mime_round_trip(goldens, tmp_path):
    """REX_Local writes PD's MIME checkpoint (one section per replica rung) and
    reads it back into the systems at those rungs."""
    from pd_gb300 import checkpoint
    from pd_gb300.forcefield import FF_Bonded_GPU, FF_GeneralizedBorn_Still_GPU, Forcefield
    from pd_gb300.md import MolecularDynamics, REX_Local
    from pd_gb300.workspace import SystemImage, WorkSpace
    d = goldens["peptide30"]
    im = SystemImage.concat([SystemImage._from_fixture(d)] * 3)
    ws = WorkSpace(im)
    ws.Padding = 2.0
    ff = Forcefield(ws)
    ff.add(FF_Bonded_GPU(ws))
    gb = FF_GeneralizedBorn_Still_GPU(ws)
    for k, v in gb_kwargs(d).items():
        setattr(gb, k, v)
    ff.add(gb)
    md = MolecularDynamics(ff)
    md.Timestep = 1e-15
    md.UpdateNList = 1          # the test is about the checkpoint, not the list cadence
    rex = REX_Local(md, [300.0, 350.0, 400.0])
    rex.ExchangeFreq = 20
    rex.run(2)
    path = str(tmp_path / "remd.mime")
    rex.writeCheckPointMIME(path)
    ctx = ws.context()
    pos0, vel0 = ctx.get_positions(), ctx.get_velocities()
    rungs = rex._rung_systems(ctx)
    off = im.offsets
    for r, k in enumerate(rungs):
        s = checkpoint.read_snapshot(path, "remd%d" % r)
        assert np.array_equal(s["pos"], pos0[off[k]:off[k + 1]])
        assert np.array_equal(s["vel"], vel0[off[k]:off[k + 1]])
    rex.run(1)                                   # move on, then restore
    rex.readCheckPointMIME(path)
    now = rex._rung_systems(ctx)                 # replica r goes to the system now at rung r
    pos1 = ctx.get_positions()
    for r in range(3):
        assert np.array_equal(pos1[off[now[r]]:off[now[r] + 1]], pos0[off[rungs[r]]:off[rungs[r] + 1]])


def _four_copies(d, ladder, what_extra=0, update_nlist=10):
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    n = len(ladder)
    im = SystemImage.concat([SystemImage._from_fixture(d)] * n)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(d))
    rng = np.random.default_rng(5)
    ctx.set_positions(np.concatenate([d["pos"] + 0.01 * rng.standard_normal(d["pos"].shape) for _ in range(n)]))
    ctx.md_setup(np.asarray(ladder, float), integrator=1, timestep=1e-15, update_nlist=update_nlist,
                 what=ffi.GB | ffi.BONDED | what_extra, seed=3)
    return im, ctx


@pytest.mark.parametrize("mode", [1, 2])
def test_remd_copy_modes_move_structures(goldens, mode):
    """Downward (1) / Upward (2) exchange (remd.cpp:186-200): equal temperatures
    always accept; the destination rung gets the other structure and PD's
    velocity rescaling (factor 1 at equal T), temperatures stay with the systems."""
    d = goldens["peptide30"]
    im, ctx = _four_copies(d, [300.0, 300.0, 400.0, 400.0])
    ctx.remd_set_modes(mode)
    ctx.md_run(3, energy_on_last=True)
    p0, v0 = ctx.get_positions(), ctx.get_velocities()
    acc, temps = ctx.remd_exchange(0)          # rung pairs (0,1) and (2,3)
    assert acc[0] == 1 and acc[2] == 1
    assert np.allclose(temps, [300, 300, 400, 400])
    p1, v1 = ctx.get_positions(), ctx.get_velocities()
    n = im.natoms[0]
    sl = lambda k: slice(k * n, (k + 1) * n)
    for lo, hi in ((0, 1), (2, 3)):
        dst, src = (lo, hi) if mode == 1 else (hi, lo)
        assert np.array_equal(p1[sl(dst)], p0[sl(src)]) and np.array_equal(p1[sl(src)], p0[sl(src)])
        assert np.allclose(v1[sl(dst)], v0[sl(src)], rtol=1e-15, atol=0)
    ctx.md_run(3)                              # the list is rebuilt after the copies: no stale-list error
    acc, temps = ctx.remd_exchange(1)          # rungs (1,2): 300 K <-> 400 K
    if acc[1]:
        p2 = ctx.get_positions()
        dst, src = (1, 2) if mode == 1 else (2, 1)
        assert np.array_equal(p2[sl(dst)], p2[sl(src)])


def test_remd_copy_modes_need_one_molecule(goldens):
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    names = ["peptide30", "peptide120"]
    im = SystemImage.concat([SystemImage._from_fixture(goldens[k]) for k in names])
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(goldens["peptide30"]))
    ctx.set_positions(np.concatenate([goldens[k]["pos"] for k in names]))
    ctx.md_setup([300.0, 350.0], integrator=1, timestep=1e-15, what=ffi.GB, seed=1)
    with pytest.raises(ffi.PDGPUError) as ei:
        ctx.remd_set_modes(1)
    assert ei.value.status == -7
    ctx.remd_set_modes(0)                       # swapping temperatures works for any batch


def test_crash_rescue_restores_unstable_system(goldens):
    """A system whose state turns non-finite (planted from the host: one atom's
    position NaN) is put back to the checkpoint with fresh velocities at its
    target temperature; the other systems keep their state (remd.cpp:118-147)."""
    from pd_gb300 import ffi
    d = goldens["peptide30"]
    im, ctx = _four_copies(d, [300.0, 350.0])
    ctx.md_run(5)
    ctx.md_checkpoint()
    p0 = ctx.get_positions()
    bad = p0.copy()
    n = im.natoms[0]
    bad[n + 3, 1] = np.nan                      # system 1
    ctx.set_positions(bad)
    with pytest.raises(ffi.PDGPUError) as ei:
        ctx.md_run(4)
    # a non-finite atom drops out of every cutoff test, so the round ends on the
    # list check (or on NaN / overflow if its forces were formed)
    assert ei.value.status in (-5, -4, -8)
    p_ok, v_ok = ctx.get_positions()[:n], ctx.get_velocities()[:n]
    flags = ctx.md_rescue(17)
    assert list(flags) == [False, True]
    p1, v1 = ctx.get_positions(), ctx.get_velocities()
    assert np.array_equal(p1[n:], p0[n:])
    assert np.array_equal(p1[:n], p_ok) and np.array_equal(v1[:n], v_ok)
    ke = 0.5 * (im.mass[n:, None] * v1[n:] ** 2).sum()
    assert np.isclose(ke, 1.5 * n * 1.38065e-23 * 350.0, rtol=1e-9)
    ctx.md_run(10)                              # runs on from the rescued state
    assert np.all(np.isfinite(ctx.get_positions()))


def test_trajectory_frames_without_host_sync(goldens, tmp_path):
    """Frames copied every UpdateTra steps into the host ring equal the positions a
    step-by-step run reaches, and the PDB writer stores them as models."""
    from pd_gb300.trajectory import PDBTrajectory, read_pdb_models
    d = goldens["peptide30"]
    im, ctx = _four_copies(d, [300.0, 320.0])
    ring = ctx.md_set_trajectory(5, nslots=4)
    ctx.md_run(20)
    assert ctx.md_trajectory_frames() == 4
    assert np.array_equal(ring[3], ctx.get_positions())
    assert not np.array_equal(ring[0], ring[3])
    # the same trajectory run step by step from the same start reproduces frame 2 (step 15)
    im2, ctx2 = _four_copies(d, [300.0, 320.0])
    ctx2.md_run(15)
    assert np.array_equal(ring[2], ctx2.get_positions())
    path = str(tmp_path / "tra.pdb")
    w = PDBTrajectory(path, im)
    w.append(ring)
    back = read_pdb_models(path)
    assert back.shape == (4, im.natom, 3) and np.allclose(back, ring, atol=6e-4)


def test_autotune_restores_the_state_and_picks_listed_settings(goldens):
    """pdgpu_md_autotune runs trial dynamics from a saved state and puts it back:
    positions and velocities bit-identical, and the next step (the step counter
    keys the Langevin noise) the same as on a context that never tuned, to the
    FP32 rounding the chosen list settings allow.  Every setting comes from the
    tuner's candidate sets."""
    from pd_gb300 import ffi
    from pd_gb300.md import maxwell_boltzmann
    d = goldens["water_c1"]
    v_init = maxwell_boltzmann(d["mass"], 300.0, 5)
    ctxs = []
    for _ in range(2):
        ctx = water_ctx(d, 1, ffi.NB | ffi.BONDED)
        ctx.set_velocities(v_init)
        ctx.md_run(5)
        ctxs.append(ctx)
    tuned_ctx, plain_ctx = ctxs
    p0, v0 = tuned_ctx.get_positions(), tuned_ctx.get_velocities()
    tuned = tuned_ctx.autotune(trial_steps=10)
    assert tuned["UpdateNList"] in (1, 2, 3, 5, 10, 20, 40, 80)
    assert tuned["ctas_per_sm"] in (2, 4, 8, 16)
    assert tuned["gb_tiles_per_item"] in (1, 2)
    assert tuned["nb_groups"] in (True, False)
    assert np.array_equal(tuned_ctx.get_positions(), p0)
    assert np.array_equal(tuned_ctx.get_velocities(), v0)
    tuned_ctx.md_run(1)
    plain_ctx.md_run(1)
    assert np.allclose(tuned_ctx.get_positions(), plain_ctx.get_positions(), rtol=0, atol=1e-9)
    assert rel_rms(tuned_ctx.get_velocities(), plain_ctx.get_velocities()) <= 1e-6
    for c in ctxs:
        c.close()
