#!/usr/bin/env python3
"""Benchmark of the GB300 nonbonded / GB-SA path of PD.

Headline workload (default, ``--workload c4``): batched REMD of 64 GB/SA
peptides of uneven size (30-478 residues, ~210k atoms in total, built by PD),
Langevin at 2 fs over a geometric 300-500 K ladder, exchange attempts every
500 steps, all replicas advanced together by the batched kernels replayed from
captured CUDA graphs.  One "step" = one MD step of every replica.

metric: atom-steps/s (sum over systems of atoms x steps / s), reported beside
the plain single-system GPU path on the same systems (one context per system,
no batching, no graphs), the force error against the FP64 oracle, and the
oracle's CPU throughput on the host cores.

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c1|c2|c3|c4|c5] [--impl reference]
(c5 is the parameter-fitting task through the adjoint kernels: its own JSON
line, frame-atom gradient evaluations per second, with a finite-difference
check against the FP64 oracle.)
Under torchrun each rank runs its own replica set (replicas only: the path has
no exchange between GPUs); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

KB = 1.38065E-23
METRIC = "atom-steps/s batched vs plain GPU at force rel err <=1e-5 vs FP64; % HBM roofline"

# FP32 flops per pair of the pair kernels by the branch the pair takes (FMA =
# 2 flops, each MUFU operation = 1), counted from the pair law each kernel
# evaluates; pairs per branch come from pdgpu_pair_census at the final state.
#   GB fused pair (k_gb_pair), every pair inside the GB cutoff: d (3), r^2 (5),
#     u = -r^2/(4 a_i a_j) for the threshold test (4), 1/r (1), q_i q_j (1),
#     Coulomb energy and dE/dr (3), LJ 12-6 (12), dE/dr / r (3), forces on both
#     atoms (12): 44.  Above ExpApproxThreshold the GB cross term adds exp,
#     f_GB = 1/sqrt(r^2 + a_i a_j e^u), E, dE/dr, dE/da for both atoms: +23.
#   FF_NonBonded pair inside the cutoff (k_nb_tiles, energy-switched LJ and
#     Coulomb): d (3), r^2 (5), 1/r and r (2), LJ (12), both switches (22),
#     sum and 1/r (2), forces (12): 58.
#   Born-radius pair (k_gb_born, both directions): d, r^2 (8), R_i + R_j and
#     the contact test (3), 1/r^2 (1), P4 / r^4 (3), two sums (4): 19; in close
#     contact the CCF adds 7.
#   Chain-rule pair (k_gb_chain, both directions): d, r^2 (8), contact test
#     (3), 1/r^2 (1), c_i V_j + c_j V_i (3), the factor over r^6 (4), forces
#     (12): 31; in close contact the CCF and its derivative add 13.
FLOPS = {"gb_pair": 44, "gb_term": 23, "nb": 58, "born": 19, "born_contact": 7, "chain": 31, "chain_contact": 13}
# bytes per atom-step of the integrator: read p, v, f (24 B each) + mass (8 B), write p, v
INTEGRATOR_BYTES = 80 + 48

WORKLOADS = {
    "c1": dict(image="c1_water", desc="667 TIP3P waters (2,001 atoms), 27.5 A box, LJ+Coulomb 12/10 A energy switch, "
               "2 A skin, velocity Verlet 1 fs", what=("NB", "BONDED"), integrator=0, dt=1e-15, padding=2.0),
    "c2": dict(image="c2_solvated", desc="120-residue peptide in TIP3P (22,489 atoms), 62 A box, LJ+Coulomb 12/10 A, "
               "2 A skin, Langevin 2 fs 300 K", what=("NB", "BONDED"), integrator=1, dt=2e-15, padding=2.0),
    "c3": dict(image="c3_gb256", desc="256-residue peptide (4,235 atoms), GB/SA all pairs, Langevin 2 fs 300 K",
               what=("GB", "SA", "BONDED"), integrator=1, dt=2e-15, padding=2.0),
    "c4": dict(image="c4_remd64", desc="batched REMD of 64 GB/SA peptides (30-478 residues), all pairs, Langevin 2 fs, "
               "geometric 300-500 K, exchange every 500 steps", what=("GB", "SA", "BONDED"), integrator=1, dt=2e-15,
               padding=2.0),
}


# ---------------------------------------------------------------------------
# distributed helpers (replicas only; barrier and a max over ranks of the time)
# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def reduce_max_sum(dist, t, units):
    """(max over ranks of the time, sum over ranks of the units processed)."""
    if dist is None:
        return t, units
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    a = torch.tensor([t], dtype=torch.float64, device=dev)
    b = torch.tensor([units], dtype=torch.float64, device=dev)
    dist.all_reduce(a, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return float(a.item()), float(b.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload construction
# ---------------------------------------------------------------------------
def flags(names):
    from pd_gb300 import ffi
    w = 0
    for n in names:
        w |= getattr(ffi, n)
    return w


def gb_settings(image):
    """FF_GeneralizedBorn_Still attributes of the GB workloads: all pairs, eps 1 / 80."""
    s14v, s14e = image.scaling14
    P = image.gb_P
    return dict(Cutoff=999.0, InnerCutoff=998.0, VdwCutoff=999.0, VdwInnerCutoff=998.0, Vdw14Scaling=s14v,
                Elec14Scaling=s14e, DielectricSolute=1.0, DielectricSolvent=80.0, GbsaStillCutoff=999.0,
                ExpApproxThreshold=-4.0, BornRadiusOffset=0.0, P4=P[3], P5=P[4])


NB_CUTOFF = 12.0   # FF_NonBonded Cutoff and VdwCutoff of the C1/C2 workloads (A)

# DRAM bytes (read + write) per launch of the roofline kernels, from one ncu
# capture of each workload (the DRAM traffic summary under profiles/)
NCU_TRAFFIC = {
    "c4": {"k_gb_pair": 41.33e6, "k_langevin": 23.55e6},
    "c3": {"k_gb_pair": 0.85e6, "k_langevin": 0.50e6},
    "c2": {"k_nb_tiles": 17.47e6, "k_langevin": 2.00e6},
    "c1": {"k_nb_tiles": 0.30e6},
}


def configure(ctx, wl, image):
    """Component parameters of each workload (PD attribute names)."""
    s14v, s14e = image.scaling14
    if "NB" in wl["what"]:
        ctx.set_nb(Cutoff=NB_CUTOFF, InnerCutoff=10.0, VdwCutoff=NB_CUTOFF, VdwInnerCutoff=10.0, Vdw14Scaling=s14v,
                   Elec14Scaling=s14e, Dielectric=1.0, EnergySwitch=1, ForceSwitch=0, DoVdw=1, DoElec=1)
    if "GB" in wl["what"]:
        ctx.set_gb(**gb_settings(image))
    ctx.set_list(wl["padding"])


def temperatures(image, key):
    if key == "c4":
        n = image.nsystems
        return 300.0 * (500.0 / 300.0) ** (np.arange(n) / max(n - 1, 1))
    return np.full(image.nsystems, 300.0)


RELAX = dict(steps=300, dt=0.2e-15, fric=5e13, update_nlist=1)


def make_context(image, wl, key, seed, use_graph=True, device=0, update_nlist=10, relax=True):
    """Context at the workload's settings.  The PD-built starting structures are
    not equilibrated (lattice waters, compacted chains), so an untimed relaxation
    (Langevin, 0.2 fs, strong friction, list rebuilt every step) runs first;
    production then starts from fresh Maxwell-Boltzmann velocities."""
    from pd_gb300.engine import DeviceContext
    from pd_gb300.md import maxwell_boltzmann
    ctx = DeviceContext(image, device)
    configure(ctx, wl, image)
    ctx.set_positions(image.pos)
    temps = temperatures(image, key)
    what = flags(wl["what"])
    if relax and RELAX["steps"] > 0:
        ctx.md_setup(temps, integrator=1, timestep=RELAX["dt"], fric=RELAX["fric"], update_nlist=RELAX["update_nlist"],
                     update_sasa=5, what=what, seed=seed + 7, use_graph=True)
        ctx.md_run(RELAX["steps"])
    ctx.md_setup(temps, integrator=wl["integrator"], timestep=wl["dt"], fric=1e13, update_nlist=update_nlist,
                 update_sasa=5, what=what, seed=seed, use_graph=use_graph)
    ctx.set_velocities(maxwell_boltzmann(image.mass, temps, seed, image.natoms))
    return ctx, temps


# ---------------------------------------------------------------------------
# parity against the FP64 oracle on one system of the workload
# ---------------------------------------------------------------------------
def parity_check(image, wl, key, pos=None):
    """Energy and forces of one system (the median-size one of a batch) on the GPU
    against the FP64 oracle, at the image's positions or at `pos` (all systems)."""
    from oracle import pdoracle as O
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    k = 0
    if image.nsystems > 1:   # the median-size system of the batch
        k = int(np.argsort(image.natoms)[image.nsystems // 2])
    sub = image.subset(k)
    if pos is not None:
        sub.pos = np.ascontiguousarray(pos[image.offsets[k]:image.offsets[k + 1]])
    ctx = DeviceContext(sub)
    configure(ctx, wl, sub)
    ctx.set_positions(sub.pos)
    f = np.zeros((sub.natom, 3))
    e = ctx.compute(flags(wl["what"]), f)[0]
    ctx.close()
    s = O.OracleSystem(sub.pos, sub.charge, sub.radius, sub.epsilon, sub.excl, tuple(sub.box[0]))
    ref_f = np.zeros((sub.natom, 3))
    ref_e = 0.0
    threads = os.cpu_count() or 1
    s14v, s14e = sub.scaling14
    if "NB" in wl["what"]:
        p = O.nb_params(Cutoff=12, InnerCutoff=10, Vdw14Scaling=s14v, Elec14Scaling=s14e, EnergySwitch=1,
                        ListCutoff=12 + wl["padding"])
        ee, ff = O.nonbonded(s, p, threads)
        ref_f += ff
        ref_e += ee[0]
    if "GB" in wl["what"]:
        P = sub.gb_P
        gp = O.gb_params(Cutoff=999, InnerCutoff=998, VdwCutoff=999, VdwInnerCutoff=998, Vdw14Scaling=s14v,
                         Elec14Scaling=s14e, GbsaStillCutoff=999, P1=P[0], P2=P[1], P3=P[2], P4=P[3], P5=P[4],
                         ListCutoff=999 + wl["padding"])
        ee, ff, _ = O.gb_forces(s, gp, sub.gb_radius, sub.gb_vj, sub.gb_terms123, threads)
        ref_f += ff
        ref_e += ee[0]
    if "SA" in wl["what"]:
        ee, ff, _ = O.lcpo_forces(s, 999 + wl["padding"], sub.lcpo_radius, sub.lcpo_p, sub.lcpo_sigma, sub.lcpo_use,
                                  threads)
        ref_f += ff
        ref_e += ee[0]
    if "BONDED" in wl["what"]:
        ee, ff = O.bonded(sub.pos, *sub.bonds, *sub.angles, *sub.torsions, *sub.impropers)
        ref_f += ff
        ref_e += ee.sum()
    frms = float(np.sqrt(((f - ref_f) ** 2).sum(1).mean() / (ref_f ** 2).sum(1).mean()))
    return {"system_atoms": int(sub.natom), "force_rel_rms": frms, "energy_rel_err": abs(e["epot"] - ref_e) / abs(ref_e)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's FP64 restatement of PD's path on the host cores
# ---------------------------------------------------------------------------
class CPUSystem:
    """The oracle's FP64 restatement of PD's path stepping one system of a
    workload: forces of the workload's components (PD's O(N^2) list kept for
    UpdateNList = 10 steps for cutoff systems, LCPO every 5 steps), then the
    FP64 integrator.  State (positions, velocities, stored list) carries over
    between steps."""

    def __init__(self, O, sub, wl, threads, seed):
        self.O, self.sub, self.wl, self.threads = O, sub, wl, threads
        self.pos = sub.pos.copy()
        self.vel = np.zeros_like(self.pos)
        self.rng = np.random.default_rng(seed)
        self.steps = 0
        self.nlist = None
        self.f_sa = np.zeros_like(self.pos)

    def step(self):
        O, wl, sub, threads = self.O, self.wl, self.sub, self.threads
        s14v, s14e = sub.scaling14
        s = O.OracleSystem(self.pos, sub.charge, sub.radius, sub.epsilon, sub.excl, tuple(sub.box[0]))
        f = np.zeros_like(self.pos)
        if "NB" in wl["what"]:
            # PD keeps the list for UpdateNList = 10 steps (protocolbase.cpp:135-144)
            if self.steps % 10 == 0:
                self.nlist = O.StoredList(s, NB_CUTOFF + wl["padding"], threads)
            _, ff = O.nonbonded_list(s, self.nlist, O.nb_params(Cutoff=NB_CUTOFF, InnerCutoff=10, Vdw14Scaling=s14v,
                                                                Elec14Scaling=s14e,
                                                                ListCutoff=NB_CUTOFF + wl["padding"]), threads)
            f += ff
        if "GB" in wl["what"]:
            P = sub.gb_P
            gp = O.gb_params(Cutoff=999, InnerCutoff=998, VdwCutoff=999, VdwInnerCutoff=998, Vdw14Scaling=s14v,
                             Elec14Scaling=s14e, GbsaStillCutoff=999, P1=P[0], P2=P[1], P3=P[2], P4=P[3], P5=P[4],
                             ListCutoff=999 + wl["padding"])
            _, ff, _ = O.gb_forces(s, gp, sub.gb_radius, sub.gb_vj, sub.gb_terms123, threads)
            f += ff
        if "SA" in wl["what"]:
            if self.steps % 5 == 0:     # FF_SASA_LCPO::UpdateSasa (lcpo.cpp:193-206): cached between
                _, self.f_sa, _ = O.lcpo_forces(s, 999 + wl["padding"], sub.lcpo_radius, sub.lcpo_p, sub.lcpo_sigma,
                                                sub.lcpo_use, threads)
            f += self.f_sa
        if "BONDED" in wl["what"]:
            _, ff = O.bonded(self.pos, *sub.bonds, *sub.angles, *sub.torsions, *sub.impropers)
            f += ff
        if wl["integrator"] == 1:
            self.pos, self.vel, _ = O.langevin_step(self.pos, self.vel, f, sub.mass, wl["dt"], 1e13, 300.0,
                                                    self.rng.standard_normal((sub.natom, 6)),
                                                    first_step=(self.steps == 0))
        else:
            self.pos, self.vel, _ = O.vv_step(self.pos, self.vel, f, sub.mass, wl["dt"])
        self.steps += 1


def _cpu_worker(conn, key, systems, threads):
    """One host process: loads the workload itself and steps its systems on
    every 'step' message, answering with the seconds it took."""
    sys.path.insert(0, ROOT)
    from oracle import pdoracle as O
    from pd_gb300.workspace import load_workload
    wl = WORKLOADS[key]
    image = load_workload(wl["image"])
    mine = [CPUSystem(O, image.subset(k) if image.nsystems > 1 else image, wl, threads, 1 + k) for k in systems]
    conn.send("ready")
    while True:
        msg = conn.recv()
        if msg != "step":
            break
        t0 = time.perf_counter()
        for c in mine:
            c.step()
        conn.send(time.perf_counter() - t0)
    conn.close()


class CPUWorkload:
    """PD's FP64 path (the oracle restatement) stepping EVERY system of the
    workload on the host cores: one worker process per core (PD is single-
    threaded; one independent process per core is how it runs a batch), systems
    dealt to workers largest cost first (n^2 for all-pairs GB, n for cutoff
    systems).  A single-system workload runs in one process over every host
    thread (the oracle's OpenMP loops).  One step = one MD step of every
    system; its time is the wall clock until the slowest worker is done.
    Workers are started with 'spawn', never forked from a process holding a
    CUDA context."""

    def __init__(self, image, wl, key):
        import multiprocessing as mp
        self.cores = os.cpu_count() or 1
        n = image.nsystems
        self.natom = image.natom
        self.nsystems = n
        if n == 1:
            groups, threads = [[0]], self.cores
        else:
            w = min(self.cores, n)
            cost = image.natoms.astype(np.float64) ** (2 if "GB" in wl["what"] else 1)
            load = np.zeros(w)
            groups = [[] for _ in range(w)]
            for k in np.argsort(-cost):
                j = int(np.argmin(load))
                groups[j].append(int(k))
                load[j] += cost[k]
            threads = 1
        self.threads_used = len(groups) * threads
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for g in groups:
            a, b = ctx.Pipe()
            p = ctx.Process(target=_cpu_worker, args=(b, key, g, threads), daemon=True)
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        for c in self.conns:
            assert c.recv() == "ready"

    def step(self):
        t0 = time.perf_counter()
        for c in self.conns:
            c.send("step")
        for c in self.conns:
            c.recv()
        return time.perf_counter() - t0

    def close(self):
        for c in self.conns:
            try:
                c.send("stop")
            except (OSError, BrokenPipeError):
                pass
        for p in self.procs:
            p.join(timeout=10)

    def describe(self, steps, seconds):
        how = ("one process per host core (%d processes, one thread each), systems dealt largest first" %
               len(self.procs) if self.nsystems > 1 else "one process, OpenMP over %d host threads" % self.threads_used)
        return ("MD steps of every system of the workload (%d systems, %d atoms): forces (PD's O(N^2) list kept "
                "10 steps for cutoff systems, all pairs for GB, LCPO every 5 steps) + FP64 integrator; %s; %d "
                "timed steps in %.2f s" % (self.nsystems, self.natom, how, steps, seconds))


def cpu_baseline(image, wl, key, steps=2, warmup=1):
    """A bounded sample of the same workload on the host cores: `warmup` + `steps`
    MD steps of every system (a few to tens of seconds)."""
    cw = CPUWorkload(image, wl, key)
    try:
        for _ in range(warmup):
            cw.step()
        ts = [cw.step() for _ in range(steps)]
    finally:
        cw.close()
    return {"value": image.natom * steps / sum(ts), "unit": "atom-steps/s", "cores": cw.threads_used,
            "kind": "port", "sample": cw.describe(steps, sum(ts))}


def workload_config(key, wl, image):
    """The `config` object of both arms: the workload and nothing about how an
    arm measured it."""
    return {"workload": key, "description": wl["desc"], "atoms": int(image.natom), "systems": int(image.nsystems),
            "l2": "flushed before every timed GPU step (256 MB write); host arm: not applicable",
            "parallelism": "replicas only"}


# ---------------------------------------------------------------------------
# the reference arm: PD's FP64 CPU path (oracle restatement) on the host cores
# ---------------------------------------------------------------------------
REF_BUDGET_S = 90.0


def run_reference(args, key, wl, image):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import pdoracle as O  # noqa: F401  (builds the C restatement if needed)
    cw = CPUWorkload(image, wl, key)
    # each step of the whole workload is timed; the run stops after the
    # requested steps or REF_BUDGET_S of timed steps (at least 3), so the arm
    # ends within minutes whatever --steps asks for (a C4 step takes ~2 s on 16 cores)
    try:
        for _ in range(min(args.warmup, 1)):
            cw.step()
        ts = []
        t0 = time.perf_counter()
        while len(ts) < args.steps and (len(ts) < 3 or time.perf_counter() - t0 < REF_BUDGET_S):
            ts.append(cw.step())
    finally:
        cw.close()
    t = float(np.median(ts))
    v = image.natom / t
    out = {"metric": METRIC, "value": v, "unit": "atom-steps/s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic systems built by PD (NewProtein + seeded compaction, TIP3P lattice)",
           "config": workload_config(key, wl, image),
           "cpu_baseline": {"value": v, "unit": "atom-steps/s", "cores": cw.threads_used, "kind": "port",
                            "sample": "median step of %d timed (of %d requested; %.0f s budget), " % (
                                len(ts), args.steps, REF_BUDGET_S) + cw.describe(len(ts), sum(ts)),
                            "cpu": cpu_model()},
           "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def cpu_model():
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu model", "hardware")):
                return ln.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def roofline_flops(census, dom):
    """Algorithmic FP32 flops of one launch of the dominant pair kernel, from the
    pair census (counts of each branch) and FLOPS."""
    if dom == "gb_pair":
        return FLOPS["gb_pair"] * census["gb"] + FLOPS["gb_term"] * census["gb_term"]
    return FLOPS["nb"] * census["nb"]


def list_build_bytes(image, stats, groups):
    """Algorithmic DRAM bytes of one list build: per atom the FP64 position read
    (24 B), the sorted-slot record written and read back (16 B position + 16 B
    parameters + 4 B index), the cell key written and read (8 B); per block its
    centre, extent, grid cell and row count (48 B); per tile its 32 B record
    written; per masked tile 32 lanes x 8 B of exclusion masks; per NB j-atom
    group 32 x 16 B entries."""
    n = image.natom
    ngroups = max(groups[1], 0)
    nblocks = stats["slots"] // 32
    return (n * (24 + 36 + 8) + nblocks * 48 + stats["tiles"] * 32 + stats["masked_tiles"] * 256 +
            ngroups * 32 * 16)


def run_list_scaling(args):
    """List build of the C2 box (peptide in TIP3P, 22,489 atoms, 62 A) replicated
    1x, 2x, 4x and 8x at the same density, one JSON line: per size the tiles, the
    bytes of the list arrays, the device memory the context holds, the build time
    (CUDA events, L2 flushed, mean of 10) and, for comparison, what arrays sized
    by every block pair (candidate flags, tiles, masks, NB groups) would hold."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import load_workload
    wl = WORKLOADS["c2"]
    base = load_workload(wl["image"])
    rows = []
    for reps in ((1, 1, 1), (2, 1, 1), (2, 2, 1), (2, 2, 2)):
        image = base.replicate(reps)
        b0 = ffi.device_allocations()[1]
        ctx = DeviceContext(image)
        configure(ctx, wl, image)
        ctx.set_positions(image.pos)
        held = ffi.device_allocations()[1] - b0
        ms = ctx.time_kernel("list", reps=10)
        tiles, cap, lbytes = ctx.list_tiles()
        nb = (image.natom + 31) // 32
        pairs = nb * (nb + 1) // 2
        all_pairs = pairs * (32 + 4 + 4 + 1 + 8 + 256) + min(32 * pairs + 32 * nb, 8192 * nb) * 16
        rows.append({"replicas": int(np.prod(reps)), "atoms": image.natom, "blocks": nb, "tiles": int(len(tiles)),
                     "tile_capacity": int(cap), "list_bytes": int(lbytes), "context_bytes": int(held),
                     "build_ms": ms, "block_pairs": pairs, "all_pairs_list_bytes": int(all_pairs)})
        ctx.close()
    print(json.dumps({"list_scaling": rows, "workload": "c2 replicated", "radius": NB_CUTOFF + wl["padding"]}))


def run_ours(args, key, wl, image):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = dist_init(world, "nccl")
    from pd_gb300 import ffi
    seed = 1000 + rank
    ctx, temps = make_context(image, wl, key, seed, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream())
    tuned = None
    if not args.no_autotune:
        tuned = ctx.autotune(trial_steps=10)
    natom = image.natom
    exch_every = 500 if key == "c4" else 0
    # warm-up (captures the step graphs)
    ctx.md_run(args.warmup)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    step0 = args.warmup
    launches0 = ctx.kernel_launches()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    ev = []
    exchanges = 0
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(k & 0xff)   # L2 flushed between steps (256 MB write > 126 MB L2)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s = step0 + k
            due = exch_every and (s + 1) % exch_every == 0
            ctx.md_enqueue(1, energy_on_last=bool(due))
            if due:
                ffi.check(ctx.lib.pdgpu_remd_exchange(ctx.h, (s // exch_every) % 2, None, None), "exchange")
                exchanges += 1
            e1.record(stream)
            ev.append((e0, e1))
        # REMD exchange attempts belong to the workload at one per exch_every steps.
        # When the window holds fewer than its share, one attempt (an energy step
        # plus the exchange sweep) is timed here and its extra cost over a plain
        # step is counted for the missing share.
        ex_extra = None
        if exch_every:
            owed = args.steps / exch_every - exchanges
            if owed > 0:
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                ctx.md_enqueue(1, energy_on_last=True)
                ffi.check(ctx.lib.pdgpu_remd_exchange(ctx.h, 0, None, None), "exchange")
                e1.record(stream)
                ex_pair = (e0, e1, owed)
    torch.cuda.synchronize()
    ctx.synchronize()
    clocks = sampler.stop()
    t_dev = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    exchange_info = None
    if exch_every:
        owed = args.steps / exch_every - exchanges
        exchange_info = {"every": exch_every, "in_window": exchanges}
        if owed > 0:
            e0, e1, owed = ex_pair
            t_ex = e0.elapsed_time(e1) / 1e3
            ex_extra = max(t_ex - t_dev / args.steps, 0.0)
            t_dev += owed * ex_extra
            exchange_info.update({"attempt_extra_ms": ex_extra * 1e3, "counted": owed,
                                  "how": "one attempt timed after the window; its extra cost over a plain step "
                                         "added %.2f times (steps / %d minus attempts in the window)" % (
                                             owed, exch_every)})
    launches = ctx.kernel_launches() - launches0
    # list rebuilds belong to the workload at one per UpdateNList steps (the
    # autotuned cadence; steps s with s % UpdateNList == 0 rebuild).  The window
    # holds however many fall inside it; the difference from its share is
    # charged (or credited) at the measured cost of one list build.
    nl = tuned["UpdateNList"] if tuned else 10
    rebuilds = sum(1 for s in range(step0, step0 + args.steps) if s % nl == 0)
    ms_build = ctx.time_kernel("list", reps=10)
    ctx.compute(flags(wl["what"]))   # Born radii etc. in the order of the list just built
    owed_builds = args.steps / nl - rebuilds
    t_dev += owed_builds * ms_build / 1e3
    rebuild_info = {"update_nlist": nl, "in_window": rebuilds, "share": args.steps / nl,
                    "build_ms": ms_build, "charged_ms": owed_builds * ms_build,
                    "how": "(steps / UpdateNList - rebuilds in the window) x the measured list-build time"}
    if dist is not None:
        dist.barrier()
    t_max, units = reduce_max_sum(dist, t_dev, float(natom) * args.steps)
    value = units / t_max

    # kernel rooflines (measured on the live state, L2 flushed before each launch)
    dom = "gb_pair" if "GB" in wl["what"] else "nb"
    ms_dom = ctx.time_kernel(dom, reps=10)
    census = ctx.pair_census()
    ms_int = ctx.time_kernel("integrate", reps=10)
    ms_list = ms_build
    list_stats = ctx.list_stats()
    groups = ctx.nb_groups()
    result = {}
    if rank == 0:
        fp32 = ffi.fp32_peak(local)
        peak = max(fp32["ffma_tflops"], fp32["ffma2_tflops"])
        flops = roofline_flops(census, dom)
        achieved = flops / (ms_dom / 1e3) / 1e12
        peaks = {}
        pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pk):
            peaks = json.load(open(pk))
        hbm = peaks.get("hbm_gbs", 6800.0)
        int_gbs = INTEGRATOR_BYTES * natom / (ms_int / 1e3) / 1e9
        kdom = "k_gb_pair" if dom == "gb_pair" else "k_nb_tiles"
        kint = "k_langevin" if wl["integrator"] else "k_vv"
        traffic = NCU_TRAFFIC.get(key, {})
        roof = {"bound": "fp32", "kernel": kdom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic.get(kdom), "traffic_unit": "bytes per launch (ncu)",
                "peak_source": "measured: FP32 FMA probe on this GPU (pdgpu_fp32_peak, best of FFMA %.1f / "
                               "FFMA2 %.1f TFLOP/s; SM clock in `clocks`)" % (fp32["ffma_tflops"],
                                                                              fp32["ffma2_tflops"]),
                "flops_per_launch": flops, "ms_per_launch": ms_dom, "census": census}
        if dom == "gb_pair":
            roof["flops"] = ("%d per pair inside the GB cutoff + %d per pair above ExpApproxThreshold "
                             "(GB cross term)" % (FLOPS["gb_pair"], FLOPS["gb_term"]))
        else:
            visited = 1024 * (max(groups[1], 0) + (groups[2] if groups[2] >= 0 else list_stats["tiles"]))
            roof["flops"] = "%d per pair inside the cutoff" % FLOPS["nb"]
            roof["visited_pairs"] = visited
            roof["in_cutoff_over_visited"] = census["nb"] / visited if visited else None
        result["roofline"] = roof
        result["hbm_roofline"] = {"bound": "hbm", "kernel": kint,
                                  "achieved": int_gbs, "peak": hbm, "unit": "GB/s", "frac": int_gbs / hbm,
                                  "traffic": traffic.get(kint), "traffic_unit": "bytes per launch (ncu)",
                                  "bytes_per_atom": INTEGRATOR_BYTES, "ms_per_launch": ms_int,
                                  "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
        lb = list_build_bytes(image, list_stats, groups)
        result["list_roofline"] = {"bound": "hbm", "kernel": "list build (all its kernels)", "bytes": lb,
                                   "ms_per_build": ms_list, "achieved": lb / (ms_list / 1e3) / 1e9, "peak": hbm,
                                   "unit": "GB/s", "frac": lb / (ms_list / 1e3) / 1e9 / hbm,
                                   "tiles": list_stats["tiles"], "masked_tiles": list_stats["masked_tiles"]}
    ctx.close()

    # plain single-system path on the same systems (rank 0, N=1 semantics per rank)
    plain = None
    if rank == 0 and image.nsystems > 1 and not args.no_plain:
        plain = run_plain(args, key, wl, image, torch, nl)

    # end to end through the C ABI with host buffers
    e2e = None
    if rank == 0 and not args.no_e2e:
        e2e = run_e2e(args, key, wl, image, torch, nl)

    if rank != 0:
        return
    out = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math / int64 fixed-point sums / f64 state",
           "data": "synthetic systems built by PD (NewProtein + seeded compaction, TIP3P lattice)",
           "config": workload_config(key, wl, image),
           "preparation": "untimed relaxation: %d Langevin steps at %.1f fs, friction %.0e/s, then "
                          "Maxwell-Boltzmann velocities" % (RELAX["steps"], RELAX["dt"] * 1e15, RELAX["fric"]),
           "timing": {"graphs": True, "exchanges_in_timed_region": exchanges, "exchange": exchange_info,
                      "rebuilds": rebuild_info, "autotune": tuned, "ranks": world},
           "gpu_launches": int(launches), "clocks": clocks}
    out.update(result)
    if plain:
        out["plain"] = plain
        out["batched_over_plain"] = value / plain["value"] if plain["value"] else None
    out["e2e"] = e2e or {"value": None, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    if not args.no_parity:
        out["parity"] = parity_check(image, wl, key)
    if not args.no_cpu and world == 1:
        out["cpu_baseline"] = cpu_baseline(image, wl, key, steps=args.cpu_steps)
    print(json.dumps(out))


def run_plain(args, key, wl, image, torch, update_nlist):
    """The single-system path on the same systems, as PD's REX_Local runs its
    replicas: one system at a time, each advanced a chunk of steps through its
    own context (graphs on), waiting for it before moving to the next."""
    ctxs = []
    for k in range(image.nsystems):
        sub = image.subset(k)
        c, _ = make_context(sub, wl, key, 2000 + k, update_nlist=update_nlist)
        ctxs.append(c)
    chunk = max(5, min(args.steps, 50))
    for c in ctxs:
        c.md_run(chunk)
    torch.cuda.synchronize()
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        for c in ctxs:
            c.md_run(chunk)
        times.append(time.perf_counter() - t0)
    el = sorted(times)[1]
    for c in ctxs:
        c.close()
    return {"value": image.natom * chunk / el, "unit": "atom-steps/s", "steps": chunk,
            "how": "one context per system (%d), each run %d steps in turn (PD REX_Local order), wall clock, "
                   "median of 3 passes" % (image.nsystems, chunk)}


def run_e2e(args, key, wl, image, torch, update_nlist):
    """Per step through the C ABI with page-locked host buffers: positions H2D,
    one MD step of every system, positions and kinetic energies D2H.  The copies
    and the step are queued on the context's stream in that order each step
    (pdgpu_set_positions_async, pdgpu_md_enqueue, pdgpu_get_kinetic_async,
    pdgpu_get_positions_async): step k+1 reads the positions step k wrote to the
    host buffer, and the host waits once per stretch (pdgpu_synchronize, which
    also collects the device status)."""
    from pd_gb300 import ffi
    ctx, _ = make_context(image, wl, key, 3000, use_graph=True, update_nlist=update_nlist)
    n = image.natom
    pos_h = ffi.host_array((n, 3))
    ke_h = ffi.host_array((image.nsystems,))
    # each timed stretch is whole list-rebuild windows, so it holds its share of rebuilds
    steps = max(3, min(args.steps, 100))
    steps = -(-steps // update_nlist) * update_nlist
    ctx.get_positions(out=pos_h)

    def run(k):
        for _ in range(k):
            ctx.set_positions_async(pos_h)
            ctx.md_enqueue(1)
            ctx.kinetic_async(ke_h)
            ctx.get_positions_async(pos_h)
        ctx.synchronize()

    run(2 * update_nlist + 3)   # warm: every step of a rebuild window, the same calls
    rates = []
    for _ in range(3):          # median of three timed stretches
        t0 = time.perf_counter()
        run(steps)
        rates.append(n * steps / (time.perf_counter() - t0))
    ok = bool(np.all(np.isfinite(pos_h)) and np.all(ke_h > 0))
    ctx.close()
    return {"value": float(np.median(rates)), "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * n,
            "d2h_bytes_per_step": 24 * n + 8 * image.nsystems, "steps": steps, "repeats": 3,
            "rebuilds_per_stretch": steps // update_nlist,
            "spread": [float(min(rates)), float(max(rates))], "host_results_valid": ok,
            "how": "copies and steps queued in stream order, one host wait per stretch"}


# ---------------------------------------------------------------------------
# C5: parameter fitting through the adjoint (not the headline metric)
# ---------------------------------------------------------------------------
def oracle_frame_loss(image, frames, tables, theta, target, thresh=-4.0):
    """The C5 loss of a few frames from the FP64 oracle (for the finite-difference check)."""
    from oracle import pdoracle as O
    from pd_gb300.adjoint import KCAL_TO_J
    q, r, e, R, V, T = [a.detach().cpu().numpy() for a in tables.atom_arrays(
        theta["radius"], theta["sqrt_well"], theta["charge"], theta["gb_radius"])]
    s14v, s14e = image.scaling14
    P = image.gb_P
    gp = O.gb_params(Cutoff=999, InnerCutoff=998, VdwCutoff=999, VdwInnerCutoff=998, Vdw14Scaling=s14v,
                     Elec14Scaling=s14e, GbsaStillCutoff=999, P1=P[0], P2=P[1], P3=P[2], P4=P[3], P5=P[4],
                     ExpApproxThreshold=thresh, ListCutoff=1001)
    threads = os.cpu_count() or 1
    tot = 0.0
    for f, pos in enumerate(frames):
        s = O.OracleSystem(pos, q, r, e, image.excl, tuple(image.box[0]))
        E, _, _ = O.gb_forces(s, gp, R, V, T, threads)
        tot += ((E[1] + E[2] + E[3] - float(target[f])) / KCAL_TO_J) ** 2
    return tot / len(frames)


def run_adjoint(args):
    """C5: 256 frames taken every 100 Langevin steps of C3; loss = mean over frames
    of (E(theta') - E(theta))^2 for the GB + LJ + Coulomb energy; Adam steps on
    per-type LJ radius / sqrt(well depth), per-type GB radius and per-atom
    charges through the adjoint kernels.  One timed step = energy + parameter
    gradient of every frame (one device call), the torch chain rule through the
    GB fixed terms and the per-type tables, and the Adam update."""
    import torch
    from pd_gb300 import ffi
    from pd_gb300.adjoint import FrameSet, ParamTables, frame_loss, perturb
    from pd_gb300.workspace import load_workload
    wl = WORKLOADS["c3"]
    image = load_workload(wl["image"])
    nframes, every = args.frames, 100
    ctx, _ = make_context(image, wl, "c3", 5, update_nlist=10)
    frames = []
    for _ in range(nframes):
        ctx.md_run(every)
        frames.append(ctx.get_positions())
    ctx.close()
    T = ParamTables(image, device="cuda")
    fs = FrameSet(image, frames, ffi.GB, gb_settings(image), padding=wl["padding"])
    with torch.no_grad():
        target = fs.energies(*T.atom_arrays(T.radius, T.sqrt_well, T.charge, T.gb_radius))
    theta0 = perturb(T, seed=5)
    logp = ("radius", "sqrt_well", "gb_radius")
    x0 = {k: v.detach() for k, v in theta0.items()}
    svar = {k: torch.zeros_like(x0[k], requires_grad=True) for k in logp}
    dq = torch.zeros_like(x0["charge"], requires_grad=True)
    opt = torch.optim.Adam(list(svar.values()) + [dq], lr=1e-2)

    def theta():
        th = {k: x0[k] * torch.exp(svar[k]) for k in logp}
        th["charge"] = x0["charge"] + 0.1 * (dq - dq.mean())
        return th

    def step():
        opt.zero_grad()
        loss = frame_loss(fs, T, theta(), target)
        loss.backward()
        opt.step()
        return float(loss.detach())

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    hist = [step() for _ in range(args.warmup)]
    launches0 = fs.ctx.kernel_launches()
    sampler = ClockSampler(0)
    sampler.start()
    t_steps = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hist.append(step())
        torch.cuda.synchronize()
        t_steps.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    launches = fs.ctx.kernel_launches() - launches0
    el = sum(t_steps)
    # finite-difference check of d loss / d theta on 32 parameters, loss over the
    # first frames.  PD's ExpApproxThreshold switch makes the energy jump where a
    # pair's u = -r^2/(4 a_i a_j) crosses it, and the Born radii move with the GB
    # radii, so differences across it do not converge; the check uses the
    # energy without that switch (threshold -1e30), on the GPU and in the oracle.
    nfd = min(8, nframes)
    smooth = -1e30
    fs8 = FrameSet(image, frames[:nfd], ffi.GB, dict(gb_settings(image), ExpApproxThreshold=smooth),
                   padding=wl["padding"])
    th = {k: v.detach().clone().requires_grad_(True) for k, v in theta0.items()}
    loss8 = frame_loss(fs8, T, th, target[:nfd])
    loss8.backward()
    rng = np.random.default_rng(32)
    worst, within = 0.0, 0
    checks = []
    left = 32
    for name in ("radius", "sqrt_well", "gb_radius", "charge"):
        g = th[name].grad.detach().cpu().numpy()
        x = th[name].detach()
        cand = np.flatnonzero(x.cpu().numpy() != 0)
        # 8 per-type parameters of each kind (fewer if the kind has fewer types), charges fill up to 32
        take = min(left if name == "charge" else 8, len(cand))
        left -= take
        for a in rng.choice(cand, take, replace=False):
            h = 1e-4 * (1.0 if name == "charge" else abs(float(x[a])))
            tp = {k: v.detach().clone() for k, v in th.items()}
            tm = {k: v.detach().clone() for k, v in th.items()}
            tp[name][a] += h
            tm[name][a] -= h
            fd = (oracle_frame_loss(image, frames[:nfd], T, tp, target, smooth) -
                  oracle_frame_loss(image, frames[:nfd], T, tm, target, smooth)) / (2 * h)
            err = abs(g[a] - fd) / max(abs(fd), 1e-300)
            ok = abs(g[a] - fd) <= 1e-4 * abs(fd) + 1e-6 * float(np.max(np.abs(g)))
            within += int(ok)
            worst = max(worst, err)
            checks.append((name, int(a), float(g[a]), float(fd), bool(ok)))
    n_atoms = image.natom
    out = {"metric": "C5 adjoint: frame-atom energy+gradient evaluations/s inside Adam steps",
           "value": nframes * n_atoms * args.steps / el, "unit": "frame-atoms/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math / f64 energies and sums",
           "data": "synthetic: frames of the C3 peptide (%d atoms) every %d Langevin steps" % (n_atoms, every),
           "config": {"workload": "c5", "frames": nframes, "atoms_per_frame": n_atoms,
                      "parameters": {k: int(v.numel()) for k, v in theta0.items()},
                      "l2": "flushed before every timed step (256 MB write)",
                      "timing": "wall clock per Adam step with device synchronisation on both sides"},
           "loss": {"first": hist[0], "last": hist[-1], "steps": len(hist)},
           "fd_check": {"parameters": len(checks), "within_tolerance": within, "worst_rel_err": worst,
                        "frames": nfd, "h": "1e-4 (relative; absolute e for charges)",
                        "tolerance": "|g-fd| <= 1e-4|fd| + 1e-6 max|g|", "samples": checks[:4],
                        "energy": "GB without the ExpApproxThreshold switch (discontinuous in the Born radii)",
                        "outside": [c for c in checks if not c[4]]},
           "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(out))


# full run lengths of the workloads (steps) and the interval of the oracle checks
LONG = {"c1": (1000, 100), "c2": (10000, 1000), "c3": (5000, 500), "c4": (20000, 2000)}


def run_long(args, key, wl, image):
    """The workload's full run (C1 1,000 VV steps, C2 10,000 and C3 5,000 Langevin
    steps, C4 20,000 steps with REMD exchange attempts every 500), with the GPU's
    energy and forces checked against the FP64 oracle at fixed intervals on the
    trajectory's own positions.  Not a timing run: one JSON line of the checks."""
    ctx, temps = make_context(image, wl, key, 4242)
    tuned = ctx.autotune(trial_steps=10)   # the list cadence and launch shape of the timed runs
    steps, every = LONG[key]
    exch_every = 500 if key == "c4" else 0
    from pd_gb300 import ffi
    checks, accepted, attempts, stale = [], 0, 0, 0
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        n = min(every, steps - done)
        left = n
        while left > 0:
            chunk = left
            if exch_every:
                chunk = min(left, exch_every - done % exch_every)
            due = exch_every and (done + chunk) % exch_every == 0
            try:
                ctx.md_run(chunk, energy_on_last=bool(due))
            except ffi.PDGPUError as e:
                if e.status != ffi.ERR_STALE_LIST:
                    raise
                stale += 1           # an atom moved past half the skin: rebuild and go on (counted)
                ctx.rebuild_list()
            done += chunk
            left -= chunk
            if due:
                par = (done // exch_every) % 2
                acc, _ = ctx.remd_exchange(par)
                accepted += int(np.sum(acc[par::2]))     # rungs (par, par+1), (par+2, par+3), ...
                attempts += len(acc[par::2])
        ke = ctx.kinetic()
        t_sys = 2.0 * ke / (3.0 * image.natoms * 1.380649e-23)
        chk = parity_check(image, wl, key, pos=ctx.get_positions())
        checks.append({"step": done, "force_rel_rms": chk["force_rel_rms"], "energy_rel_err": chk["energy_rel_err"],
                       "mean_temperature_K": float(np.mean(t_sys))})
    ctx.close()
    out = {"workload": key, "steps": steps, "check_every": every, "system_atoms": chk["system_atoms"],
           "checks": checks, "max_force_rel_rms": max(c["force_rel_rms"] for c in checks),
           "max_energy_rel_err": max(c["energy_rel_err"] for c in checks), "wall_s": time.perf_counter() - t0,
           "target": "force rel RMS <= 1e-5, |dE|/|E| <= 1e-6 vs the FP64 oracle", "autotune": tuned,
           "stale_list_events": stale}
    if exch_every:
        out["exchange_attempts"] = attempts
        out["exchanges_accepted"] = accepted
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--workload", default="c4", choices=sorted(WORKLOADS) + ["c5"])
    ap.add_argument("--frames", type=int, default=256, help="c5: frames of the C3 trajectory")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=2, help="timed steps of the CPU baseline sample")
    ap.add_argument("--long", action="store_true",
                    help="the workload's full run length with oracle checks at intervals (validation, not timing)")
    ap.add_argument("--list-scaling", action="store_true",
                    help="list build memory and time on the C2 box replicated 1x-8x (one JSON line)")
    ap.add_argument("--relax-steps", type=int, default=RELAX["steps"],
                    help="untimed relaxation steps before timing (0 for short profiling runs)")
    args = ap.parse_args()
    RELAX["steps"] = args.relax_steps
    args.warmup = max(args.warmup, 3)
    from pd_gb300.workspace import load_workload
    if args.list_scaling:
        from pd_gb300 import build as _b
        _b.build()
        run_list_scaling(args)
        return
    if args.workload == "c5":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "PD has no parameter gradient; its derivative is "
                              "a finite difference of calcEnergies (c5 is checked against that in fd_check)"}))
            return
        from pd_gb300 import build as _b
        _b.build()
        run_adjoint(args)
        return
    wl = WORKLOADS[args.workload]
    image = load_workload(wl["image"])
    if args.impl == "reference":
        run_reference(args, args.workload, wl, image)
    else:
        from pd_gb300 import build as _b
        _b.build()
        if args.long:
            run_long(args, args.workload, wl, image)
        else:
            run_ours(args, args.workload, wl, image)


if __name__ == "__main__":
    main()
