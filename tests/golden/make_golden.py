"""Generate the golden fixtures and workload images from the compiled PD reference.

Runs here only (it needs the PD sources to build ``oracle/_ref/ref_driver``):

    make -C oracle ref REF=<PD checkout>
    PD_SOURCES=<PD checkout> python tests/golden/make_golden.py [--fixtures] [--workloads] [--configs]

``PD_SOURCES`` names the PD checkout (its ``param/`` directory holds the force
field files); ``PD_PARAM_PATH`` may name the parameter directory directly.

Outputs
-------
tests/golden/<case>.npz
    System description plus PD's own FP64 energies (J), forces (N), Born radii,
    per-atom SASA, neighbour-list checksums and pair-law scans for that system.
    These pin the C restatement in ``oracle/`` and the CUDA path.
tests/golden/cfg_<workload>.npz
    PD's FP64 energies, forces (stored as float32, a relative rounding of
    6e-8, far inside the 1e-5 force tolerance), Born radii and per-atom SASA
    for the benchmark workloads themselves: the solvated C2 box, the C3
    peptide and the smallest and largest C4 peptides, evaluated by PD at the
    very positions stored in the workload images (checked by a hash of their
    float32 bytes).
pd_gb300/workloads/<name>.npz
    Compact system images (float32-exact positions, per-atom parameter classes,
    exclusion table, bonded terms) for the benchmark workloads.  Positions were
    rounded to float32 inside the driver before anything was evaluated, so the
    stored float32 values are the exact inputs.

Every system is built by PD itself (``NewProtein``, ``NewMolecule("TIP3")``,
``setResiduePhiPsi``, PD's minimiser) from a fixed seed; the seeds and driver
options are listed below so the files can be regenerated bit for bit.
"""
import argparse
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
WORKLOADS = os.path.join(ROOT, "pd_gb300", "workloads")
sys.path.insert(0, HERE)
from refbin import read_container  # noqa: E402

FIXTURES = {
    # 667 TIP3P waters, jittered cubic lattice, 27.5 A periodic box, LJ+Coulomb 12/10 A, 2 A skin
    "water_c1": ("water", dict(seed=1, nwat=667, box=27.5, cutoff=12, inner=10, padding=2, elec="eswitch", scan=1)),
    # 30-residue peptide, GB (Cutoff 12 / Inner 9 / GbsaStillCutoff 10, FastMode) + LCPO + vacuum LJ/Coulomb
    "peptide30": ("peptide", dict(seed=3, nres=30, padding=2, gbcutoff=12, gbinner=9, gbsastill=10,
                                  cutoff=12, inner=10, elec="eswitch")),
    # same peptide, all pairs (every cutoff 999 / inner 998, no switching reached)
    "peptide30_ap": ("peptide", dict(seed=3, nres=30, padding=2, gbcutoff=999, gbinner=998, gbsastill=999,
                                     cutoff=999, inner=998, elec="eswitch")),
    # 120-residue peptide with the default GB cutoffs, force-switched vacuum electrostatics
    "peptide120": ("peptide", dict(seed=2, nres=120, padding=2, gbcutoff=12, gbinner=9, gbsastill=10,
                                   cutoff=12, inner=10, elec="fswitch")),
}
# extra electrostatics modes evaluated on an already generated fixture system
FIXTURE_VARIANTS = {
    "water_c1": [("fswitch", dict(elec="fswitch")), ("normal", dict(elec="normal")),
                 ("vdwsplit", dict(elec="eswitch", vdwcut=10, vdwinner=8))],
}

WORKLOAD_SPECS = {
    "c1_water": ("water", dict(seed=1, nwat=667, box=27.5, cutoff=12, inner=10, padding=2, elec="eswitch", gb=0, sasa=0)),
    "c2_solvated": ("solvated", dict(seed=2, nres=120, box=62, side=20, exclude=2.6, cutoff=12, inner=10,
                                     padding=2, elec="eswitch", gb=0, sasa=0)),
    "c3_gb256": ("peptide", dict(seed=3, nres=256, padding=2, gbcutoff=999, gbinner=998, gbsastill=999,
                                 cutoff=999, inner=998, nb=0)),
}
C4_SYSTEMS = 64
C4_SEED = 4


def param_path():
    """PD's parameter directory: PD_PARAM_PATH, else $PD_SOURCES/param."""
    if os.environ.get("PD_PARAM_PATH"):
        return os.environ["PD_PARAM_PATH"]
    src = os.environ.get("PD_SOURCES")
    if not src:
        sys.exit("set PD_SOURCES to the PD checkout (or PD_PARAM_PATH to its param/ directory)")
    return os.path.join(src, "param")


def run_driver(kind, opts):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out.bin")
        args = [DRIVER, kind, out] + ["%s=%s" % (k, v) for k, v in opts.items()]
        env = dict(os.environ)
        env.setdefault("PD_PARAM_PATH", param_path())
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, env=env)
        return read_container(out)


def make_fixtures():
    for name, (kind, opts) in FIXTURES.items():
        d = run_driver(kind, opts)
        for tag, extra in FIXTURE_VARIANTS.get(name, []):
            o = dict(opts)
            o.update(extra)
            o["scan"] = 0
            v = run_driver(kind, o)
            assert np.array_equal(v["pos"], d["pos"])
            for k in list(v):
                if k.startswith("nb_"):
                    d["nb%s_%s" % (tag, k[3:])] = v[k]
        d["gen_kind"] = np.array(kind)
        d["gen_opts"] = np.array(repr(sorted(opts.items())))
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **d)
        print("%-14s natoms=%6d  %7.1f kB" % (name, len(d["pos"]), os.path.getsize(path) / 1024))


# ---------------------------------------------------------------------------
# compact workload images
# ---------------------------------------------------------------------------
PER_ATOM_FLOAT = ["charge", "radius", "epsilon", "mass", "gb_radius", "gb_vj", "gb_terms123",
                  "lcpo_radius", "lcpo_sigma"]


def compact_image(d):
    n = len(d["pos"])
    cols = []
    for k in PER_ATOM_FLOAT:
        cols.append(d[k] if k in d else np.zeros(n))
    if "lcpo_P" in d:
        cols += [d["lcpo_P"][:, c] for c in range(4)]
        use = d["lcpo_use"].astype(np.float64)
    else:
        cols += [np.zeros(n)] * 4
        use = np.zeros(n)
    cols += [d["Z"].astype(np.float64), use]
    table = np.stack(cols, axis=1)
    uniq, cls = np.unique(table, axis=0, return_inverse=True)
    assert len(uniq) < 65536
    img = {
        "pos": d["pos"].astype(np.float32),
        "box": d["box"],
        "class_table": uniq,
        "class_cols": np.array(PER_ATOM_FLOAT + ["lcpo_P1", "lcpo_P2", "lcpo_P3", "lcpo_P4", "Z", "lcpo_use"]),
        "atom_class": cls.reshape(-1).astype(np.uint16),
        "excl_i": d["excl"][:, 0].astype(np.int32),
        "excl_dj": (d["excl"][:, 1] - d["excl"][:, 0]).astype(np.int32),
        "excl_bo": d["excl"][:, 2].astype(np.int8),
    }
    assert np.array_equal(d["pos"].astype(np.float32).astype(np.float64), d["pos"])
    for k in ("bond", "angle", "torsion", "improper"):
        idx, par = d[k + "_idx"], d[k + "_par"]
        up, pc = np.unique(par, axis=0, return_inverse=True)
        img[k + "_idx"] = idx.astype(np.int32)
        img[k + "_partable"] = up
        img[k + "_parclass"] = pc.reshape(-1).astype(np.uint16)
    for k in ("gb_P", "cfg_padding", "ires", "sequence"):
        if k in d:
            img[k] = d[k]
    for k in d:
        if k.endswith("_ene"):
            img["ref_" + k] = d[k]
    return img


def encode_indices(img):
    """Delta-encode the index arrays of an image: first atom of each row as the
    difference from the previous row, the other atoms relative to the first
    (all small integers, so the npz compresses them to almost nothing)."""
    out = dict(img)
    for k in ("bond", "angle", "torsion", "improper"):
        idx = img.pop(k + "_idx") if k + "_idx" in img else out.pop(k + "_idx")
        out.pop(k + "_idx", None)
        natom_cols = {"bond": 2, "angle": 3, "torsion": 4, "improper": 4}[k]
        first = idx[:, 0].astype(np.int64)
        out[k + "_first_delta"] = np.diff(first, prepend=0).astype(np.int32)
        out[k + "_rel"] = (idx[:, 1:natom_cols] - idx[:, :1]).astype(np.int16)
        if idx.shape[1] > natom_cols:
            out[k + "_terms"] = idx[:, natom_cols].astype(np.int8)
    ei = out.pop("excl_i")
    out["excl_first_delta"] = np.diff(ei.astype(np.int64), prepend=0).astype(np.int32)
    return out


def make_workloads(which):
    os.makedirs(WORKLOADS, exist_ok=True)
    for name, (kind, opts) in WORKLOAD_SPECS.items():
        if which and name not in which:
            continue
        d = run_driver(kind, opts)
        img = encode_indices(compact_image(d))
        path = os.path.join(WORKLOADS, name + ".npz")
        np.savez_compressed(path, **img)
        print("%-14s natoms=%6d  %7.1f kB" % (name, len(d["pos"]), os.path.getsize(path) / 1024))
    if not which or "c4_remd64" in which:
        make_c4()


def c4_residue_counts():
    """Residue counts floor(exp(U(ln 30, ln 500))) from a fixed numpy seed."""
    rng = np.random.default_rng(C4_SEED)
    return np.floor(np.exp(rng.uniform(math.log(30), math.log(500), size=C4_SYSTEMS))).astype(int)


def make_c4():
    counts = c4_residue_counts()
    parts = []
    for k, nres in enumerate(counts):
        d = run_driver("peptide", dict(seed=4000 + k, nres=int(nres), padding=2, gbcutoff=999, gbinner=998,
                                       gbsastill=999, cutoff=999, inner=998, nb=0, gb=1, sasa=1))
        parts.append(compact_image(d))
        print("  c4 system %2d: %3d residues, %5d atoms" % (k, nres, len(d["pos"])))
    # concatenate with a shared class table
    tables = [p["class_table"] for p in parts]
    allt = np.concatenate(tables)
    uniq, inv = np.unique(allt, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    off = 0
    img = {"box": np.zeros(3), "class_table": uniq, "class_cols": parts[0]["class_cols"]}
    pos, cls, natoms = [], [], []
    ex_i, ex_dj, ex_bo = [], [], []
    bonded = {k: ([], [], []) for k in ("bond", "angle", "torsion", "improper")}
    base = 0
    for p, t in zip(parts, tables):
        remap = inv[off:off + len(t)]
        off += len(t)
        pos.append(p["pos"])
        cls.append(remap[p["atom_class"]].astype(np.uint16))
        natoms.append(len(p["pos"]))
        ex_i.append(p["excl_i"] + base)
        ex_dj.append(p["excl_dj"])
        ex_bo.append(p["excl_bo"])
        for k in bonded:
            bonded[k][0].append(p[k + "_idx"] + np.where(np.arange(p[k + "_idx"].shape[1]) < (4 if k in ("torsion", "improper") else 99), base, 0))
            bonded[k][1].append(p[k + "_partable"])
            bonded[k][2].append(p[k + "_parclass"])
        base += len(p["pos"])
    img["pos"] = np.concatenate(pos)
    img["atom_class"] = np.concatenate(cls)
    img["system_natoms"] = np.array(natoms, dtype=np.int32)
    img["system_nres"] = counts.astype(np.int32)
    img["excl_i"] = np.concatenate(ex_i).astype(np.int32)
    img["excl_dj"] = np.concatenate(ex_dj).astype(np.int32)
    img["excl_bo"] = np.concatenate(ex_bo).astype(np.int8)
    for k, (idx, tabs, pcs) in bonded.items():
        allp = np.concatenate(tabs) if tabs else np.zeros((0, 2))
        up, pinv = np.unique(allp, axis=0, return_inverse=True)
        pinv = pinv.reshape(-1)
        o = 0
        classes = []
        for tb, pc in zip(tabs, pcs):
            classes.append(pinv[o:o + len(tb)][pc])
            o += len(tb)
        img[k + "_idx"] = np.concatenate(idx).astype(np.int32)
        img[k + "_partable"] = up
        img[k + "_parclass"] = np.concatenate(classes).astype(np.uint16)
    img["gb_P"] = parts[0]["gb_P"]
    img["cfg_padding"] = parts[0]["cfg_padding"]
    path = os.path.join(WORKLOADS, "c4_remd64.npz")
    np.savez_compressed(path, **encode_indices(img))
    print("%-14s natoms=%6d  %7.1f kB" % ("c4_remd64", len(img["pos"]), os.path.getsize(path) / 1024))


# ---------------------------------------------------------------------------
# goldens at the benchmark workloads' own sizes
# ---------------------------------------------------------------------------
def c4_system_opts(k):
    counts = c4_residue_counts()
    return dict(seed=4000 + k, nres=int(counts[k]), padding=2, gbcutoff=999, gbinner=998, gbsastill=999,
                cutoff=999, inner=998, nb=0, gb=1, sasa=1)


def config_golden_specs():
    """name -> (driver kind, driver options, workload image, system index or None)."""
    counts = c4_residue_counts()
    return {
        "cfg_c2": ("solvated", WORKLOAD_SPECS["c2_solvated"][1], "c2_solvated", None),
        "cfg_c3": ("peptide", WORKLOAD_SPECS["c3_gb256"][1], "c3_gb256", None),
        "cfg_c4_small": ("peptide", c4_system_opts(int(counts.argmin())), "c4_remd64", int(counts.argmin())),
        "cfg_c4_large": ("peptide", c4_system_opts(int(counts.argmax())), "c4_remd64", int(counts.argmax())),
    }


def pos_hash(pos):
    """sha256 of the positions as float32 (the workload images store them so)."""
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(pos, dtype=np.float32).tobytes()).hexdigest()


def make_config_goldens(which):
    sys.path.insert(0, ROOT)
    from pd_gb300.workspace import load_workload
    for name, (kind, opts, image, k) in config_golden_specs().items():
        if which and name not in which:
            continue
        d = run_driver(kind, opts)
        im = load_workload(image)
        sub = im if k is None else im.subset(k)
        assert len(d["pos"]) == sub.natom and np.array_equal(d["pos"], sub.pos.astype(np.float64)), name
        out = {"natoms": np.array([sub.natom]), "pos_sha256": np.array(pos_hash(sub.pos)),
               "image": np.array(image), "system": np.array([-1 if k is None else k]),
               "cfg_list_cutoff": d["cfg_list_cutoff"], "cfg_padding": d["cfg_padding"],
               "gen_kind": np.array(kind), "gen_opts": np.array(repr(sorted(opts.items())))}
        for tag in ("bonded", "nb", "gb", "sasa", "gbslow"):
            if tag + "_ene" in d:
                out[tag + "_ene"] = d[tag + "_ene"]
        for tag in ("nb", "gb", "sasa"):
            if tag + "_f" in d:
                out[tag + "_f"] = d[tag + "_f"].astype(np.float32)
        for key in d:
            if (key.startswith("nb_") or key.startswith("gb_")) and d[key].size == 1:
                out[key] = d[key]
        if "gb_P" in d:
            out["gb_P"] = d["gb_P"]
            out["gb_born"] = d["gb_born"].astype(np.float32)
        if "lcpo_sasa" in d:
            out["lcpo_sasa"] = d["lcpo_sasa"].astype(np.float32)
            out["lcpo_GlobalASP"] = d["lcpo_GlobalASP"]
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print("%-14s natoms=%6d  %7.1f kB" % (name, sub.natom, os.path.getsize(path) / 1024))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--fixtures", action="store_true")
    ap.add_argument("--workloads", nargs="*")
    ap.add_argument("--configs", nargs="*", help="goldens at the workloads' own sizes (cfg_*.npz)")
    a = ap.parse_args()
    if not os.path.exists(DRIVER):
        sys.exit("build the reference first: make -C oracle ref")
    if a.fixtures or (a.workloads is None and a.configs is None):
        make_fixtures()
    if a.workloads is not None:
        make_workloads(a.workloads)
    if a.configs is not None:
        make_config_goldens(a.configs)


if __name__ == "__main__":
    main()
