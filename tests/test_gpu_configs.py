"""The CUDA path at the benchmark workloads' own sizes, through the C ABI, against
PD's FP64 outputs written by PD itself at the very positions the workload images
hold (tests/golden/cfg_*.npz, made by tests/golden/make_golden.py --configs):

  cfg_c2        120-residue peptide in 6,844 TIP3P waters, 22,489 atoms, periodic
                62 A box: FF_NonBonded energy switch 12/10 A, 2 A skin (the only
                periodic system with a bonded solute: 1-2/1-3 exclusions and 1-4
                scaling meet per-pair minimum images here)
  cfg_c3        256-residue peptide, 4,235 atoms: GB (FastMode) + LCPO, all pairs
  cfg_c4_small  the smallest peptide of the 64-system batch (33 residues, 525 atoms)
  cfg_c4_large  the largest (478 residues, 7,741 atoms)

Tolerances per component: |dE|/|E| <= 1e-6, per-atom force relative RMS <= 1e-5
(PD's forces are stored as float32, a relative rounding of 6e-8).
"""
import hashlib

import numpy as np
import pytest

from conftest import golden, rel_err, rel_rms
from helpers import gb_kwargs, nb_kwargs, ref_energy

pytestmark = pytest.mark.gpu

E_TOL = 1e-6
F_TOL = 1e-5


def _image(d):
    """The workload image (or its system) PD evaluated, checked by position hash."""
    from pd_gb300.workspace import load_workload
    im = load_workload(str(d["image"]))
    k = int(d["system"][0])
    sub = im if k < 0 else im.subset(k)
    assert sub.natom == int(d["natoms"][0])
    h = hashlib.sha256(np.ascontiguousarray(sub.pos, dtype=np.float32).tobytes()).hexdigest()
    assert h == str(d["pos_sha256"]), "workload positions differ from the ones PD evaluated"
    return sub


def _ctx(image, d):
    from pd_gb300.engine import DeviceContext
    ctx = DeviceContext(image)
    ctx.set_list(float(d["cfg_padding"][0]))
    ctx.set_positions(image.pos)
    return ctx


def _check_gb(d, e, f, born=None):
    for k in ("vdw", "elec", "pol", "pol_self", "pol_cross", "epot"):
        assert rel_err(e[k], ref_energy(d, "gb", k)) <= E_TOL, (k, e[k], ref_energy(d, "gb", k))
    assert rel_rms(f, d["gb_f"]) <= F_TOL
    if born is not None:
        assert np.max(np.abs(born / d["gb_born"] - 1)) < 1e-6


def test_c2_solvated_nonbonded_matches_pd():
    """Energy kernel (groups on, as the autotuner picks for C2) and the force-only
    kernel the dynamics step runs, both against PD."""
    torch = pytest.importorskip("torch")
    from pd_gb300 import ffi
    d = golden("cfg_c2")
    im = _image(d)
    for groups in (1, 0):
        ctx = _ctx(im, d)
        ctx.set_nb(**nb_kwargs(d, "nb"))
        ctx.set_nb_groups(groups)
        f = np.zeros((im.natom, 3))
        e = ctx.compute(ffi.NB, f)[0]
        for k in ("vdw", "elec", "epot"):
            assert rel_err(e[k], ref_energy(d, "nb", k)) <= E_TOL, (groups, k, e[k], ref_energy(d, "nb", k))
        assert rel_err(e["virial"], ref_energy(d, "nb", "virial")) <= 1e-5
        assert rel_rms(f, d["nb_f"]) <= F_TOL
        fd = torch.zeros((im.natom, 3), dtype=torch.float64, device="cuda")
        ctx.compute_device(ffi.NB, fd.data_ptr())
        ctx.synchronize()
        assert rel_rms(fd.cpu().numpy(), d["nb_f"]) <= F_TOL
        if groups:
            assert ctx.nb_groups()[1] > 0
        ctx.close()


@pytest.mark.parametrize("name", ["cfg_c3", "cfg_c4_small", "cfg_c4_large"])
@pytest.mark.parametrize("tiles", [1, 2])
def test_gb_sa_workloads_match_pd(name, tiles):
    """Energy evaluation, and the force-only evaluation the dynamics step runs,
    against PD, with single tiles and with tile pairs as GB work items."""
    torch = pytest.importorskip("torch")
    from pd_gb300 import ffi
    d = golden(name)
    im = _image(d)
    ctx = _ctx(im, d)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_work_items(tiles)
    f = np.zeros((im.natom, 3))
    e = ctx.compute(ffi.GB, f)[0]
    _check_gb(d, e, f, ctx.born_radii())
    fd = torch.zeros((im.natom, 3), dtype=torch.float64, device="cuda")
    ctx.compute_device(ffi.GB, fd.data_ptr())
    ctx.synchronize()
    assert rel_rms(fd.cpu().numpy(), d["gb_f"]) <= F_TOL
    f = np.zeros((im.natom, 3))
    e = ctx.compute(ffi.SA, f)[0]
    assert rel_err(e["surf"], ref_energy(d, "sasa", "surf")) <= E_TOL
    assert np.max(np.abs(ctx.sasa() - d["lcpo_sasa"])) <= 1e-4 * max(1.0, float(np.max(d["lcpo_sasa"])))
    assert rel_rms(f, d["sasa_f"]) <= F_TOL
    ctx.close()


def test_c4_extremes_batched_match_pd():
    """The smallest and largest peptides of the C4 batch as one two-system batch
    (the concatenated layout the 64-system step uses), each against PD."""
    from pd_gb300 import ffi
    from pd_gb300.workspace import SystemImage
    ds = [golden("cfg_c4_small"), golden("cfg_c4_large")]
    subs = [_image(d) for d in ds]
    im = SystemImage.concat(subs)
    ctx = _ctx(im, ds[0])
    ctx.set_gb(**gb_kwargs(ds[0]))
    f = np.zeros((im.natom, 3))
    es = ctx.compute(ffi.GB | ffi.SA, f)
    o = 0
    for d, sub, e in zip(ds, subs, es):
        ref_e = ref_energy(d, "gb", "epot") + ref_energy(d, "sasa", "epot")
        assert rel_err(e["epot"], ref_e) <= E_TOL
        ref_f = d["gb_f"].astype(np.float64) + d["sasa_f"]
        assert rel_rms(f[o:o + sub.natom], ref_f) <= F_TOL
        o += sub.natom
    ctx.close()
