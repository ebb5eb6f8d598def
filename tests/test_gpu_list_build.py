"""The tile list, which the list build finds through a grid over block centres,
against an all-pairs scan of the same blocks on the host; and the list's
memory and build time on replicated copies of the C2 box.

Tile rule: block pair (bi, bj), bi <= bj, of one system is a tile when the
bounding boxes of the two blocks' atoms come within the list radius
R = max(cutoffs) + Padding.  The boxes are taken over positions wrapped into
the box when periodic, grown by 1e-4 A, and the separation of their centres is
taken at the minimum image.  The device decides in FP32, 1e-3 A to the safe
side; the host scan below is in FP64, so it checks that:
  - every pair closer than R - 1e-3 A is a tile (the grid misses nothing);
  - every tile is closer than R + 2e-3 A (nothing stray);
  - each row's tiles sit together with ascending columns (rows take their
    places in the list by an atomic, in any order), and no pair comes twice.
"""
import numpy as np
import pytest

from conftest import golden
from helpers import gb_kwargs, nb_kwargs

pytestmark = pytest.mark.gpu


def _blocks(ctx, image):
    """Block centres and half-extents from the device's slot order, as the list build forms them."""
    slots = ctx.list_slots()
    nb = len(slots) // 32
    pos = image.pos.copy()
    offs = image.offsets
    sys_of_atom = np.repeat(np.arange(image.nsystems), image.natoms)
    centre = np.zeros((nb, 3))
    half = np.zeros((nb, 3))
    bsys = np.zeros(nb, dtype=np.int64)
    for b in range(nb):
        a = slots[32 * b:32 * b + 32]
        a = a[a >= 0]
        s = int(sys_of_atom[a[0]])
        x = pos[a]
        L = image.box[s]
        if np.all(L > 0):
            x = x - L * np.floor(x / L)
        lo, hi = x.min(0), x.max(0)
        centre[b] = 0.5 * (lo + hi)
        half[b] = 0.5 * (hi - lo) + 1e-4
        bsys[b] = s
    return centre, half, bsys, offs


def _box_distance(centre, half, box, bi, bj):
    d = centre[bj] - centre[bi]
    if np.all(box > 0):
        d = d - box * np.rint(d / box)
    g = np.maximum(np.abs(d) - (half[bi] + half[bj]), 0.0)
    return np.sqrt((g * g).sum(-1))


def _check_list(ctx, image, R):
    tiles, cap, _ = ctx.list_tiles()
    centre, half, bsys, _ = _blocks(ctx, image)
    bi, bj = tiles[:, 0].astype(np.int64), tiles[:, 1].astype(np.int64)
    # each row contiguous with ascending columns, each pair once
    starts = np.flatnonzero(np.r_[True, bi[1:] != bi[:-1]])
    assert len(starts) == len(np.unique(bi)), "a row's tiles are split"
    same = bi[1:] == bi[:-1]
    assert np.all(bj[1:][same] > bj[:-1][same])
    key = bi * len(centre) + bj
    assert len(np.unique(key)) == len(key)
    assert np.all(bj >= bi) and np.all(bsys[bi] == bsys[bj])
    assert len(tiles) <= cap
    got = set(key.tolist())
    for s in range(image.nsystems):
        blk = np.flatnonzero(bsys == s)
        I, J = np.triu_indices(len(blk))
        gi, gj = blk[I], blk[J]
        dist = _box_distance(centre, half, image.box[s], gi, gj)
        must = gi[dist < R - 1e-3] * len(centre) + gj[dist < R - 1e-3]
        assert set(must.tolist()) <= got, "a block pair inside the list radius is missing"
        # tiles of this system, all within the radius
        mine = (bsys[bi] == s)
        d_t = _box_distance(centre, half, image.box[s], bi[mine], bj[mine])
        assert np.all(d_t < R + 2e-3), float(d_t.max())
    return len(tiles)


def test_periodic_solvated_list_matches_all_pairs_scan():
    """C2 (peptide in TIP3P, 62 A box, 14 A list radius) and the same box
    replicated 2x along x: the grid path with periodic wrap of the cell range."""
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import load_workload
    d = golden("cfg_c2")
    im = load_workload(str(d["image"]))
    for image in (im, im.replicate((2, 1, 1))):
        ctx = DeviceContext(image)
        ctx.set_list(float(d["cfg_padding"][0]))
        ctx.set_nb(**nb_kwargs(d, "nb"))
        ctx.set_positions(image.pos)
        ctx.rebuild_list()
        R = max(float(d["nb_Cutoff"][0]), float(d["nb_VdwCutoff"][0])) + float(d["cfg_padding"][0])
        n = _check_list(ctx, image, R)
        assert n > 0
        ctx.close()


def test_open_space_batch_list_matches_all_pairs_scan():
    """Two peptides of the C4 batch (525 and 7,741 atoms) as one batch in open
    space, at a 12 A cutoff (the grid over each system's own bounding box), and
    at all pairs (every row walks its columns directly)."""
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage, load_workload
    ds = [golden("cfg_c4_small"), golden("cfg_c4_large")]
    subs = [load_workload(str(d["image"])).subset(int(d["system"][0])) for d in ds]
    im = SystemImage.concat(subs)
    for cutoff in (12.0, 999.0):
        ctx = DeviceContext(im)
        ctx.set_list(2.0)
        kw = gb_kwargs(ds[0])
        kw.update(Cutoff=cutoff, InnerCutoff=cutoff - 2.0, VdwCutoff=cutoff, VdwInnerCutoff=cutoff - 2.0)
        ctx.set_gb(**kw)
        ctx.set_positions(im.pos)
        ctx.rebuild_list()
        n = _check_list(ctx, im, cutoff + 2.0)
        if cutoff > 100:
            nb = [(s.natom + 31) // 32 for s in subs]
            assert n == sum(b * (b + 1) // 2 for b in nb)
        ctx.close()


NB_OPEN = dict(Cutoff=12.0, InnerCutoff=10.0, VdwCutoff=12.0, VdwInnerCutoff=10.0, Vdw14Scaling=0.5,
               Elec14Scaling=0.83333, Dielectric=1.0, EnergySwitch=1, ForceSwitch=0, DoVdw=1, DoElec=1)


def test_list_grows_when_atoms_gather():
    """The largest C4 peptide (7,741 atoms, open space, 12 A cutoff): the first
    positions, spread to twice their extent, size the list; at the peptide's
    own positions the next build needs more tiles, grows the arrays, and the
    evaluation equals a fresh context's."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import load_workload
    d = golden("cfg_c4_large")
    im = load_workload(str(d["image"])).subset(int(d["system"][0]))
    centre = im.pos.mean(0)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_nb(**NB_OPEN)
    ctx.set_positions(centre + (im.pos - centre) * 2.0)
    _, cap0, _ = ctx.list_tiles()
    ctx.set_positions(im.pos)
    ctx.rebuild_list()
    tiles, cap1, _ = ctx.list_tiles()
    assert len(tiles) > cap0 and cap1 >= len(tiles), (cap0, len(tiles), cap1)
    _check_list(ctx, im, 14.0)
    f = np.zeros((im.natom, 3))
    e = ctx.compute(ffi.NB, f)[0]
    ctx.close()
    ref = DeviceContext(im)
    ref.set_list(2.0)
    ref.set_nb(**NB_OPEN)
    ref.set_positions(im.pos)
    f0 = np.zeros((im.natom, 3))
    e0 = ref.compute(ffi.NB, f0)[0]
    ref.close()
    for k in ("vdw", "elec", "epot"):
        assert abs(e[k] - e0[k]) <= 1e-12 * abs(e0[k]), (k, e[k], e0[k])
    assert np.array_equal(f, f0)


def test_list_memory_scales_linearly_with_the_box():
    """C2 replicated 1x, 2x and 4x (22,489 to 89,956 atoms at the same density):
    the bytes held by the list arrays grow in proportion to the atoms."""
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import load_workload
    d = golden("cfg_c2")
    im = load_workload(str(d["image"]))
    per_atom = []
    for reps in ((1, 1, 1), (2, 1, 1), (2, 2, 1)):
        image = im.replicate(reps)
        ctx = DeviceContext(image)
        ctx.set_list(float(d["cfg_padding"][0]))
        ctx.set_nb(**nb_kwargs(d, "nb"))
        ctx.set_positions(image.pos)
        tiles, cap, nbytes = ctx.list_tiles()
        per_atom.append((nbytes / image.natom, len(tiles) / image.natom))
        ctx.close()
    b1, t1 = per_atom[0]
    for b, t in per_atom[1:]:
        assert b <= 1.25 * b1, per_atom
        assert abs(t / t1 - 1) < 0.15, per_atom


def test_tile_overflow_inside_a_device_sized_build_is_reported_and_recovers():
    """A build that cannot read the tile count back (as inside a captured
    dynamics step) and finds more tiles than the arrays hold writes a short
    list and reports PDGPU_ERR_LIST_OVERFLOW; the next host-side rebuild grows
    the arrays and the evaluation equals a fresh context's."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import load_workload
    d = golden("cfg_c4_large")
    im = load_workload(str(d["image"])).subset(int(d["system"][0]))
    centre = im.pos.mean(0)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_nb(**NB_OPEN)
    ctx.set_positions(centre + (im.pos - centre) * 2.0)   # sizes the list on a spread copy
    tiles0, cap0, _ = ctx.list_tiles()
    ctx.set_positions(im.pos)
    ctx.time_kernel("list", reps=1, flush_l2=False)        # a build without the host round trip
    with pytest.raises(ffi.PDGPUError) as err:
        ctx.synchronize()
    assert err.value.status == -3                          # PDGPU_ERR_LIST_OVERFLOW
    tiles, cap, _ = ctx.list_tiles()
    assert cap == cap0 and len(tiles) == cap0              # the short list fills the arrays
    ctx.rebuild_list()
    tiles, cap1, _ = ctx.list_tiles()
    assert cap1 > cap0 and len(tiles) < cap1
    f = np.zeros((im.natom, 3))
    e = ctx.compute(ffi.NB, f)[0]
    ctx.close()
    ref = DeviceContext(im)
    ref.set_list(2.0)
    ref.set_nb(**NB_OPEN)
    ref.set_positions(im.pos)
    f0 = np.zeros((im.natom, 3))
    e0 = ref.compute(ffi.NB, f0)[0]
    ref.close()
    for k in ("vdw", "elec"):
        assert abs(e[k] - e0[k]) <= 1e-12 * abs(e0[k]), (k, e[k], e0[k])
    assert np.array_equal(f, f0)
