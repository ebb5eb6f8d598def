"""Failure statuses planted on the host, through the C ABI: each evaluation
returns its status (PD would throw its exception there) and leaves the context
usable for the next evaluation.  No input here can fault the device: the
kernels clamp what they write and only set status bits.

  PDGPU_ERR_FIXED_OVERFLOW  a pair force beyond the 64-bit fixed-point range
                            (two charges of 50 e 0.05 A apart: ~3e8 kcal/mol/A,
                            above the 2^28 kcal/mol/A per partial sum)
  PDGPU_ERR_LIST_OVERFLOW   an LCPO candidate list beyond its capacity (343
                            atoms on a 0.5 A lattice: every atom overlaps 342
                            others, past the 160 candidates kept to reproduce
                            PD's first-80 neighbour list, lcpo.h:24)
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _image(pos, charge, lcpo=None):
    from pd_gb300.workspace import SystemImage
    n = len(pos)
    kw = {}
    if lcpo is not None:
        radius, P, sigma = lcpo
        kw = dict(lcpo_radius=np.full(n, radius), lcpo_p=np.tile(P, (n, 1)), lcpo_sigma=np.full(n, sigma),
                  lcpo_use=np.ones(n, np.int32))
    return SystemImage([n], np.zeros(3), charge, np.full(n, 1.5), np.zeros(n), np.full(n, 2e-26),
                       np.zeros((0, 3), np.int32), pos=pos, **kw)


def test_fixed_point_overflow_is_reported_and_the_context_recovers():
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    close = np.array([[0.0, 0.0, 0.0], [0.05, 0.0, 0.0]])
    im = _image(close, np.array([50.0, -50.0]))
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_nb(Cutoff=12.0, InnerCutoff=10.0, VdwCutoff=12.0, VdwInnerCutoff=10.0, Vdw14Scaling=0.5,
               Elec14Scaling=0.83333, Dielectric=1.0, EnergySwitch=1, ForceSwitch=0, DoVdw=1, DoElec=1)
    ctx.set_positions(close)
    f = np.zeros((2, 3))
    with pytest.raises(ffi.PDGPUError) as err:
        ctx.compute(ffi.NB, f)
    assert err.value.status == -4          # PDGPU_ERR_FIXED_OVERFLOW
    # the same context, atoms 4 A apart (moved past the skin: new list, as PD's
    # calcNewList): plain Coulomb (no switching inside 10 A)
    far = np.array([[0.0, 0.0, 0.0], [4.0, 0.0, 0.0]])
    ctx.set_positions(far)
    ctx.rebuild_list()
    f = np.zeros((2, 3))
    e = ctx.compute(ffi.NB, f)[0]
    kcal = 4184.0 / 6.0221418E23
    econv = 332.0637 * kcal                 # e^2 / (4 pi eps0 A) in J (PD forcefield.cpp:35-55)
    assert abs(e["elec"] / (-2500.0 * econv / 4.0) - 1) < 1e-4
    assert f[0, 0] > 0 and abs(f[0, 0] + f[1, 0]) <= 1e-6 * abs(f[0, 0])
    ctx.close()


def test_lcpo_candidate_overflow_is_reported_and_the_context_recovers():
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    d = golden("peptide30")
    heavy = int(np.flatnonzero(d["lcpo_use"])[0])
    lcpo = (float(d["lcpo_radius"][heavy]), d["lcpo_P"][heavy], float(d["lcpo_sigma"][heavy]))
    g = np.arange(7, dtype=np.float64)
    dense = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) * 0.5
    im = _image(dense, np.zeros(len(dense)), lcpo)
    ctx = DeviceContext(im)
    ctx.set_list(2.0)
    ctx.set_positions(dense)
    with pytest.raises(ffi.PDGPUError) as err:
        ctx.compute(ffi.SA)
    assert err.value.status == -3          # PDGPU_ERR_LIST_OVERFLOW
    # the same atoms 8 A apart: no overlaps, every atom keeps its full sphere
    ctx.set_positions(dense * 16.0)
    ctx.rebuild_list()
    e = ctx.compute(ffi.SA)[0]
    sasa = ctx.sasa()
    r = lcpo[0]
    P1 = float(lcpo[1][0])
    assert np.allclose(sasa, P1 * 4.0 * np.pi * r * r, rtol=1e-6)
    assert e["surf"] > 0
    ctx.close()
