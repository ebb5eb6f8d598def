"""pdgpu_param_grad_device_noalloc, the gradient call for hosts that cannot let
a call allocate device memory (cudaMalloc synchronises the whole device, or
their own pool holds the free memory), against pdgpu_param_grad_device, two
calls in a row, through the C ABI.

The allocation-free calls run first, on a fresh context of their own, and the
library's allocation counter (pdgpu_device_allocations) must not move across
them; the allocating entry point then runs on a second context of the same
system.  The file name sorts last, so a run that stops at the first failure
has run every other test before this one; it also passes alone in a fresh
process.  Tolerance: both entry points run the same kernels on the same list,
so the gradients agree to 1e-12 relative (in practice bit for bit)."""
import ctypes

import numpy as np
import pytest

from helpers import gb_kwargs, nb_kwargs

pytestmark = pytest.mark.gpu

NAMES = ("charge", "radius", "epsilon", "gb_radius", "gb_vj", "gb_terms123")


def _ctx(d, image=None):
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    ctx = DeviceContext(image if image is not None else SystemImage._from_fixture(d))
    ctx.set_list(float(d["cfg_padding"][0]))
    return ctx


def _grads(ctx, what, entry):
    import torch
    from pd_gb300 import ffi
    out = {n: torch.full((ctx.natom,), float("nan"), dtype=torch.float64, device="cuda") for n in NAMES}
    torch.cuda.synchronize()
    g = ffi.ParamGrads(*[out[n].data_ptr() for n in NAMES])
    ffi.check(getattr(ctx.lib, entry)(ctx.h, what, ctypes.byref(g)), entry)
    ctx.synchronize()
    E = ctx.energies()
    return {n: t.cpu().numpy() for n, t in out.items()}, E


def _setup(goldens, case):
    from pd_gb300 import ffi
    if case == "gb":
        d = goldens["peptide30"]
        ctx = _ctx(d)
        ctx.set_gb(**gb_kwargs(d))
        what = ffi.GB
    else:
        d = goldens["water_c1"]
        ctx = _ctx(d)
        ctx.set_nb(**nb_kwargs(d, "nbfswitch"))
        what = ffi.NB
    ctx.set_positions(d["pos"])
    return ctx, what


@pytest.mark.parametrize("case", ["gb", "nb"])
def test_noalloc_matches_allocating_entry(goldens, case):
    from pd_gb300 import ffi
    fresh, what = _setup(goldens, case)
    got = []
    for _ in range(2):
        import torch
        torch.cuda.synchronize()
        n0, b0 = ffi.device_allocations()
        got.append(_grads(fresh, what, "pdgpu_param_grad_device_noalloc"))
        n1, b1 = ffi.device_allocations()
        assert (n1, b1) == (n0, b0), "the allocation-free entry point allocated device memory"
    fresh.close()
    other, _ = _setup(goldens, case)
    ref, e_ref = _grads(other, what, "pdgpu_param_grad_device")
    other.close()
    for g, e in got:
        for n in NAMES:
            assert np.all(np.isfinite(g[n])), n
            scale = max(float(np.max(np.abs(ref[n]))), 1e-300)
            assert np.max(np.abs(g[n] - ref[n])) <= 1e-12 * scale, n
        for k in ("vdw", "elec", "pol", "epot"):
            assert e[0][k] == e_ref[0][k], k


def test_noalloc_rejects_contexts_beyond_its_scratch(goldens):
    """At most 65,536 sorted slots: a 40-copy batch of the 120-residue peptide is
    refused before anything is queued, and the context stays usable."""
    import torch
    from pd_gb300 import ffi
    from pd_gb300.workspace import SystemImage
    d = goldens["peptide120"]
    im = SystemImage.concat([SystemImage._from_fixture(d)] * 40)
    ctx = _ctx(d, im)
    ctx.set_gb(**gb_kwargs(d))
    ctx.set_positions(np.concatenate([d["pos"]] * 40))
    assert ctx.list_stats()["slots"] > 65536
    out = torch.zeros(im.natom, dtype=torch.float64, device="cuda")
    g = ffi.ParamGrads(out.data_ptr(), None, None, None, None, None)
    st = ctx.lib.pdgpu_param_grad_device_noalloc(ctx.h, ffi.GB, ctypes.byref(g))
    assert st == ffi.ERR_CAPACITY
    assert b"static scratch" in ctx.lib.pdgpu_error_string(st)
    assert float(out.abs().sum()) == 0.0
    ctx.compute(ffi.GB)   # still usable through the allocating path
    ctx.close()
