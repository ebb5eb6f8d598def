"""Parameter gradients on the GPU (pdgpu_param_grad through the C ABI, and the
torch autograd wrapper) against central finite differences of the oracle's
FP64 energies, as a force-field fit would check them.

Tolerance per checked entry: |g - fd| <= 1e-4 |fd| + 1e-6 max|g| (max over the
parameter array's entries), FP32 pair arithmetic with fixed-point sums against
FP64 differences."""
import numpy as np
import pytest

from helpers import gb_kwargs, gb_params, nb_kwargs, nb_params

pytestmark = pytest.mark.gpu

REL, ABS = 1e-4, 1e-6
NAMES = ("charge", "radius", "epsilon", "gb_radius", "gb_vj", "gb_terms123")
# finite-difference step: (size, relative to the entry's magnitude?)
STEP = {"charge": (1e-4, False), "radius": (1e-5, False), "epsilon": (1e-4, True), "gb_radius": (1e-5, False),
        "gb_vj": (1e-4, True), "gb_terms123": (1e-5, True)}


def make_ctx(d):
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    ctx = DeviceContext(SystemImage._from_fixture(d))
    ctx.set_list(float(d["cfg_padding"][0]))
    ctx.set_positions(d["pos"])
    return ctx


def oracle_gb(d, p):
    from oracle import pdoracle as O
    s = O.OracleSystem(d["pos"], p["charge"], p["radius"], p["epsilon"], d["excl"], tuple(d["box"]))
    E, _, _ = O.gb_forces(s, gb_params(d), p["gb_radius"], p["gb_vj"], p["gb_terms123"])
    return E[1] + E[2] + E[3]


def oracle_nb(d, tag, p):
    from oracle import pdoracle as O
    s = O.OracleSystem(d["pos"], p["charge"], p["radius"], p["epsilon"], d["excl"], tuple(d["box"]))
    E, _ = O.nonbonded(s, nb_params(d, tag))
    return E[1] + E[2]


def check_fd(base, grads, energy, names, npick, seed):
    rng = np.random.default_rng(seed)
    checked = 0
    for name in names:
        g = grads[name]
        scale = float(np.max(np.abs(g)))
        cand = np.flatnonzero(base[name] != 0) if STEP[name][1] else np.arange(len(g))
        for a in rng.choice(cand, npick, replace=False):
            h = STEP[name][0] * (abs(base[name][a]) if STEP[name][1] else 1.0)
            pp = {k: v.copy() for k, v in base.items()}
            pm = {k: v.copy() for k, v in base.items()}
            pp[name][a] += h
            pm[name][a] -= h
            fd = (energy(pp) - energy(pm)) / (2 * h)
            assert abs(g[a] - fd) <= REL * abs(fd) + ABS * scale, (name, int(a), g[a], fd, scale)
            checked += 1
    return checked


def test_gb_param_grad_matches_finite_differences(goldens):
    from pd_gb300 import ffi
    d = goldens["peptide30"]
    ctx = make_ctx(d)
    ctx.set_gb(**gb_kwargs(d))
    e, g = ctx.param_grad(ffi.GB)
    e_plain = ctx.compute(ffi.GB)[0]
    for k in ("vdw", "elec", "pol", "epot"):   # the gradient call's energies: FP32 pair terms, FP64 sums
        assert abs(e[0][k] - e_plain[k]) <= 1e-6 * abs(e_plain[k]), k
    base = {n: np.array(d[n], dtype=np.float64) for n in NAMES}
    n = check_fd(base, g, lambda p: oracle_gb(d, p), NAMES, 6, seed=11)
    assert n == 36


@pytest.mark.parametrize("tag", ["nb", "nbfswitch"])
def test_nb_param_grad_matches_finite_differences(goldens, tag):
    from pd_gb300 import ffi
    d = goldens["water_c1"]
    ctx = make_ctx(d)
    ctx.set_nb(**nb_kwargs(d, tag))
    e, g = ctx.param_grad(ffi.NB)
    for k in ("gb_radius", "gb_vj", "gb_terms123"):
        assert not np.any(g[k])
    base = {n: np.array(d[n], dtype=np.float64) for n in ("charge", "radius", "epsilon")}
    check_fd(base, g, lambda p: oracle_nb(d, tag, p), ("charge", "radius", "epsilon"), 6, seed=12)


def test_param_grad_batch_is_per_system(goldens):
    """In a batch each atom gets the gradient of its own system's energy."""
    from pd_gb300 import ffi
    from pd_gb300.engine import DeviceContext
    from pd_gb300.workspace import SystemImage
    names = ["peptide30", "peptide120"]
    batch = SystemImage.concat([SystemImage._from_fixture(goldens[n]) for n in names])
    ctx = DeviceContext(batch)
    ctx.set_list(2.0)
    ctx.set_gb(**gb_kwargs(goldens["peptide30"]))
    ctx.set_positions(np.concatenate([goldens[n]["pos"] for n in names]))
    _, gb = ctx.param_grad(ffi.GB)
    o = batch.offsets
    for k, n in enumerate(names):
        c1 = make_ctx(goldens[n])
        c1.set_list(2.0)
        c1.set_gb(**gb_kwargs(goldens["peptide30"]))
        _, g1 = c1.param_grad(ffi.GB)
        for name in NAMES:
            assert np.array_equal(gb[name][o[k]:o[k + 1]], g1[name]), name


def _frames(d, nframes, seed=7, sigma=0.05):
    rng = np.random.default_rng(seed)
    return np.stack([d["pos"] + sigma * rng.standard_normal(d["pos"].shape) for _ in range(nframes)])


def test_autograd_per_type_gradient_matches_oracle(goldens):
    """Loss = mean_f (E_f(theta) - E_f(theta0))^2 over 3 frames; d loss / d theta for
    per-type LJ radius, well depth, GB radius and per-atom charges against central
    differences of the same loss built from oracle energies."""
    import torch
    from oracle import pdoracle as O
    from pd_gb300 import ffi
    from pd_gb300.adjoint import KCAL_TO_J, FrameSet, ParamTables, frame_loss, perturb
    from pd_gb300.workspace import SystemImage
    d = goldens["peptide30"]
    im = SystemImage._from_fixture(d)
    T = ParamTables(im)
    frames = _frames(d, 3)
    fs = FrameSet(im, frames, ffi.GB, gb_kwargs(d), padding=2.0)
    off = float(d["gb_DielectricOffset"][0])
    with torch.no_grad():
        target = fs.energies(*[a.cuda() for a in T.atom_arrays(T.radius, T.sqrt_well, T.charge, T.gb_radius, off)])
    theta = perturb(T, seed=5)
    loss = frame_loss(fs, T, theta, target)
    loss.backward()

    def oracle_loss(th):
        q, r, e, R, V, Tt = [a.detach().numpy() for a in T.atom_arrays(th["radius"], th["sqrt_well"], th["charge"],
                                                                     th["gb_radius"], off)]
        tot = 0.0
        for f, pos in enumerate(frames):
            s = O.OracleSystem(pos, q, r, e, d["excl"], tuple(d["box"]))
            E, _, _ = O.gb_forces(s, gb_params(d), R, V, Tt)
            tot += ((E[1] + E[2] + E[3] - float(target[f])) / KCAL_TO_J) ** 2
        return tot / len(frames)

    rng = np.random.default_rng(21)
    for name, h in (("radius", 1e-6), ("sqrt_well", 1e-7), ("gb_radius", 1e-6), ("charge", 1e-6)):
        g = theta[name].grad.cpu().numpy()
        scale = float(np.max(np.abs(g)))
        cand = np.flatnonzero(theta[name].detach().cpu().numpy() != 0)
        for a in rng.choice(cand, min(8, len(cand)), replace=False):
            tp = {k: v.detach().clone() for k, v in theta.items()}
            tm = {k: v.detach().clone() for k, v in theta.items()}
            tp[name][a] += h
            tm[name][a] -= h
            fd = (oracle_loss(tp) - oracle_loss(tm)) / (2 * h)
            assert abs(g[a] - fd) <= REL * abs(fd) + ABS * scale, (name, int(a), g[a], fd)


def test_fit_reduces_loss(goldens):
    import torch
    from pd_gb300 import ffi
    from pd_gb300.adjoint import FrameSet, ParamTables, fit, perturb
    from pd_gb300.workspace import SystemImage
    d = goldens["peptide30"]
    im = SystemImage._from_fixture(d)
    T = ParamTables(im)
    fs = FrameSet(im, _frames(d, 8), ffi.GB, gb_kwargs(d), padding=2.0)
    off = float(d["gb_DielectricOffset"][0])
    with torch.no_grad():
        target = fs.energies(*[a.cuda() for a in T.atom_arrays(T.radius, T.sqrt_well, T.charge, T.gb_radius, off)])
    theta = perturb(T, seed=5)
    fitted, hist = fit(fs, T, theta, target, steps=40, lr=1e-2)
    assert np.all(np.isfinite(hist))
    assert hist[-1] < 0.25 * hist[0], hist[::5]
    assert abs(float(fitted["charge"].sum() - T.charge.sum())) < 1e-9
