"""Parameter gradients of the nonbonded / GB energy and force-field fitting.

PD has no adjoint: a parameter derivative there is a finite difference of
``Forcefield::calcEnergies`` with ``setup()`` re-run after every edit
(src/mmlib/forcefields/nonbonded.cpp:1078-1084).  Here one device call
(``pdgpu_param_grad_device``) returns every system's energy and dE/dp for the
per-atom parameter arrays; this module wraps it as a ``torch.autograd.Function``
and adds the differentiable pieces PD computes once at set-up:

* per-type tables -> per-atom arrays (LJ Rmin/2 and well depth per LJ type,
  GB radius per GB type, charges per atom);
* the GB fixed terms Vj and terms123 from the GB radii
  (``FF_GeneralizedBorn_Still::calcFixedBornRadiiTerms``, gbff.cpp:324-398),
  restated in torch so the chain rule through them is automatic.

A frame set holds F snapshots of one system as F systems of one device context;
the energy of frame f is E_f(theta), and the gradient reaching a per-atom
parameter is summed over frames by autograd (the per-atom arrays are the
single-system arrays repeated F times).
"""
import math

import numpy as np
import torch

from . import ffi
from .engine import DeviceContext
from .workspace import SystemImage

KCAL_TO_J = 4184.0 / 6.0221418e23          # kcal/mol -> J per molecule (forcefield.cpp:35-55)
EPS_STORE = math.sqrt(4184.0 / 6.0221418e23)  # PD stores sqrt(eps in J): sqrt(kcal/mol) -> that unit


def covalent_pairs(image):
    """1-2 and 1-3 partner lists with PD's covalent distances: 1-2 at the bond's
    equilibrium length, 1-3 by the law of cosines from the two bond lengths and
    the angle's equilibrium value (both directions, in bond / angle order) —
    the ``cov12atom`` / ``cov13atom`` tables FF_Bonded fills at set-up."""
    bidx, bpar = image.bonds
    l0 = {}
    for (i, j), p in zip(bidx, bpar):
        l0[(int(i), int(j))] = l0[(int(j), int(i))] = float(p[0])
    c12 = np.concatenate([bidx[:, :2], bidx[:, [1, 0]]]) if len(bidx) else np.zeros((0, 2), np.int64)
    d12 = np.concatenate([bpar[:, 0], bpar[:, 0]]) if len(bidx) else np.zeros(0)
    aidx, apar = image.angles
    c13, d13 = [], []
    for (i, j, k), (th, _) in zip(aidx, apar):
        a, b = l0[(int(i), int(j))], l0[(int(j), int(k))]
        r = math.sqrt(a * a + b * b - 2.0 * a * b * math.cos(th))
        c13.append((int(i), int(k)))
        d13.append(r)
    c13 = np.asarray(c13, np.int64).reshape(-1, 2)
    c13 = np.concatenate([c13, c13[:, [1, 0]]])
    d13 = np.concatenate([d13, d13]) if len(d13) else np.zeros(0)
    return c12.astype(np.int64), np.asarray(d12), c13, np.asarray(d13)


def gb_fixed_terms(R, cov12, d12, cov13, d13, P, dielectric_offset):
    """Vj and terms123 (gbff.cpp:324-398), differentiable in the GB radii R.

    Vj = 4/3 pi R^3 minus the cap of every 1-2 partner (centre distance
    1.01 x the covalent distance), clamped at 0; terms123 = -166/(R + offset + P1)
    + sum over 1-2 partners P2 Vj / d^4 + sum over 1-3 partners P3 Vj / d^4.
    Radii <= 0.01 count as 1.15 A here (gbff.cpp:340-341)."""
    Rf = torch.where(R <= 0.01, torch.full_like(R, 1.15), R)
    vj = 4.0 * math.pi * Rf ** 3 / 3.0
    if len(cov12):
        j, k = cov12[:, 0], cov12[:, 1]
        Rj, Rk = Rf[j], Rf[k]
        rjk = 1.01 * d12
        h = Rj * (1.0 + (Rk * Rk - Rj * Rj - rjk * rjk) / (2.0 * Rj * rjk))
        vj = vj.index_add(0, j, -math.pi * h * h * (3.0 * Rj - h) / 3.0)
    vj = torch.clamp(vj, min=0.0)
    t = -166.0 / (Rf + dielectric_offset + P[0])
    if len(cov12):
        t = t.index_add(0, cov12[:, 0], P[1] * vj[cov12[:, 1]] / d12 ** 4)
    if len(cov13):
        t = t.index_add(0, cov13[:, 0], P[2] * vj[cov13[:, 1]] / d13 ** 4)
    return vj, t


class ParamTables:
    """Learnable parameters of one system in PD's per-type layout.

    LJ types are the distinct (Rmin/2, epsilon) pairs of the image, GB types the
    distinct GB radii; ``radius`` (A), ``sqrt_well`` (sqrt(kcal/mol), the square
    root of the LJ well depth, which is what PD stores per atom) and
    ``gb_radius`` (A) are per type, ``charge`` (e) per atom."""

    def __init__(self, image, device="cpu", dielectric_offset=-0.09):
        self.natom = image.natom
        self.dielectric_offset = float(dielectric_offset)  # GB DielectricOffset (gbff.cpp:44)
        lj = np.stack([image.radius, image.epsilon], axis=1)
        lj_types, lj_of = np.unique(lj, axis=0, return_inverse=True)
        self.lj_of = torch.as_tensor(lj_of.reshape(-1), device=device)
        self.radius = torch.tensor(lj_types[:, 0], dtype=torch.float64, device=device)
        self.sqrt_well = torch.tensor(lj_types[:, 1] / EPS_STORE, dtype=torch.float64, device=device)
        self.charge = torch.tensor(image.charge, dtype=torch.float64, device=device)
        self.has_gb = image.has_gb
        if self.has_gb:
            gb_types, gb_of = np.unique(image.gb_radius, return_inverse=True)
            self.gb_of = torch.as_tensor(gb_of.reshape(-1), device=device)
            self.gb_radius = torch.tensor(gb_types, dtype=torch.float64, device=device)
            c12, d12, c13, d13 = covalent_pairs(image)
            t = lambda a, dt: torch.as_tensor(a, dtype=dt, device=device)
            self.cov = (t(c12, torch.int64), t(d12, torch.float64), t(c13, torch.int64), t(d13, torch.float64))
            self.P = tuple(image.gb_P)

    def leaves(self):
        out = {"radius": self.radius, "sqrt_well": self.sqrt_well, "charge": self.charge}
        if self.has_gb:
            out["gb_radius"] = self.gb_radius
        return out

    def atom_arrays(self, radius, sqrt_well, charge, gb_radius=None, dielectric_offset=None):
        """Per-atom desc arrays (charge, radius, epsilon in PD storage, gb_radius, gb_vj, gb_terms123)."""
        out = [charge, radius[self.lj_of], (sqrt_well * EPS_STORE)[self.lj_of]]
        if self.has_gb:
            R = gb_radius[self.gb_of]
            c12, d12, c13, d13 = self.cov
            off = self.dielectric_offset if dielectric_offset is None else dielectric_offset
            vj, t = gb_fixed_terms(R, c12, d12, c13, d13, self.P, off)
            out += [R, vj, t]
        return out


class FrameSet:
    """F frames of one system, evaluated as F systems of one device context.

    ``what`` is ffi.GB (Still GB with its vacuum LJ + Coulomb, gbff.cpp FastMode)
    or ffi.NB (FF_NonBonded).  ``energies(*atom_arrays)`` returns the per-frame
    energy (J) of that component as a differentiable CUDA tensor."""

    PARAM_NAMES = ("charge", "radius", "epsilon", "gb_radius", "gb_vj", "gb_terms123")

    def __init__(self, image, frames, what, params, padding=2.0, device_index=0):
        frames = np.asarray(frames, dtype=np.float64).reshape(-1, image.natom, 3)
        self.nframes = len(frames)
        self.n = image.natom
        self.what = what
        batch = SystemImage.concat([image] * self.nframes)
        self.ctx = DeviceContext(batch, device=device_index)
        self.ctx.set_list(padding, check_skin=False)
        if what == ffi.GB:
            self.ctx.set_gb(**params)
        else:
            self.ctx.set_nb(**params)
        self.ctx.set_positions(frames.reshape(-1, 3))
        self.dev = torch.device("cuda", device_index)
        self.sys_of = torch.arange(self.nframes, device=self.dev).repeat_interleave(self.n)
        self.nparam = 6 if what == ffi.GB else 3
        N = self.n * self.nframes
        self._in = [torch.zeros(N, dtype=torch.float64, device=self.dev) for _ in range(self.nparam)]
        self.evaluations = 0

    def energies(self, *atom_params):
        """atom_params: per-atom arrays of ONE frame (length n), in PARAM_NAMES order."""
        assert len(atom_params) == self.nparam
        rep = [p.repeat(self.nframes) for p in atom_params]
        return _FrameEnergy.apply(self, *rep)


class _FrameEnergy(torch.autograd.Function):
    """Per-frame energies of a FrameSet from per-atom arrays of the whole batch;
    backward weights each atom's dE_s/dp by dL/dE_s of its own frame."""

    @staticmethod
    def forward(ctx, fs, *params):
        for dst, src in zip(fs._in, params):
            dst.copy_(src.detach())
        torch.cuda.synchronize(fs.dev)
        ptr = [t.data_ptr() for t in fs._in] + [0] * (6 - fs.nparam)
        fs.ctx.update_params_device(*ptr)
        grads = [torch.empty_like(t) for t in fs._in]
        fs.ctx.param_grad_device(fs.what, {n: g.data_ptr() for n, g in zip(FrameSet.PARAM_NAMES, grads)})
        E = fs.ctx.energies()
        fs.ctx.synchronize()
        key = ("vdw", "elec", "pol") if fs.what == ffi.GB else ("vdw", "elec")
        fs.evaluations += 1
        ctx.save_for_backward(*grads)
        ctx.fs = fs
        return torch.tensor([sum(e[k] for k in key) for e in E], dtype=torch.float64, device=fs.dev)

    @staticmethod
    def backward(ctx, gE):
        fs = ctx.fs
        w = gE[fs.sys_of]
        return (None,) + tuple(w * g for g in ctx.saved_tensors)


def perturb(tables, seed=5):
    """Start point of the fitting task: per-type LJ radius and well depth x U(0.9, 1.1),
    charges + N(0, 0.02) shifted back to the original net charge, per-type GB
    radius x U(0.95, 1.05).  Returns a dict of leaf tensors (requires_grad)."""
    g = torch.Generator().manual_seed(seed)
    u = lambda t, lo, hi: t * (lo + (hi - lo) * torch.rand(t.shape, generator=g, dtype=torch.float64).to(t.device))
    out = {"radius": u(tables.radius, 0.9, 1.1), "sqrt_well": torch.sqrt(u(tables.sqrt_well ** 2, 0.9, 1.1))}
    dq = 0.02 * torch.randn(tables.charge.shape, generator=g, dtype=torch.float64).to(tables.charge.device)
    out["charge"] = tables.charge + dq - dq.mean()
    if tables.has_gb:
        out["gb_radius"] = u(tables.gb_radius, 0.95, 1.05)
    return {k: v.detach().clone().requires_grad_(True) for k, v in out.items()}


def frame_loss(fs, tables, theta, target):
    """MSE over frames of E(theta) - target, in (kcal/mol)^2."""
    arrs = tables.atom_arrays(theta["radius"], theta["sqrt_well"], theta["charge"], theta.get("gb_radius"))
    E = fs.energies(*[a.to(fs.dev) for a in arrs])
    return torch.mean(((E - target) / KCAL_TO_J) ** 2)


def fit(fs, tables, theta, target, steps=200, lr=1e-2, charge_scale=0.1):
    """Adam against per-frame target energies (J), starting from theta (dict of
    physical parameters as ``perturb`` returns).  Positive parameters move in log
    space (x = x0 exp(s), so zero entries stay zero and none changes sign),
    charges by charge_scale x a shift with its mean removed (net charge kept;
    Adam moves every variable by about lr per step).  Returns the
    fitted parameters and the loss history."""
    logp = [k for k in ("radius", "sqrt_well", "gb_radius") if k in theta]
    x0 = {k: v.detach() for k, v in theta.items()}
    s = {k: torch.zeros_like(x0[k], requires_grad=True) for k in logp}
    dq = torch.zeros_like(x0["charge"], requires_grad=True)
    opt = torch.optim.Adam(list(s.values()) + [dq], lr=lr)

    def current():
        th = {k: x0[k] * torch.exp(s[k]) for k in logp}
        th["charge"] = x0["charge"] + charge_scale * (dq - dq.mean())
        return th

    hist = []
    for _ in range(steps):
        opt.zero_grad()
        loss = frame_loss(fs, tables, current(), target)
        loss.backward()
        opt.step()
        hist.append(float(loss.detach()))
    with torch.no_grad():
        return {k: v.detach() for k, v in current().items()}, hist
