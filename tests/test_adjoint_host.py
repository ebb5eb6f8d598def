"""Host side of the parameter-gradient path: the torch restatement of PD's GB
fixed terms and the per-type parameter tables, against PD's own set-up output
(fixture arrays written by PD's FF_GeneralizedBorn_Still::setup) and the oracle."""
import numpy as np
import pytest
import torch

from helpers import gb_params


def _image(d):
    from pd_gb300.workspace import SystemImage
    return SystemImage._from_fixture(d)


@pytest.mark.parametrize("name", ["peptide30", "peptide120"])
def test_covalent_pairs_match_pd(goldens, name):
    """cov12/cov13 tables rebuilt from bonds and angles equal PD's (atom.cov12atom/cov13atom)."""
    from pd_gb300.adjoint import covalent_pairs
    d = goldens[name]
    c12, d12, c13, d13 = covalent_pairs(_image(d))
    key = lambda c, dd: sorted(zip(map(tuple, np.asarray(c).tolist()), np.asarray(dd).tolist()))
    for mine, ref in ((key(c12, d12), key(d["cov12"], d["cov12d"])), (key(c13, d13), key(d["cov13"], d["cov13d"]))):
        assert [m[0] for m in mine] == [r[0] for r in ref]
        assert max(abs(m[1] - r[1]) for m, r in zip(mine, ref)) < 1e-12


@pytest.mark.parametrize("name", ["peptide30", "peptide120"])
def test_fixed_terms_match_pd_and_oracle(goldens, name):
    from oracle import pdoracle as O
    from pd_gb300.adjoint import gb_fixed_terms
    d = goldens[name]
    R = torch.tensor(d["gb_radius"])
    t = lambda a, dt=torch.float64: torch.as_tensor(a, dtype=dt)
    vj, tt = gb_fixed_terms(R, t(d["cov12"], torch.int64), t(d["cov12d"]), t(d["cov13"], torch.int64), t(d["cov13d"]),
                            tuple(d["gb_P"]), float(d["gb_DielectricOffset"][0]))
    assert np.max(np.abs(vj.numpy() - d["gb_vj"])) <= 1e-12 * np.max(np.abs(d["gb_vj"]))
    assert np.max(np.abs(tt.numpy() - d["gb_terms123"])) <= 1e-12 * np.max(np.abs(d["gb_terms123"]))
    ovj, ot = O.gb_fixed_terms(d["gb_radius"], d["cov12"], d["cov12d"], d["cov13"], d["cov13d"], gb_params(d))
    assert np.max(np.abs(vj.numpy() - ovj)) <= 1e-12 * np.max(np.abs(ovj))
    assert np.max(np.abs(tt.numpy() - ot)) <= 1e-12 * np.max(np.abs(ot))


def test_fixed_terms_gradient_is_exact(goldens):
    """Autograd through Vj / terms123 against central differences (FP64)."""
    from pd_gb300.adjoint import covalent_pairs, gb_fixed_terms
    d = goldens["peptide30"]
    c12, d12, c13, d13 = [torch.as_tensor(a) for a in covalent_pairs(_image(d))]
    P, off = tuple(d["gb_P"]), float(d["gb_DielectricOffset"][0])
    R = torch.tensor(d["gb_radius"], requires_grad=True)
    w1 = torch.linspace(-1, 1, len(R), dtype=torch.float64)
    w2 = torch.cos(torch.arange(len(R), dtype=torch.float64))
    f = lambda R: (lambda v, t: (w1 * v).sum() + (w2 * t).sum())(*gb_fixed_terms(R, c12, d12, c13, d13, P, off))
    f(R).backward()
    rng = np.random.default_rng(3)
    for a in rng.choice(len(R), 16, replace=False):
        h = 1e-6
        Rp, Rm = R.detach().clone(), R.detach().clone()
        Rp[a] += h
        Rm[a] -= h
        fd = float(f(Rp) - f(Rm)) / (2 * h)
        assert abs(float(R.grad[a]) - fd) <= 1e-6 * max(abs(fd), 1.0), (a, float(R.grad[a]), fd)


def test_param_tables_reproduce_image(goldens):
    """The per-type tables map back to the image's per-atom arrays exactly."""
    from pd_gb300.adjoint import ParamTables
    d = goldens["peptide120"]
    T = ParamTables(_image(d))
    q, r, e, R, vj, t = [a.detach().numpy() for a in
                         T.atom_arrays(T.radius, T.sqrt_well, T.charge, T.gb_radius, float(d["gb_DielectricOffset"][0]))]
    assert np.array_equal(q, d["charge"]) and np.array_equal(r, d["radius"]) and np.array_equal(R, d["gb_radius"])
    assert np.max(np.abs(e - d["epsilon"])) <= 1e-15 * np.max(d["epsilon"])
    assert np.max(np.abs(vj - d["gb_vj"])) <= 1e-12 * np.max(d["gb_vj"])
    assert np.max(np.abs(t - d["gb_terms123"])) <= 1e-12 * np.max(np.abs(d["gb_terms123"]))


def test_perturbation_keeps_net_charge(goldens):
    from pd_gb300.adjoint import ParamTables, perturb
    T = ParamTables(_image(goldens["peptide30"]))
    th = perturb(T, seed=5)
    assert abs(float(th["charge"].detach().sum() - T.charge.sum())) < 1e-12
    nz = T.radius > 0
    rr = (th["radius"].detach()[nz] / T.radius[nz]).numpy()
    assert rr.min() >= 0.9 and rr.max() <= 1.1
    gr = (th["gb_radius"].detach() / T.gb_radius).numpy()
    assert gr.min() >= 0.95 and gr.max() <= 1.05
