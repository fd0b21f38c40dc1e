"""The MLL oracle against finite differences and against a closed form."""

import math

import torch

from oracle.gp import kernel_matrix
from oracle.mll import exact_mll


def _case(n=40, d=3, seed=0):
    g = torch.Generator().manual_seed(seed)
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    y = torch.sin(3 * X).sum(-1) + 0.05 * torch.randn(n, generator=g, dtype=torch.float64)
    y = (y - y.mean()) / y.std()
    ls = 0.3 + 0.5 * torch.rand(d, generator=g, dtype=torch.float64)
    return X, y, ls


def test_value_matches_closed_form():
    X, y, ls = _case()
    v, _ = exact_mll(X, y, ls, 1.3, 1e-2, 0.1, "matern52")
    K = kernel_matrix(X, X, ls, 1.3, "matern52") + 1e-2 * torch.eye(X.shape[0], dtype=torch.float64)
    ref = torch.distributions.MultivariateNormal(torch.full_like(y, 0.1), K).log_prob(y) / X.shape[0]
    assert abs(v - float(ref)) < 1e-12


def test_gradient_matches_finite_differences():
    X, y, ls = _case()
    kw = dict(outputscale=1.3, noise=1e-2, mean_constant=0.1, kind="rbf")
    _, g = exact_mll(X, y, ls, **kw)
    h = 1e-6
    for k in range(ls.numel()):
        lp, lm = ls.clone(), ls.clone()
        lp[k] += h
        lm[k] -= h
        fd = (exact_mll(X, y, lp, **kw)[0] - exact_mll(X, y, lm, **kw)[0]) / (2 * h)
        assert math.isclose(fd, float(g["lengthscale"][k]), rel_tol=1e-6, abs_tol=1e-9)
    for name in ("outputscale", "noise", "mean_constant"):
        kp, km = dict(kw), dict(kw)
        kp[name] += h
        km[name] -= h
        fd = (exact_mll(X, y, ls, **kp)[0] - exact_mll(X, y, ls, **km)[0]) / (2 * h)
        assert math.isclose(fd, g[name], rel_tol=1e-6, abs_tol=1e-9), name


def test_library_prior_terms_match_torch_distributions():
    """The prior densities the library adds to the MLL (botorch_gb300.kernels) against
    torch.distributions, value and derivative."""
    from botorch_gb300.kernels import GammaPrior, LogNormalPrior

    x = torch.tensor([0.03, 0.4, 2.5], dtype=torch.float64)
    loc = math.sqrt(2) + 0.5 * math.log(6)
    for prior, ref in ((LogNormalPrior(loc, math.sqrt(3)),
                        torch.distributions.LogNormal(torch.tensor(loc, dtype=torch.float64),
                                                      torch.tensor(math.sqrt(3), dtype=torch.float64))),
                       (GammaPrior(2.0, 0.15), torch.distributions.Gamma(torch.tensor(2.0, dtype=torch.float64),
                                                                       torch.tensor(0.15, dtype=torch.float64)))):
        xg = x.clone().requires_grad_(True)
        lp = ref.log_prob(xg)
        (gr,) = torch.autograd.grad(lp.sum(), xg)
        assert torch.allclose(prior.log_prob(x), lp.detach(), rtol=0, atol=1e-13)
        assert torch.allclose(prior.grad_log_prob(x), gr, rtol=1e-13, atol=1e-13)


def test_mll_priors_gradient_matches_finite_differences():
    X, y, ls = _case()
    pri = {"lengthscale": ("lognormal", 1.9, 1.7), "outputscale": ("gamma", 2.0, 0.15),
           "noise": ("lognormal", -4.0, 1.0)}
    kw = dict(outputscale=1.3, noise=1e-2, mean_constant=0.1, kind="matern52", priors=pri)
    _, g = exact_mll(X, y, ls, **kw)
    h = 1e-6
    for k in range(ls.numel()):
        lp, lm = ls.clone(), ls.clone()
        lp[k] += h
        lm[k] -= h
        fd = (exact_mll(X, y, lp, **kw)[0] - exact_mll(X, y, lm, **kw)[0]) / (2 * h)
        assert math.isclose(fd, float(g["lengthscale"][k]), rel_tol=1e-6, abs_tol=1e-9)
    for name in ("outputscale", "noise"):
        kp, km = dict(kw), dict(kw)
        kp[name] += h
        km[name] -= h
        fd = (exact_mll(X, y, ls, **kp)[0] - exact_mll(X, y, ls, **km)[0]) / (2 * h)
        assert math.isclose(fd, g[name], rel_tol=1e-6, abs_tol=1e-9), name
