"""ORACLE (test infrastructure): exact marginal log-likelihood of the GP and its
gradient w.r.t. the hyperparameters, float64 on CPU by torch autograd.

Restated from the training loss of the reference: botorch/fit.py:76
(``fit_gpytorch_mll``) minimises ``-mll(model(*train_inputs), train_targets)``
(botorch/optim/closures/model_closures.py:117-143), where ``mll`` is gpytorch's
``ExactMarginalLogLikelihood`` (external, gpytorch >= 1.15.2): the Gaussian
log density of the standardised targets under N(m, K + noise I), divided by
the number of data points, plus the log densities of the priors registered on
the modules, which ExactMarginalLogLikelihood adds before that division (the
reference's default SingleTaskGP registers LogNormal(sqrt(2) + log(d) / 2,
sqrt(3)) on each lengthscale and LogNormal(-4, 1) on the noise,
botorch/models/utils/gpytorch_modules.py:76-133). The prior densities are
torch.distributions' LogNormal / Gamma.
"""

from __future__ import annotations

import math

import torch
from torch import Tensor

from oracle.gp import kernel_from_sq_dist


def prior_log_prob(spec, x: Tensor) -> Tensor:
    """Summed log density of x under spec = ("lognormal", loc, scale) or ("gamma", a, b)."""
    kind, p1, p2 = spec
    if kind == "lognormal":
        dist = torch.distributions.LogNormal(torch.tensor(p1, dtype=torch.float64),
                                             torch.tensor(p2, dtype=torch.float64))
    elif kind == "gamma":
        dist = torch.distributions.Gamma(torch.tensor(p1, dtype=torch.float64),
                                         torch.tensor(p2, dtype=torch.float64))
    else:
        raise ValueError(kind)
    return dist.log_prob(x).sum()


def exact_mll(train_X: Tensor, y: Tensor, lengthscale: Tensor, outputscale: float, noise: float,
              mean_constant: float, kind: str, priors: dict | None = None) -> tuple[float, dict]:
    """(log N(y | m, K + noise I) + log priors) / n and its gradient w.r.t. lengthscale
    (d), outputscale, noise and the mean constant; ``y`` is the standardised target (n);
    ``priors`` maps "lengthscale" / "outputscale" / "noise" to a prior spec (see
    ``prior_log_prob``)."""
    X = train_X.to(torch.float64)
    y = y.to(torch.float64).reshape(-1)
    n = X.shape[0]
    ls = torch.as_tensor(lengthscale, dtype=torch.float64).expand(X.shape[-1]).clone().requires_grad_(True)
    os_ = torch.tensor(float(outputscale), dtype=torch.float64, requires_grad=True)
    nz = torch.tensor(float(noise), dtype=torch.float64, requires_grad=True)
    m = torch.tensor(float(mean_constant), dtype=torch.float64, requires_grad=True)
    Z = X / ls
    r2 = ((Z.unsqueeze(-2) - Z.unsqueeze(-3)) ** 2).sum(-1)
    K = kernel_from_sq_dist(r2, kind, 1.0) * os_ + nz * torch.eye(n, dtype=torch.float64)
    L = torch.linalg.cholesky(K)
    res = (y - m).unsqueeze(-1)
    alpha = torch.cholesky_solve(res, L)
    ll = -0.5 * (res * alpha).sum() - torch.log(torch.diagonal(L)).sum() - 0.5 * n * math.log(2 * math.pi)
    for name, x in (("lengthscale", ls), ("outputscale", os_), ("noise", nz)):
        if priors and priors.get(name) is not None:
            ll = ll + prior_log_prob(priors[name], x)
    mll = ll / n
    g_ls, g_os, g_nz, g_m = torch.autograd.grad(mll, (ls, os_, nz, m))
    return float(mll.detach()), {"lengthscale": g_ls, "outputscale": float(g_os), "noise": float(g_nz),
                        "mean_constant": float(g_m)}
