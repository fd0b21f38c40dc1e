"""ORACLE (test infrastructure): restatement of botorch/utils/safe_math.py.

Every function here follows the reference function of the same name; the
line numbers cite ``botorch/utils/safe_math.py`` in BoTorch 0.18.1.
"""

from __future__ import annotations

import math

import torch
from torch import Tensor
from torch.nn.functional import softplus

ALPHA = 2.0  # safe_math.py:31 (default power decay of the Pareto kernel)


def cauchy(x: Tensor) -> Tensor:
    """Un-normalised Lorentzian 1 / (1 + x^2) (safe_math.py:461)."""
    return 1 / (1 + x.square())


def fatplus(x: Tensor, tau: float) -> Tensor:
    """tau * (softplus(x/tau) + 0.1 * cauchy(x/tau)) (safe_math.py:307-325).

    ``softplus`` keeps torch's default threshold of 20: for z > 20 it returns z.
    """
    z = x / tau
    return tau * (softplus(z) + 1e-1 * cauchy(z))


def log_fatplus(x: Tensor, tau: float) -> Tensor:
    """log(fatplus(x, tau)) (safe_math.py:298-304)."""
    return fatplus(x, tau=tau).log()


def pareto(x: Tensor, alpha: float = ALPHA) -> Tensor:
    """Rational kernel with value, first and second derivative 1 at 0 (safe_math.py:466-490).

    With alpha=2: a = 1, beta_1 = 2, beta_0 = 2 -> 2 / (2 + 2x + x^2).
    """
    a = alpha / 2
    beta_1 = 2 * a
    beta_0 = a * beta_1
    return (beta_0 / (beta_0 + beta_1 * x + x.square())).pow(a)


def _inf_max_helper(max_fun, x: Tensor, dim: int, keepdim: bool = False) -> Tensor:
    """Masked treatment of +-inf for smooth maxima (safe_math.py:146-191)."""
    if x.shape[dim] == 0:
        return x.sum(dim=dim, keepdim=keepdim) - torch.inf
    M = x.amax(dim=dim, keepdim=True)
    is_inf_max = torch.logical_and(*torch.broadcast_tensors(M.isinf(), x == M))
    has_inf_max = is_inf_max.any(dim=dim, keepdim=True)
    y_inf = x.masked_fill(~is_inf_max, 0.0)
    M_no_inf = M.masked_fill(M.isinf(), 0.0)
    y_no_inf = x.masked_fill(has_inf_max, 0.0) - M_no_inf
    res = torch.where(
        has_inf_max,
        y_inf.sum(dim=dim, keepdim=True),
        M_no_inf + max_fun(y_no_inf, dim=dim, keepdim=True),
    )
    return res if keepdim else res.sum(dim=dim)


def logsumexp(x: Tensor, dim: int, keepdim: bool = False) -> Tensor:
    """logsumexp with the reference's inf handling (safe_math.py:123-143)."""
    return _inf_max_helper(torch.logsumexp, x=x, dim=dim, keepdim=keepdim)


def logmeanexp(x: Tensor, dim: int, keepdim: bool = False) -> Tensor:
    """logsumexp(x) - log(n) over ``dim`` (safe_math.py:213-225)."""
    return logsumexp(x, dim=dim, keepdim=keepdim) - math.log(x.shape[dim])


def fatmax(x: Tensor, dim: int, keepdim: bool = False, tau: float = 1.0,
           alpha: float = ALPHA) -> Tensor:
    """Fat-tailed smooth maximum (safe_math.py:328-356).

    M + tau * log(sum_j pareto(-(x_j - M) / tau)), through _inf_max_helper.
    """

    def max_fun(y: Tensor, dim: int, keepdim: bool = False) -> Tensor:
        return tau * pareto(-y / tau, alpha=alpha).sum(dim=dim, keepdim=keepdim).log()

    return _inf_max_helper(max_fun=max_fun, x=x, dim=dim, keepdim=keepdim)


def log_improvement(Y: Tensor, best_f: Tensor, tau: float) -> Tensor:
    """log_fatplus(Y - best_f[..., None], tau) (botorch/acquisition/logei.py:688-715, fat=True)."""
    return log_fatplus(Y - best_f.unsqueeze(-1).to(Y), tau=tau)
