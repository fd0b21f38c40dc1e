"""Exact marginal log-likelihood of a ``SingleTaskGP`` and its gradient.

The loss that hyperparameter fitting minimises in the reference
(botorch/fit.py:76, ``fit_gpytorch_mll``, with the closure of
botorch/optim/closures/model_closures.py:117-143: minus gpytorch's
``ExactMarginalLogLikelihood`` of the standardised training targets, per data
point). The Gaussian log density and its gradient are evaluated in float64 on
the GPU from the model's training cache (the Cholesky factor, its inverse and
alpha) by ``bgb_gp_mll``; the log densities of the priors registered on the
modules (the reference's defaults: LogNormal on the lengthscales and on the
noise, botorch/models/utils/gpytorch_modules.py:76-133), which
ExactMarginalLogLikelihood adds before dividing by n, are d + 2 scalar terms
added here.
"""

from __future__ import annotations

import ctypes

import torch

from botorch_gb300 import _native as nat
from botorch_gb300.gp_regression import SingleTaskGP
from botorch_gb300.kernels import module_priors


def exact_marginal_log_likelihood(model: SingleTaskGP, include_priors: bool = True) -> tuple[float, dict]:
    """(mll / n, gradient) with the gradient w.r.t. ``lengthscale`` (d), ``outputscale``,
    ``noise`` and ``mean_constant`` at the model's current hyperparameters; with
    ``include_priors`` the modules' log priors are part of mll, as in the reference."""
    lib = nat.lib()
    n, d = model.n, model.d
    out = (ctypes.c_double * (d + 4))()
    ws = nat.Workspace(model.device)
    wp, wb = ws.get(lib.bgb_gp_mll_workspace_bytes(n, d))
    gp = model.gp_struct()
    with torch.cuda.device(model.device):
        rc = lib.bgb_gp_mll(ctypes.byref(gp), nat.ptr(model.train_targets), nat.ptr(model.L),
                            nat.ptr(model.Linv), nat.ptr(model.alpha), out, wp, wb,
                            nat.stream_handle(model.device))
    nat.check(rc, "exact marginal log-likelihood")
    vals = list(out)
    value = vals[0]
    grad = {"lengthscale": torch.tensor(vals[1:1 + d], dtype=torch.float64),
            "outputscale": vals[1 + d], "noise": vals[2 + d], "mean_constant": vals[3 + d]}
    if include_priors:
        pri = module_priors(model.covar_module, model.likelihood)
        if pri["lengthscale"] is not None:
            ls = model.lengthscale.double()
            value += float(pri["lengthscale"].log_prob(ls).sum()) / n
            grad["lengthscale"] = grad["lengthscale"] + pri["lengthscale"].grad_log_prob(ls) / n
        for name, x in (("outputscale", model.outputscale), ("noise", model.noise)):
            if pri[name] is not None:
                value += float(pri[name].log_prob(x)) / n
                grad[name] += float(pri[name].grad_log_prob(x)) / n
    return value, grad
