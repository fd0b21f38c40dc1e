"""Hyperparameter fitting on the GPU MLL against the same optimiser on the oracle MLL.

Both fits run scipy's L-BFGS-B over the parameters of the reference's modules
(lengthscales and noise as bounded raw values, a ScaleKernel's outputscale
through softplus, the mean constant free; botorch_gb300/fit.py), on minus the
exact MLL per data point, with the log priors of the modules included as
gpytorch's ExactMarginalLogLikelihood adds them.
"""

import math

import numpy as np
import pytest
import torch

from botorch_gb300 import SingleTaskGP
from botorch_gb300 import testing as T
from botorch_gb300.fit import LENGTHSCALE_FLOOR, NOISE_FLOOR, fit_gpytorch_mll, inv_softplus, softplus
from oracle.mll import exact_mll

from tests.test_gpu_parity import gpu_model

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def oracle_fit(train_X, y, theta0, kind, scaled, priors, maxiter):
    from scipy.optimize import minimize

    d = train_X.shape[-1]

    def obj(theta):
        ls = torch.from_numpy(np.array(theta[:d]))
        os_ = softplus(theta[d]) if scaled else 1.0
        nz, m = theta[-2], theta[-1]
        v, g = exact_mll(train_X, y, ls, os_, nz, m, kind, priors=priors)
        grad = list(g["lengthscale"].numpy())
        if scaled:
            grad.append(g["outputscale"] / (1.0 + math.exp(-theta[d])))
        grad += [g["noise"], g["mean_constant"]]
        return -v, -np.array(grad)

    bounds = [(LENGTHSCALE_FLOOR, None)] * d + ([(None, None)] if scaled else []) + \
        [(NOISE_FLOOR, None), (None, None)]
    ref = minimize(obj, theta0, method="L-BFGS-B", jac=True, bounds=bounds, options={"maxiter": maxiter})
    return ref, obj(theta0)[0]


def test_fit_matches_oracle_fit(cuda_lib):
    """A ScaleKernel(Matern-5/2) model without priors."""
    w = T.qlognei_diff(b=1, q=1, n=96)
    w.lengthscale = torch.full((12,), 0.8, dtype=torch.float64)
    w.noise = 1e-2
    gm = gpu_model(w)
    y = gm.train_targets.cpu()
    theta0 = np.array(list(w.lengthscale.numpy()) + [inv_softplus(w.outputscale), w.noise, 0.0])
    ref, f0 = oracle_fit(w.train_X, y, theta0, "matern52", True, None, 50)
    info = fit_gpytorch_mll(gm, maxiter=50)
    assert -info["mll"] < f0  # improved on the start
    assert abs(info["mll"] - (-ref.fun)) < 1e-6, (info["mll"], -ref.fun)
    # the likelihood can be flat along some lengthscales: compare the parameters loosely
    assert float((gm.lengthscale.log() - torch.from_numpy(np.log(ref.x[:12]))).abs().max()) < 5e-2


def test_default_model_fit_with_priors_matches_oracle(cuda_lib):
    """The reference's default SingleTaskGP: ARD RBF with the dimension-scaled LogNormal
    lengthscale prior, LogNormal(-4, 1) noise prior, Standardize; the fit's loss holds
    the log priors (botorch/models/utils/gpytorch_modules.py:76-133, botorch/fit.py:76)."""
    g = torch.Generator().manual_seed(11)
    n, d = 80, 4
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    Y = (torch.sin(4 * X[:, :1]) + X[:, 1:2] ** 2 + 0.05 * torch.randn(n, 1, generator=g, dtype=torch.float64))
    gm = SingleTaskGP(X, Y, device=DEV)
    mode_ls = math.exp(math.sqrt(2) + 0.5 * math.log(d) - 3.0)
    assert torch.allclose(gm.lengthscale, torch.full((d,), mode_ls, dtype=torch.float64))
    assert gm.noise == pytest.approx(math.exp(-4.0 - 1.0))
    y = gm.train_targets.cpu()
    priors = {"lengthscale": ("lognormal", math.sqrt(2) + 0.5 * math.log(d), math.sqrt(3)),
              "noise": ("lognormal", -4.0, 1.0)}
    theta0 = np.array([mode_ls] * d + [gm.noise, 0.0])
    ref, f0 = oracle_fit(X, y, theta0, "rbf", False, priors, 100)
    info = fit_gpytorch_mll(gm, maxiter=100)
    assert -info["mll"] < f0
    assert abs(info["mll"] - (-ref.fun)) < 1e-6, (info["mll"], -ref.fun)
    assert float((gm.lengthscale - torch.from_numpy(ref.x[:d])).abs().max()) < 1e-3
    # the priors pull the fit: without them the loss at the fitted point differs
    v_np, _ = exact_mll(X, y, gm.lengthscale, 1.0, gm.noise, gm.mean_constant, "rbf")
    assert abs(v_np - info["mll"]) > 1e-4
