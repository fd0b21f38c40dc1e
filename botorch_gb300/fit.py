"""Hyperparameter fitting of a ``SingleTaskGP`` by maximising the exact MLL.

The reference's ``fit_gpytorch_mll`` (botorch/fit.py:76) runs scipy's L-BFGS-B
(botorch/optim/fit.py, botorch/optim/core.py) on the modules' raw parameters,
minimising minus gpytorch's ExactMarginalLogLikelihood per data point, log
priors included (botorch/optim/closures/model_closures.py:117-143). The same
here: the loss and its gradient come from the GPU
(``exact_marginal_log_likelihood``, float64, from a fresh training cache per
step), the optimiser is scipy's L-BFGS-B, and the parameters are those of the
reference's modules: the lengthscales and the noise as raw values with the
lower bounds of their GreaterThan(transform=None) constraints (2.5e-2 and
1e-4, botorch/models/utils/gpytorch_modules.py:76-133), the outputscale of a
ScaleKernel through softplus (gpytorch's default Positive constraint), and the
mean constant unconstrained.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from botorch_gb300.gp_regression import SingleTaskGP
from botorch_gb300.kernels import ScaleKernel
from botorch_gb300.mll import exact_marginal_log_likelihood

NOISE_FLOOR = 1e-4          # GreaterThan(MIN_INFERRED_NOISE_LEVEL) on the Gaussian noise
LENGTHSCALE_FLOOR = 2.5e-2  # GreaterThan(2.5e-2) on the default kernel's lengthscales


def softplus(x: float) -> float:
    return x + math.log1p(math.exp(-x)) if x > 0 else math.log1p(math.exp(x))


def inv_softplus(y: float) -> float:
    return y + math.log(-math.expm1(-y))


def parameter_layout(model: SingleTaskGP):
    """(theta0, bounds, unpack(theta) -> hyperparameters, chain(theta, grads) -> d mll / d theta)
    for the model's modules."""
    d = model.d
    scaled = isinstance(model.covar_module, ScaleKernel)
    theta0 = list(model.lengthscale.double().numpy())
    bounds = [(LENGTHSCALE_FLOOR, None)] * d
    if scaled:
        theta0.append(inv_softplus(model.outputscale))
        bounds.append((None, None))
    theta0 += [model.noise, float(model.mean_constant)]
    bounds += [(NOISE_FLOOR, None), (None, None)]

    def unpack(theta: np.ndarray) -> dict:
        hp = {"lengthscale": torch.from_numpy(np.array(theta[:d])).double(), "noise": float(theta[-2]),
              "mean_constant": float(theta[-1])}
        if scaled:
            hp["outputscale"] = softplus(float(theta[d]))
        return hp

    def chain(theta: np.ndarray, g: dict) -> np.ndarray:
        out = list(g["lengthscale"].numpy())
        if scaled:
            out.append(g["outputscale"] / (1.0 + math.exp(-float(theta[d]))))  # d softplus = sigmoid
        return np.array(out + [g["noise"], g["mean_constant"]])

    return np.array(theta0, dtype=np.float64), bounds, unpack, chain


def fit_gpytorch_mll(model: SingleTaskGP, maxiter: int = 200, options: dict | None = None,
                     include_priors: bool = True) -> dict:
    """Fit the model's hyperparameters in place; returns the optimiser's summary
    (final mll / n, iterations, evaluations, message)."""
    from scipy.optimize import minimize

    theta0, bounds, unpack, chain = parameter_layout(model)
    calls = [0]

    def objective(theta: np.ndarray):
        model.set_hyperparameters(**unpack(theta))
        v, g = exact_marginal_log_likelihood(model, include_priors)
        calls[0] += 1
        return -v, -chain(theta, g)

    res = minimize(objective, theta0, method="L-BFGS-B", jac=True, bounds=bounds,
                   options={"maxiter": maxiter, **(options or {})})
    model.set_hyperparameters(**unpack(res.x))
    v, _ = exact_marginal_log_likelihood(model, include_priors)
    return {"mll": v, "nit": int(res.nit), "nfev": calls[0], "message": str(res.message)}
