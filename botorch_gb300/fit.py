"""Hyperparameter fitting of a ``SingleTaskGP`` by maximising the exact MLL.

The reference's ``fit_gpytorch_mll`` (botorch/fit.py:76) runs scipy's L-BFGS-B
on the raw (constraint-transformed) hyperparameters, minimising minus the
exact marginal log-likelihood per data point
(botorch/optim/closures/model_closures.py:117-143). Here the MLL and its
gradient come from the GPU (``exact_marginal_log_likelihood``, float64, from a
fresh training cache per step) and the optimiser is scipy's L-BFGS-B on
unconstrained values: log lengthscales, log outputscale, log(noise - floor)
with the reference's default noise floor of 1e-4, and the mean constant. The
maximiser is the same as under the reference's softplus transforms; the path
to it can differ.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from botorch_gb300.gp_regression import SingleTaskGP
from botorch_gb300.mll import exact_marginal_log_likelihood

NOISE_FLOOR = 1e-4  # the reference's GreaterThan constraint on the Gaussian noise


def _unpack(theta: np.ndarray, d: int) -> dict:
    return {"lengthscale": torch.from_numpy(np.exp(theta[:d])).double(),
            "outputscale": math.exp(theta[d]), "noise": NOISE_FLOOR + math.exp(theta[d + 1]),
            "mean_constant": float(theta[d + 2])}


def fit_gpytorch_mll(model: SingleTaskGP, maxiter: int = 200, options: dict | None = None) -> dict:
    """Fit the model's hyperparameters in place; returns the optimiser's summary
    (final mll / n, iterations, evaluations, message)."""
    from scipy.optimize import minimize

    d = model.d
    theta0 = np.concatenate([
        np.log(model.lengthscale.double().numpy()),
        [math.log(model.outputscale), math.log(max(model.noise - NOISE_FLOOR, 1e-12)),
         float(model.mean_constant)]])
    calls = [0]

    def objective(theta: np.ndarray):
        hp = _unpack(theta, d)
        model.set_hyperparameters(**hp)
        v, g = exact_marginal_log_likelihood(model)
        calls[0] += 1
        grad = np.concatenate([
            (g["lengthscale"] * hp["lengthscale"]).numpy(),  # d / d log l = l d / d l
            [g["outputscale"] * hp["outputscale"], g["noise"] * (hp["noise"] - NOISE_FLOOR),
             g["mean_constant"]]])
        return -v, -grad

    res = minimize(objective, theta0, method="L-BFGS-B", jac=True,
                   options={"maxiter": maxiter, **(options or {})})
    model.set_hyperparameters(**_unpack(res.x, d))
    v, _ = exact_marginal_log_likelihood(model)
    return {"mll": v, "nit": int(res.nit), "nfev": calls[0], "message": str(res.message)}
