"""Hyperparameter fitting on the GPU MLL against the same optimiser on the oracle MLL."""

import math

import numpy as np
import pytest
import torch

from botorch_gb300 import testing as T
from botorch_gb300.fit import NOISE_FLOOR, fit_gpytorch_mll
from oracle.mll import exact_mll

from tests.test_gpu_parity import gpu_model

pytestmark = pytest.mark.gpu


def test_fit_matches_oracle_fit(cuda_lib):
    from scipy.optimize import minimize

    w = T.qlognei_diff(b=1, q=1, n=96)
    w.lengthscale = torch.full((12,), 0.8, dtype=torch.float64)
    w.noise = 1e-2
    gm = gpu_model(w)
    y = gm.train_targets.cpu()
    theta0 = np.concatenate([np.log(w.lengthscale.numpy()), [0.0, math.log(w.noise - NOISE_FLOOR), 0.0]])

    def oracle_obj(theta):
        ls = torch.from_numpy(np.exp(theta[:12]))
        os_, nz, m = math.exp(theta[12]), NOISE_FLOOR + math.exp(theta[13]), theta[14]
        v, g = exact_mll(w.train_X, y, ls, os_, nz, m, "matern52")
        grad = np.concatenate([(g["lengthscale"] * ls).numpy(),
                               [g["outputscale"] * os_, g["noise"] * (nz - NOISE_FLOOR), g["mean_constant"]]])
        return -v, -grad

    ref = minimize(oracle_obj, theta0, method="L-BFGS-B", jac=True, options={"maxiter": 50})
    info = fit_gpytorch_mll(gm, maxiter=50)
    assert info["mll"] > oracle_obj(theta0)[0] * -1  # improved on the start
    assert abs(info["mll"] - (-ref.fun)) < 1e-6
    # the likelihood can be flat along some lengthscales: compare the parameters loosely
    assert float((gm.lengthscale.log() - torch.from_numpy(ref.x[:12])).abs().max()) < 5e-2
