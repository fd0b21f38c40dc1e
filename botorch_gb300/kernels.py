"""Hyperparameter holders with the names of the gpytorch modules SingleTaskGP uses.

gpytorch is not a dependency of this package; these classes carry the fixed
hyperparameters (ARD lengthscales, outputscale, noise, constant mean) that
the CUDA path evaluates. Defaults follow the reference's SingleTaskGP
(botorch/models/gp_regression.py:173-201 and
botorch/models/utils/gpytorch_modules.py:76-133): an ARD RBF kernel without
outputscale whose lengthscales start at the mode of LogNormal(sqrt(2) +
log(d)/2, sqrt(3)), a Gaussian likelihood whose noise starts at the mode of
LogNormal(-4, 1), and a zero constant mean.
"""

from __future__ import annotations

import math

import torch
from torch import Tensor

SQRT2 = math.sqrt(2)
SQRT3 = math.sqrt(3)
MIN_INFERRED_NOISE_LEVEL = 1e-4


def _lognormal_mode(loc: float, scale: float) -> float:
    return math.exp(loc - scale * scale)


class _Stationary:
    kind = ""

    def __init__(self, ard_num_dims: int | None = None, lengthscale=None) -> None:
        self.ard_num_dims = ard_num_dims
        if lengthscale is None:
            d = ard_num_dims or 1
            lengthscale = _lognormal_mode(SQRT2 + 0.5 * math.log(d), SQRT3)
        self.lengthscale = lengthscale

    @property
    def lengthscale(self) -> Tensor:
        return self._lengthscale

    @lengthscale.setter
    def lengthscale(self, value) -> None:
        t = torch.as_tensor(value, dtype=torch.float64).reshape(-1)
        if self.ard_num_dims is not None and t.numel() == 1:
            t = t.expand(self.ard_num_dims).clone()
        if not bool((t > 0).all()):
            raise ValueError("lengthscales must be positive")
        self._lengthscale = t


class MaternKernel(_Stationary):
    """Matern kernel with smoothness nu in {0.5, 1.5, 2.5} (gpytorch.kernels.MaternKernel)."""

    def __init__(self, nu: float = 2.5, ard_num_dims: int | None = None, lengthscale=None) -> None:
        if nu not in (0.5, 1.5, 2.5):
            raise ValueError("nu expected to be 0.5, 1.5, or 2.5")
        super().__init__(ard_num_dims, lengthscale)
        self.nu = nu
        self.kind = {2.5: "matern52", 1.5: "matern32", 0.5: "matern12"}[nu]


class RBFKernel(_Stationary):
    """Squared-exponential kernel (gpytorch.kernels.RBFKernel)."""

    kind = "rbf"


class ScaleKernel:
    """outputscale * base_kernel (gpytorch.kernels.ScaleKernel)."""

    def __init__(self, base_kernel: _Stationary, outputscale: float = 1.0) -> None:
        self.base_kernel = base_kernel
        self.outputscale = float(outputscale)


class GaussianLikelihood:
    """Homoskedastic noise (gpytorch.likelihoods.GaussianLikelihood)."""

    def __init__(self, noise: float | None = None) -> None:
        if noise is None:
            noise = _lognormal_mode(-4.0, 1.0)
        if not noise > 0:
            raise ValueError("noise must be positive")
        self.noise = float(noise)


class ConstantMean:
    """Constant prior mean (gpytorch.means.ConstantMean)."""

    def __init__(self, constant: float = 0.0) -> None:
        self.constant = float(constant)


def unpack_covar_module(covar_module) -> tuple[str, Tensor, float]:
    """(kernel kind, lengthscale, outputscale) of a ScaleKernel or bare kernel."""
    outputscale = 1.0
    base = covar_module
    if isinstance(covar_module, ScaleKernel):
        outputscale = covar_module.outputscale
        base = covar_module.base_kernel
    if not isinstance(base, _Stationary):
        raise TypeError(f"unsupported covariance module {type(covar_module).__name__}")
    return base.kind, base.lengthscale, outputscale
