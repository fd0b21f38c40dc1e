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


class LogNormalPrior:
    """log x ~ N(loc, scale^2) (gpytorch.priors.LogNormalPrior): the prior the reference's
    default SingleTaskGP puts on its lengthscales and noise
    (botorch/models/utils/gpytorch_modules.py:76-133)."""

    def __init__(self, loc: float, scale: float) -> None:
        self.loc, self.scale = float(loc), float(scale)

    @property
    def mode(self) -> float:
        return _lognormal_mode(self.loc, self.scale)

    def log_prob(self, x: Tensor) -> Tensor:
        x = torch.as_tensor(x, dtype=torch.float64)
        z = (torch.log(x) - self.loc) / self.scale
        return -torch.log(x) - math.log(self.scale) - 0.5 * math.log(2 * math.pi) - 0.5 * z * z

    def grad_log_prob(self, x: Tensor) -> Tensor:
        x = torch.as_tensor(x, dtype=torch.float64)
        return -(1.0 + (torch.log(x) - self.loc) / (self.scale * self.scale)) / x


class GammaPrior:
    """x ~ Gamma(concentration, rate) (gpytorch.priors.GammaPrior): the priors of the
    reference's Matern-with-gamma-prior modules (botorch/models/utils/gpytorch_modules.py:34-73)."""

    def __init__(self, concentration: float, rate: float) -> None:
        self.concentration, self.rate = float(concentration), float(rate)

    def log_prob(self, x: Tensor) -> Tensor:
        x = torch.as_tensor(x, dtype=torch.float64)
        a, b = self.concentration, self.rate
        return a * math.log(b) - math.lgamma(a) + (a - 1) * torch.log(x) - b * x

    def grad_log_prob(self, x: Tensor) -> Tensor:
        x = torch.as_tensor(x, dtype=torch.float64)
        return (self.concentration - 1) / x - self.rate


class _Stationary:
    kind = ""

    def __init__(self, ard_num_dims: int | None = None, lengthscale=None,
                 lengthscale_prior=None) -> None:
        self.ard_num_dims = ard_num_dims
        self.lengthscale_prior = lengthscale_prior
        if lengthscale is None:
            if lengthscale_prior is not None and hasattr(lengthscale_prior, "mode"):
                lengthscale = lengthscale_prior.mode
            else:
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

    def __init__(self, nu: float = 2.5, ard_num_dims: int | None = None, lengthscale=None,
                 lengthscale_prior=None) -> None:
        if nu not in (0.5, 1.5, 2.5):
            raise ValueError("nu expected to be 0.5, 1.5, or 2.5")
        super().__init__(ard_num_dims, lengthscale, lengthscale_prior)
        self.nu = nu
        self.kind = {2.5: "matern52", 1.5: "matern32", 0.5: "matern12"}[nu]


class RBFKernel(_Stationary):
    """Squared-exponential kernel (gpytorch.kernels.RBFKernel)."""

    kind = "rbf"


class ScaleKernel:
    """outputscale * base_kernel (gpytorch.kernels.ScaleKernel)."""

    def __init__(self, base_kernel: _Stationary, outputscale: float = 1.0,
                 outputscale_prior=None) -> None:
        self.base_kernel = base_kernel
        self.outputscale = float(outputscale)
        self.outputscale_prior = outputscale_prior


class GaussianLikelihood:
    """Homoskedastic noise (gpytorch.likelihoods.GaussianLikelihood)."""

    def __init__(self, noise: float | None = None, noise_prior=None) -> None:
        if noise is None:
            noise = noise_prior.mode if noise_prior is not None and hasattr(noise_prior, "mode") \
                else _lognormal_mode(-4.0, 1.0)
        if not noise > 0:
            raise ValueError("noise must be positive")
        self.noise = float(noise)
        self.noise_prior = noise_prior


class ConstantMean:
    """Constant prior mean (gpytorch.means.ConstantMean)."""

    def __init__(self, constant: float = 0.0) -> None:
        self.constant = float(constant)


def default_covar_module(d: int) -> "RBFKernel":
    """The reference's default covariance module of SingleTaskGP: an ARD RBF kernel with
    the dimension-scaled LogNormal(sqrt(2) + log(d) / 2, sqrt(3)) lengthscale prior,
    lengthscales at its mode (botorch/models/utils/gpytorch_modules.py:100-133)."""
    return RBFKernel(ard_num_dims=d, lengthscale_prior=LogNormalPrior(SQRT2 + 0.5 * math.log(d), SQRT3))


def default_likelihood() -> GaussianLikelihood:
    """The reference's default likelihood: LogNormal(-4, 1) noise prior, noise at its mode
    (botorch/models/utils/gpytorch_modules.py:76-97)."""
    return GaussianLikelihood(noise_prior=LogNormalPrior(-4.0, 1.0))


def module_priors(covar_module, likelihood) -> dict:
    """The priors registered on the modules: {"lengthscale", "outputscale", "noise"} -> prior
    or None (the terms gpytorch's ExactMarginalLogLikelihood adds to the log likelihood)."""
    base = covar_module.base_kernel if isinstance(covar_module, ScaleKernel) else covar_module
    return {"lengthscale": getattr(base, "lengthscale_prior", None),
            "outputscale": getattr(covar_module, "outputscale_prior", None)
            if isinstance(covar_module, ScaleKernel) else None,
            "noise": getattr(likelihood, "noise_prior", None)}


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
