"""ORACLE (test infrastructure): the exact-GP side of the path in float64 on CPU.

Restated from:

* botorch/models/gp_regression.py:108-214 (``SingleTaskGP``: constant mean,
  scaled ARD kernel, Gaussian likelihood, Standardize outcome transform);
* botorch/models/transforms/outcome.py:312-345 (``Standardize.forward``:
  unbiased std, ``min_stdv`` 1e-8) and :431-511 (``untransform_posterior``:
  mean * s + m, covariance * s^2);
* botorch/models/gpytorch.py:544-611 (``posterior``) with the global settings
  of botorch/__init__.py:51-56 (dense Cholesky, no fast root decompositions,
  ``cholesky_max_tries`` 6);
* the published algorithms of the external, un-vendored dependencies that the
  reference calls for the arithmetic (gpytorch >= 1.15.2 and
  linear_operator >= 0.6.1 per pyproject.toml:24-34, versions unpinned):
  - ``MaternKernel`` (nu = 5/2, 3/2, 1/2) and ``RBFKernel`` with ARD
    lengthscales, wrapped in ``ScaleKernel`` (outputscale);
  - the exact prediction strategy: mean = m + K(X, Xt) (K + s2 I)^-1 (y - m),
    covariance = K(X, X) - K(X, Xt) (K + s2 I)^-1 K(Xt, X) with the inverse
    applied through the Cholesky factor of the training covariance;
  - ``psd_safe_cholesky``: a plain Cholesky first; on failure, jitter
    j * 10^i (j = 1e-8 for float64, 1e-6 for float32) is added to the
    diagonal of only the failing batch members, for i = 0 .. max_tries-1.

Pairwise scaled distances are formed from explicit coordinate differences
(not the |a|^2 + |b|^2 - 2ab expansion gpytorch uses), which is the more
accurate of the two; both agree far inside the parity tolerances.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import torch
from torch import Tensor

KERNELS = ("matern52", "matern32", "matern12", "rbf")


class NotPSDError(RuntimeError):
    """Raised when psd_safe_cholesky gives up (linear_operator.utils.errors.NotPSDError)."""


class NanError(RuntimeError):
    """Raised on NaN input to psd_safe_cholesky or non-finite samples (low_rank.py:162-171)."""


def default_jitter(dtype: torch.dtype) -> float:
    return 1e-8 if dtype == torch.float64 else 1e-6


def psd_safe_cholesky(A: Tensor, max_tries: int = 6, jitter: float | None = None,
                      return_jitter: bool = False):
    """Batched Cholesky with per-member jitter retries (linear_operator's published algorithm).

    With ``return_jitter`` the total jitter added to the last failing member's
    diagonal (0.0 when the plain factorisation succeeds) is returned beside L.
    """
    L, info = torch.linalg.cholesky_ex(A)
    if not torch.any(info):
        return (L, 0.0) if return_jitter else L
    if torch.isnan(A).any():
        raise NanError("cholesky_cpu: input matrix contains NaNs")
    if jitter is None:
        jitter = default_jitter(A.dtype)
    Aprime = A.clone()
    jitter_prev = 0.0
    for i in range(max_tries):
        jitter_new = jitter * (10 ** i)
        diag_add = ((info > 0) * (jitter_new - jitter_prev)).unsqueeze(-1).expand(*Aprime.shape[:-1])
        Aprime.diagonal(dim1=-1, dim2=-2).add_(diag_add.to(A.dtype))
        jitter_prev = jitter_new
        L, info = torch.linalg.cholesky_ex(Aprime)
        if not torch.any(info):
            return (L, jitter_new) if return_jitter else L
    raise NotPSDError(f"Matrix not positive definite after repeatedly adding jitter up to {jitter_new:.1e}.")


def scaled_sq_dist(X1: Tensor, X2: Tensor, lengthscale: Tensor, chunk: int = 256) -> Tensor:
    """rho^2 = sum_k ((x1_k - x2_k) / l_k)^2 for all pairs, by explicit differences."""
    Z1 = X1 / lengthscale
    Z2 = X2 / lengthscale
    if Z1.dim() == 2 and Z2.dim() == 2 and Z1.shape[0] > chunk:
        return torch.cat([((Z1[i:i + chunk, None, :] - Z2[None, :, :]) ** 2).sum(-1)
                          for i in range(0, Z1.shape[0], chunk)], dim=0)
    return ((Z1.unsqueeze(-2) - Z2.unsqueeze(-3)) ** 2).sum(-1)


def kernel_from_sq_dist(r2: Tensor, kind: str, outputscale: float) -> Tensor:
    """Stationary kernel value from the squared scaled distance.

    rho = sqrt(max(r2, 1e-30)) as in gpytorch's ``dist`` so that the gradient
    at coincident points is finite.
    """
    if kind == "rbf":
        return outputscale * torch.exp(-0.5 * r2)
    rho = r2.clamp_min(1e-30).sqrt()
    if kind == "matern52":
        s5 = math.sqrt(5.0) * rho
        return outputscale * (1 + s5 + (5.0 / 3.0) * r2) * torch.exp(-s5)
    if kind == "matern32":
        s3 = math.sqrt(3.0) * rho
        return outputscale * (1 + s3) * torch.exp(-s3)
    if kind == "matern12":
        return outputscale * torch.exp(-rho)
    raise ValueError(f"unknown kernel {kind}")


def kernel_matrix(X1: Tensor, X2: Tensor, lengthscale: Tensor, outputscale: float, kind: str) -> Tensor:
    return kernel_from_sq_dist(scaled_sq_dist(X1, X2, lengthscale), kind, outputscale)


@dataclass
class Standardize:
    """Standardize outcome transform state (outcome.py:236-345, 431-511)."""

    mean: float
    std: float

    @classmethod
    def fit(cls, Y: Tensor, min_stdv: float = 1e-8) -> "Standardize":
        if Y.shape[-2] == 1:
            std = 1.0
        else:
            std = float(Y.std(dim=-2, unbiased=True).item())
        if not std >= min_stdv:
            std = 1.0
        return cls(mean=float(Y.mean().item()), std=std)

    def transform(self, Y: Tensor) -> Tensor:
        return (Y - self.mean) / self.std


class ExactGP:
    """SingleTaskGP with fixed hyperparameters, evaluated in float64.

    ``train_Y`` is ``n x 1``; when ``standardize`` is True the Standardize
    outcome transform is fitted on it (the SingleTaskGP default) and the
    hyperparameters (noise, outputscale, mean constant) live in the
    standardised space, exactly as in the reference.
    """

    def __init__(self, train_X: Tensor, train_Y: Tensor, lengthscale, outputscale: float,
                 noise: float, mean_constant: float = 0.0, kind: str = "matern52",
                 standardize: bool = True) -> None:
        self.X = train_X.to(torch.float64)
        Y = train_Y.to(torch.float64).reshape(-1, 1)
        self.kind = kind
        d = self.X.shape[-1]
        self.lengthscale = torch.as_tensor(lengthscale, dtype=torch.float64).expand(d).clone()
        self.outputscale = float(outputscale)
        self.noise = float(noise)
        self.mean_constant = float(mean_constant)
        self.tf = Standardize.fit(Y) if standardize else Standardize(0.0, 1.0)
        y = self.tf.transform(Y).squeeze(-1)
        K = self.k(self.X, self.X)
        K.diagonal().add_(self.noise)
        self.L, self.jitter = psd_safe_cholesky(K, return_jitter=True)
        # a perturbation (standardised units) added to the posterior mean of the last
        # mean_shift.numel() points of every posterior call; None in normal use
        self.mean_shift: Tensor | None = None
        self.alpha = torch.cholesky_solve((y - self.mean_constant).unsqueeze(-1), self.L).squeeze(-1)

    def k(self, X1: Tensor, X2: Tensor) -> Tensor:
        return kernel_matrix(X1, X2, self.lengthscale, self.outputscale, self.kind)

    def posterior_standardized(self, X: Tensor) -> tuple[Tensor, Tensor]:
        """Mean and covariance in the standardised space for ``batch x m x d`` inputs."""
        Ks = self.k(X, self.X)                        # batch x m x n
        mean = self.mean_constant + Ks @ self.alpha
        if self.mean_shift is not None:  # sensitivity studies: shift the last points' means
            k = self.mean_shift.shape[-1]
            mean = torch.cat([mean[..., :-k], mean[..., -k:] + self.mean_shift], dim=-1)
        # one triangular solve with all batch x m right-hand sides (a batched solve
        # would broadcast the n x n factor over the batch)
        m, n = Ks.shape[-2], Ks.shape[-1]
        V = torch.linalg.solve_triangular(self.L, Ks.reshape(-1, n).transpose(0, 1), upper=False)
        V = V.transpose(0, 1).reshape(*Ks.shape[:-2], m, n)  # batch x m x n: rows L^-1 k(x_i, Xt)
        cov = self.k(X, X) - V @ V.transpose(-1, -2)
        return mean, cov

    def posterior(self, X: Tensor) -> tuple[Tensor, Tensor]:
        """Untransformed posterior mean (batch x m) and covariance (batch x m x m)."""
        mean, cov = self.posterior_standardized(X)
        s = self.tf.std
        return self.tf.mean + s * mean, (s * s) * cov
