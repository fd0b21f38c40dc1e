"""ORACLE (test infrastructure): qEI and qLogNEI of the reference in float64 on CPU.

Restated from:

* botorch/acquisition/monte_carlo.py:268-305 (sample-reducing forward: q
  reduction, then sample reduction) and :427-437 (qEI improvement,
  ``amax`` over q, ``mean`` over samples);
* botorch/acquisition/logei.py:67-68 (tau_relu 1e-6, tau_max 1e-2),
  :120-140 (fatmax q-reduction, logmeanexp sample reduction), :376-391 and
  :688-715 (log_fatplus improvement), :393-459 (baseline initialisation with
  cached root), :527-565 (joint posterior over [X_baseline; X]);
* botorch/acquisition/cached_cholesky.py:98-192 and
  botorch/utils/low_rank.py:84-172 (``sample_cached_cholesky``: bl = L_b^-1
  Sigma_bq, br = psd_safe_cholesky(Sigma_qq - bl bl^T, max_tries=6),
  Y = mu_q + [bl, br] z, NanError on non-finite samples);
* botorch/acquisition/utils.py:97-141 (best_f = max over baseline samples)
  and :276-437 (``prune_inferior_points``: 2048 posterior samples at the
  baseline, argmax counts, keep points that win at least once, in index
  order).

All arithmetic is float64 torch on the CPU. The gradient with respect to X
is torch autograd through this restatement, which is what the reference's
``torch.autograd.grad(loss.sum(), X)`` (botorch/generation/gen.py:466-469)
computes.
"""

from __future__ import annotations

import math
import warnings

import torch
from torch import Tensor

from oracle import safe_math
from oracle.gp import ExactGP, NanError, NotPSDError, psd_safe_cholesky
from oracle.sampling import draw_sobol_normal_samples, qlognei_base_samples

TAU_RELU = 1e-6
TAU_MAX = 1e-2


def _chunks(b: int, chunk: int):
    for i in range(0, b, chunk):
        yield slice(i, min(b, i + chunk))


def prune_inferior_points(model: ExactGP, X: Tensor, num_samples: int = 2048,
                          max_frac: float = 1.0, seed: int | None = None) -> Tensor:
    """Points of X that are the sampled argmax at least once (acquisition/utils.py:347-437).

    With ``seed=None`` the sampler seed is drawn from the global torch RNG
    exactly as ``MCSampler.__init__`` does (sampling/base.py:57-59).
    """
    if seed is None:
        seed = int(torch.randint(0, 1000000, (1,)).item())
    max_points = math.ceil(max_frac * X.shape[-2])
    with torch.no_grad():
        mean, cov = model.posterior(X)
        L = psd_safe_cholesky(cov)
        Z = draw_sobol_normal_samples(X.shape[-2], num_samples, seed)
        samples = mean.unsqueeze(0) + Z @ L.transpose(-1, -2)
    is_best = torch.argmax(samples, dim=-1)
    idcs, counts = torch.unique(is_best, return_counts=True)
    if len(idcs) > max_points:
        counts, order_idcs = torch.sort(counts, stable=True, descending=True)
        idcs = order_idcs[:max_points]
    return X[idcs]


def qei_from_samples(Y: Tensor, best_f) -> Tensor:
    """qEI reduction of samples S x b x q (monte_carlo.py:427-437, 194-195, 262-263)."""
    return (Y - torch.as_tensor(best_f).to(Y)).clamp_min(0).amax(dim=-1).mean(dim=0)


def qlogei_from_samples(Y: Tensor, best_f: Tensor, tau_relu: float = TAU_RELU,
                        tau_max: float = TAU_MAX) -> Tensor:
    """LogEI reduction of samples S x b x q with best_f broadcastable to S x b (logei.py:120-140)."""
    best_f = torch.as_tensor(best_f).to(Y).expand(Y.shape[:-1])
    li = safe_math.log_improvement(Y, best_f, tau=tau_relu)
    return safe_math.logmeanexp(safe_math.fatmax(li, dim=-1, tau=tau_max), dim=0)


class QExpectedImprovement:
    """qEI forward (monte_carlo.py:374-437) with a Sobol sampler of fixed seed."""

    def __init__(self, model: ExactGP, best_f: float, n_samples: int = 512, seed: int = 0) -> None:
        self.model = model
        self.best_f = float(best_f)
        self.n_samples = n_samples
        self.seed = seed
        self._Z: dict[int, Tensor] = {}

    def base_samples(self, q: int) -> Tensor:
        if q not in self._Z:
            self._Z[q] = draw_sobol_normal_samples(q, self.n_samples, self.seed)
        return self._Z[q]

    def __call__(self, X: Tensor, chunk: int = 256) -> Tensor:
        X = X if X.dim() > 2 else X.unsqueeze(0)
        X = X.to(torch.float64)
        q = X.shape[-2]
        Z = self.base_samples(q)
        out = []
        for sl in _chunks(X.shape[0], chunk):
            mean, cov = self.model.posterior(X[sl])
            Lq = psd_safe_cholesky(cov)
            Y = mean.unsqueeze(0) + torch.einsum("bij,sj->sbi", Lq, Z)
            out.append(qei_from_samples(Y, self.best_f))
        return torch.cat(out)


class QLogNoisyExpectedImprovement:
    """qLogNEI with the cached root decomposition (logei.py:246-565)."""

    def __init__(self, model: ExactGP, X_baseline: Tensor, n_samples: int = 512, seed: int = 0,
                 prune_baseline: bool = True, prune_seed: int | None = None,
                 tau_max: float = TAU_MAX, tau_relu: float = TAU_RELU,
                 cache_root: bool = True) -> None:
        self.model = model
        self.n_samples = n_samples
        self.seed = seed
        self.tau_max = tau_max
        self.tau_relu = tau_relu
        self.cache_root = cache_root
        X_baseline = X_baseline.to(torch.float64)
        if prune_baseline:
            X_baseline = prune_inferior_points(model, X_baseline, seed=prune_seed)
        self.X_baseline = X_baseline
        r = X_baseline.shape[-2]
        self.r = r
        with torch.no_grad():
            mean_b, cov_b = model.posterior(X_baseline)
            self.baseline_L = psd_safe_cholesky(cov_b)
            self.Z_baseline = draw_sobol_normal_samples(r, n_samples, seed)
            baseline_samples = mean_b.unsqueeze(0) + self.Z_baseline @ self.baseline_L.transpose(-1, -2)
            self.best_f = baseline_samples.amax(dim=-1)            # S
        self._Z: dict[int, Tensor] = {}

    def base_samples(self, q: int) -> Tensor:
        """S x (r+q) base samples; the first r are the baseline draw (normal.py:68-135).

        The uncached path (``cache_root=False``) uses the same matrix, as the
        reference's differential test does (test/acquisition/test_logei.py:513-623).
        """
        if q not in self._Z:
            self._Z[q] = qlognei_base_samples(self.r, q, self.n_samples, self.seed)
        return self._Z[q]

    def samples(self, X: Tensor) -> Tensor:
        """S x b x q posterior samples at the new points (low_rank.py:84-172)."""
        q = X.shape[-2]
        r = self.r
        Z = self.base_samples(q)
        Xb = self.X_baseline.expand(X.shape[0], r, X.shape[-1])
        X_full = torch.cat([Xb, X], dim=-2)
        mean, cov = self.model.posterior(X_full)
        if not self.cache_root:
            # the incumbent from the joint draw's own baseline samples, without gradient
            # (acquisition/utils.py:137-141)
            Yf = self._joint_samples(mean, cov, Z)
            return Yf[..., r:], Yf[..., :r].amax(dim=-1).detach()
        try:
            Y = self._cached_root_samples(mean, cov, Z, q)
        except (NanError, NotPSDError):
            # cached_cholesky.py:143-158: warn, then sample the joint posterior; the
            # incumbent stays the cached one (logei.py:501-512)
            warnings.warn("Low-rank cholesky updates failed due NaNs or due to an ill-conditioned "
                          "covariance matrix. Falling back to standard sampling.", RuntimeWarning)
            Y = self._joint_samples(mean, cov, Z)[..., r:]
        return Y, self.best_f.unsqueeze(-1).expand(Y.shape[:-1])

    @staticmethod
    def _joint_samples(mean: Tensor, cov: Tensor, Z: Tensor) -> Tensor:
        """S x b x (r+q) samples mean + chol(cov) z from the joint posterior
        (MultivariateNormal.rsample through psd_safe_cholesky of the whole covariance)."""
        Lf = psd_safe_cholesky(cov)
        return mean.unsqueeze(0) + torch.einsum("bij,sj->sbi", Lf, Z)

    def _cached_root_samples(self, mean: Tensor, cov: Tensor, Z: Tensor, q: int) -> Tensor:
        """S x b x q samples from the low-rank update of the cached root (low_rank.py:84-172)."""
        r = self.r
        bottom = cov[..., -q:, :]
        bl, br = bottom[..., :r], bottom[..., r:]
        if r > 0:
            bl_chol = torch.linalg.solve_triangular(
                self.baseline_L, bl.transpose(-1, -2), upper=False).transpose(-1, -2)
        else:
            bl_chol = bl
        br_chol = psd_safe_cholesky(br - bl_chol @ bl_chol.transpose(-1, -2), max_tries=6)
        new_Lq = torch.cat([bl_chol, br_chol], dim=-1)          # b x q x (r+q)
        Y = mean[..., -q:].unsqueeze(0) + torch.einsum("bij,sj->sbi", new_Lq, Z)
        if not torch.isfinite(Y).all():
            raise NanError("Samples contain nans or infs.")
        return Y

    def forward(self, X: Tensor) -> Tensor:
        Y, best_f = self.samples(X)
        return qlogei_from_samples(Y, best_f, self.tau_relu, self.tau_max)

    def __call__(self, X: Tensor, chunk: int = 256) -> Tensor:
        X = X if X.dim() > 2 else X.unsqueeze(0)
        X = X.to(torch.float64)
        return torch.cat([self.forward(X[sl]) for sl in _chunks(X.shape[0], chunk)])

    def value_and_grad(self, X: Tensor, chunk: int = 64) -> tuple[Tensor, Tensor]:
        """Value (b) and d value / d X (b x q x d), batch member by batch member."""
        X = X.to(torch.float64)
        vals, grads = [], []
        for sl in _chunks(X.shape[0], chunk):
            Xc = X[sl].detach().clone().requires_grad_(True)
            v = self.forward(Xc)
            (g,) = torch.autograd.grad(v.sum(), Xc)
            vals.append(v.detach())
            grads.append(g)
        return torch.cat(vals), torch.cat(grads)


def qei_value_and_grad(acqf: QExpectedImprovement, X: Tensor, chunk: int = 64):
    """Value and autograd gradient of the qEI oracle."""
    vals, grads = [], []
    for sl in _chunks(X.shape[0], chunk):
        Xc = X[sl].detach().to(torch.float64).clone().requires_grad_(True)
        v = acqf(Xc, chunk=chunk)
        (g,) = torch.autograd.grad(v.sum(), Xc)
        vals.append(v.detach())
        grads.append(g)
    return torch.cat(vals), torch.cat(grads)
