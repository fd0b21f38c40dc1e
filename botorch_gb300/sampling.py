"""Scrambled-Sobol normal base samples, bit-identical to the reference's.

The reference draws base samples on the host with
``torch.quasirandom.SobolEngine(D, scramble=True, seed)`` and maps them to
N(0, 1) by the inverse transform erfinv(2v - 1) * sqrt(2) with
v = 0.5 + (1 - eps) (u - 0.5) (botorch/sampling/qmc.py:59-97,
botorch/utils/sampling.py:114-143). This module calls the same engine and the
same float64 arithmetic, so the samples agree bit for bit for the same seed;
they are uploaded once per shape and stay resident on the device.
"""

from __future__ import annotations

import math

import torch
from torch import Tensor
from torch.quasirandom import SobolEngine

from botorch_gb300.exceptions import UnsupportedError


def draw_sobol_normal_samples(d: int, n: int, seed: int | None = None,
                              dtype: torch.dtype = torch.float64) -> Tensor:
    """n x d quasi-normal samples (host tensor)."""
    engine = SobolEngine(dimension=d, scramble=True, seed=seed)
    u = engine.draw(n, dtype=dtype)
    v = 0.5 + (1 - torch.finfo(u.dtype).eps) * (u - 0.5)
    return torch.erfinv(2 * v - 1) * math.sqrt(2)


class SobolQMCNormalSampler:
    """Sampler holding ``sample_shape`` and ``seed`` (botorch/sampling/normal.py:171-213).

    A missing seed is drawn from the global torch RNG as in
    botorch/sampling/base.py:57-59.
    """

    def __init__(self, sample_shape: torch.Size, seed: int | None = None) -> None:
        if not isinstance(sample_shape, torch.Size):
            raise TypeError(f"Expected `sample_shape` to be a `torch.Size` object, got {sample_shape}.")
        if len(sample_shape) != 1:
            raise UnsupportedError("only one sample dimension is supported")
        self.sample_shape = sample_shape
        self.seed = seed if seed is not None else int(torch.randint(0, 1000000, (1,)).item())
        self._cache: dict[int, Tensor] = {}

    @property
    def num_samples(self) -> int:
        return int(self.sample_shape[0])

    def forward(self, posterior) -> Tensor:
        """Samples ``sample_shape x batch x q x 1`` from the posterior with this sampler's
        base samples (botorch/sampling/normal.py:34-50): one q-dimensional Sobol draw,
        shared by every batch member (the batch dimensions of the base sample shape
        collapsed, botorch/sampling/normal.py:182-213)."""
        q = posterior.base_sample_shape[-2]
        nbatch = len(posterior.base_sample_shape) - 2
        base = self.base_samples(q).to(posterior.device).reshape(
            self.num_samples, *([1] * nbatch), q, 1)
        return posterior.rsample_from_base_samples(self.sample_shape, base)

    __call__ = forward

    def base_samples(self, dim: int) -> Tensor:
        """S x dim base samples of this sampler (host, float64), cached per dim."""
        if dim > SobolEngine.MAXDIM:
            raise UnsupportedError(f"SobolQMCSampler only supports dimensions <= {SobolEngine.MAXDIM}")
        if dim not in self._cache:
            self._cache[dim] = draw_sobol_normal_samples(dim, self.num_samples, self.seed)
        return self._cache[dim]
