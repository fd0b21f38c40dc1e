"""ORACLE (test infrastructure): Sobol normal base samples of the reference.

Restates botorch/sampling/qmc.py:59-97 (``NormalQMCEngine.draw`` with
``inv_transform=True``), botorch/utils/sampling.py:114-143
(``draw_sobol_normal_samples``) and the base-sample layout of
``SobolQMCNormalSampler`` / ``NormalMCSampler._update_base_samples``
(botorch/sampling/normal.py:68-135, 182-213). The scrambled Sobol points come
from the installed ``torch.quasirandom.SobolEngine``, the same engine the
reference calls, so the samples are bit-exact by construction.
"""

from __future__ import annotations

import math

import torch
from torch import Tensor
from torch.quasirandom import SobolEngine


def draw_sobol_normal_samples(d: int, n: int, seed: int | None,
                              dtype: torch.dtype = torch.float64) -> Tensor:
    """n x d quasi-normal samples by the inverse transform (qmc.py:80-83)."""
    engine = SobolEngine(dimension=d, scramble=True, seed=seed)
    u = engine.draw(n, dtype=dtype)
    v = 0.5 + (1 - torch.finfo(u.dtype).eps) * (u - 0.5)
    return torch.erfinv(2 * v - 1) * math.sqrt(2)


def qlognei_base_samples(r: int, q: int, n_samples: int, seed: int) -> Tensor:
    """S x (r+q) base samples of the cached-root qLogNEI forward.

    The sampler draws an (r+q)-dimensional Sobol set and overwrites its first r
    columns with the r-dimensional draw used for the baseline samples
    (normal.py:110-135 via cached_cholesky.py:172-192).
    """
    full = draw_sobol_normal_samples(r + q, n_samples, seed)
    if r > 0:
        full[:, :r] = draw_sobol_normal_samples(r, n_samples, seed)
    return full
