"""Seeded synthetic workloads for the GP-posterior + MC-acquisition path.

The reference publishes no benchmark data for this path, so every workload is
synthetic, generated on the host in float64 from a seeded ``torch.Generator``
(the role botorch/utils/testing.py and botorch/utils/test_helpers.py play in
the reference). The generators are:

* ``qei_small``: d=6, n=64, X ~ U[0,1]^6, y = sum_j sin(3 x_j) + N(0, 0.01^2);
  Matern-5/2 ARD with lengthscales 0.5, outputscale 1, noise 1e-4, mean 0;
  qEI with best_f = max(y) on 512 x 4 x 6 candidates, 256 Sobol samples.
* ``qlognei_diff``: the same generator at d=12, n=1024; qLogNEI on
  2048 x 4 x 12 candidates with 512 Sobol samples.
* ``qlognei_branin``: d=20, y = sum of Branin over 10 disjoint random
  coordinate pairs mapped to [-5,10] x [0,15] + N(0, 0.01^2); lengthscales
  U[0.2, 1.0]; noise 1e-4; qLogNEI on b x 8 x 20 candidates, 512 samples.
  n=4096 is the headline point, n=8192 the large-n precision case.
* ``rff_draw``: y = sqrt(2/F) sum_i w_i cos(omega_i . x + beta_i) + noise,
  the random-feature GP draw of the many-model and optimisation workloads.
* ``optimization_step``: d=50, n=4096, X ~ U[0,1]^50, y = an RFF draw (2048
  features, ARD lengthscales ~ U[0.1, 2.0]) + N(0, 0.01^2); Matern-5/2 with those
  lengthscales, outputscale 1, noise 1e-4; qLogNEI with 1024 samples, optimised
  from 65536 raw q-batches of q=16 over 64 restarts.
* ``log_areas_workload``: the inner loop of qLogEHVI with m=2 objectives and
  q=4 candidates: objective samples N(0.5, 0.3^2) for 128 MC samples x 256
  restarts (B = 32768 sample-batches), their q-subsets of sizes 1..4, and the
  64 cells of the non-dominated region of a 63-point front on
  y2 = 1 - y1^2 above the reference point (-0.1, -0.1) (the outer cells
  unbounded above).
* ``many_gps``: independent problems of uneven size, n ~ log-uniform [100, 4000]
  and d ~ uniform {4..30} per model, X ~ U[0,1]^d, y = an RFF draw (1024
  features, lengthscale 0.3) + N(0, 0.01^2); Matern-5/2 with lengthscale 0.3,
  outputscale 1, noise 1e-4; qLogNEI on 256 restarts x q=2 with 256 samples.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import torch
from torch import Tensor


@dataclass
class Workload:
    name: str
    train_X: Tensor
    train_Y: Tensor
    lengthscale: Tensor
    outputscale: float
    noise: float
    mean_constant: float
    kernel: str
    X: Tensor                       # b x q x d candidates
    n_samples: int
    seed: int
    acqf: str                       # "qEI" or "qLogNEI"
    best_f: float | None = None
    extra: dict = field(default_factory=dict)


def _branin(x1: Tensor, x2: Tensor) -> Tensor:
    """Branin on [-5,10] x [0,15] (formula of botorch/test_functions/synthetic.py:199)."""
    b = 5.1 / (4 * math.pi ** 2)
    c = 5 / math.pi
    t = 1 / (8 * math.pi)
    return (x2 - b * x1 ** 2 + c * x1 - 6) ** 2 + 10 * (1 - t) * torch.cos(x1) + 10


def qei_small(b: int = 512, q: int = 4, seed: int = 0) -> Workload:
    g = torch.Generator().manual_seed(seed)
    d, n = 6, 64
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    y = torch.sin(3 * X).sum(-1) + 0.01 * torch.randn(n, generator=g, dtype=torch.float64)
    Xc = torch.rand(b, q, d, generator=g, dtype=torch.float64)
    return Workload("qei_small_d6_n64", X, y.unsqueeze(-1), torch.full((d,), 0.5, dtype=torch.float64),
                    1.0, 1e-4, 0.0, "matern52", Xc, 256, 0, "qEI", best_f=float(y.max()))


def qlognei_diff(b: int = 2048, q: int = 4, n: int = 1024, seed: int = 0) -> Workload:
    g = torch.Generator().manual_seed(seed)
    d = 12
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    y = torch.sin(3 * X).sum(-1) + 0.01 * torch.randn(n, generator=g, dtype=torch.float64)
    Xc = torch.rand(b, q, d, generator=g, dtype=torch.float64)
    return Workload(f"qlognei_d12_n{n}", X, y.unsqueeze(-1), torch.full((d,), 0.5, dtype=torch.float64),
                    1.0, 1e-4, 0.0, "matern52", Xc, 512, 0, "qLogNEI")


def qlognei_branin(n: int = 4096, b: int = 4096, q: int = 8, d: int = 20, seed: int = 0) -> Workload:
    g = torch.Generator().manual_seed(seed)
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    perm = torch.randperm(d, generator=g)
    y = torch.zeros(n, dtype=torch.float64)
    for p in range(d // 2):
        i, j = int(perm[2 * p]), int(perm[2 * p + 1])
        y = y + _branin(-5 + 15 * X[:, i], 15 * X[:, j])
    y = y + 0.01 * torch.randn(n, generator=g, dtype=torch.float64)
    ls = 0.2 + 0.8 * torch.rand(d, generator=g, dtype=torch.float64)
    Xc = torch.rand(b, q, d, generator=g, dtype=torch.float64)
    return Workload(f"qlognei_branin_d{d}_n{n}_q{q}", X, y.unsqueeze(-1), ls, 1.0, 1e-4, 0.0,
                    "matern52", Xc, 512, 0, "qLogNEI")


def rff_draw(X: Tensor, n_features: int, lengthscale: Tensor, g: torch.Generator,
             noise_std: float = 0.01) -> Tensor:
    """Random Fourier feature draw of a squared-exponential GP at X (n x d), plus noise."""
    d = X.shape[-1]
    omega = torch.randn(n_features, d, generator=g, dtype=torch.float64) / lengthscale
    beta = 2 * math.pi * torch.rand(n_features, generator=g, dtype=torch.float64)
    w = torch.randn(n_features, generator=g, dtype=torch.float64)
    f = math.sqrt(2.0 / n_features) * torch.cos(X @ omega.T + beta) @ w
    return f + noise_std * torch.randn(X.shape[0], generator=g, dtype=torch.float64)


def many_gps(n_models: int = 64, restarts: int = 256, q: int = 2, n_samples: int = 256,
             seed: int = 0, n_range: tuple[int, int] = (100, 4000),
             d_range: tuple[int, int] = (4, 30)) -> list[Workload]:
    g = torch.Generator().manual_seed(seed)
    out = []
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    for m in range(n_models):
        n = int(round(math.exp(lo + (hi - lo) * float(torch.rand(1, generator=g, dtype=torch.float64)))))
        d = int(torch.randint(d_range[0], d_range[1] + 1, (1,), generator=g))
        X = torch.rand(n, d, generator=g, dtype=torch.float64)
        ls = torch.full((d,), 0.3, dtype=torch.float64)
        y = rff_draw(X, 1024, ls, g)
        Xc = torch.rand(restarts, q, d, generator=g, dtype=torch.float64)
        out.append(Workload(f"many_gps_{m}_n{n}_d{d}", X, y.unsqueeze(-1), ls, 1.0, 1e-4, 0.0,
                            "matern52", Xc, n_samples, seed + m, "qLogNEI"))
    return out


def optimization_step(n: int = 4096, d: int = 50, seed: int = 0) -> Workload:
    g = torch.Generator().manual_seed(seed)
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    ls = 0.1 + 1.9 * torch.rand(d, generator=g, dtype=torch.float64)
    y = rff_draw(X, 2048, ls, g)
    return Workload(f"optimize_d{d}_n{n}", X, y.unsqueeze(-1), ls, 1.0, 1e-4, 0.0, "matern52",
                    torch.empty(0, 16, d, dtype=torch.float64), 1024, seed, "qLogNEI",
                    extra={"raw_samples": 65536, "restarts": 64, "q": 16})



@dataclass
class LogAreasWorkload:
    B: int                      # sample-batches (MC samples x restarts)
    q: int
    m: int
    obj_subsets: list           # [i = 1..q] (B, C(q, i), i, m)
    cell_lower: Tensor          # (nc, m)
    cell_upper: Tensor
    tau_relu: float = 1e-6      # the reference's TAU_RELU (botorch/acquisition/logei.py:67)
    tau_max: float = 1e-2       # the reference's TAU_MAX

    @property
    def nc(self) -> int:
        return int(self.cell_lower.shape[0])

    def areas_per_step(self) -> int:
        """(sample-batch, cell, subset) log areas of one pass over all subset sizes."""
        return self.B * self.nc * sum(int(o.shape[1]) for o in self.obj_subsets)


def log_areas_workload(mc: int = 128, restarts: int = 256, q: int = 4, n_pareto: int = 63,
                       seed: int = 0, dtype: torch.dtype = torch.float64,
                       device: torch.device | str = "cpu") -> LogAreasWorkload:
    import itertools

    g = torch.Generator().manual_seed(seed)
    B = mc * restarts
    Y = 0.5 + 0.3 * torch.randn(B, q, 2, generator=g, dtype=torch.float64)
    subsets = []
    for i in range(1, q + 1):
        idx = torch.tensor(list(itertools.combinations(range(q), i)), dtype=torch.long)  # C(q,i) x i
        subsets.append(Y[:, idx.reshape(-1)].reshape(B, idx.shape[0], i, 2))
    y1 = torch.sort(torch.rand(n_pareto, generator=g, dtype=torch.float64)).values
    y2 = 1.0 - y1 ** 2
    ref = -0.1
    inf = float("inf")
    # cell k spans y1 in [x_k, x_{k+1}) above the front: x_0 = ref, x_k = y1_{k-1}
    xs = torch.cat([torch.tensor([ref], dtype=torch.float64), y1])
    lower = torch.stack([xs, torch.cat([y2, torch.tensor([ref], dtype=torch.float64)])], dim=-1)
    upper = torch.stack([torch.cat([y1, torch.tensor([inf], dtype=torch.float64)]),
                         torch.full((n_pareto + 1,), inf, dtype=torch.float64)], dim=-1)
    cast = lambda t: t.to(device=device, dtype=dtype).contiguous()  # noqa: E731
    return LogAreasWorkload(B, q, 2, [cast(o) for o in subsets], cast(lower), cast(upper))
