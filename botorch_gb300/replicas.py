"""Host logic of running the acquisition path as independent replicas, one per GPU.

Once the model and the qLogNEI baseline are cached, the t-batches of a call
are independent (nothing couples two t-batches), so N GPUs run N replicas of
the whole path on their own candidate batches with no collective on the data
path (weak scaling). The only cross-rank steps are the ones a measurement
needs: a barrier around the timed region and the maximum of the ranks' times.
These helpers work with any initialised ``torch.distributed`` backend (NCCL on
GPUs, gloo on the host).
"""

from __future__ import annotations

import torch
from torch import Tensor


def rank_candidates(X0: Tensor, rank: int, seed_base: int = 1000) -> Tensor:
    """Candidates of one replica: rank 0 keeps ``X0``; rank k > 0 draws its own
    ``X0.shape`` batch from U[0, 1)^d with seed ``seed_base + k`` (float64, host)."""
    if rank == 0:
        return X0
    g = torch.Generator().manual_seed(seed_base + rank)
    return torch.rand(X0.shape, generator=g, dtype=torch.float64)


def max_over_ranks(value: float, device: torch.device | str = "cpu") -> float:
    """The maximum of ``value`` over all ranks (the value itself without a process group)."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def evals_per_second(world: int, b: int, steps: int, total_ms: float) -> float:
    """Whole-job rate: every rank evaluates ``b`` t-batches per step for ``steps``
    steps, and the job takes the slowest rank's ``total_ms``."""
    if total_ms <= 0:
        raise ValueError("total_ms must be positive")
    return world * b * steps / (total_ms / 1e3)
