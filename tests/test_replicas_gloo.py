"""Replica host logic on two gloo ranks (CPU): distinct candidates per rank,
max-over-ranks timing, and the whole-job rate the bench reports."""

import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from botorch_gb300 import replicas


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        X0 = torch.full((4, 3, 2), 0.5, dtype=torch.float64)
        X = replicas.rank_candidates(X0, rank)
        t = replicas.max_over_ranks(10.0 * (rank + 1))
        torch.distributed.barrier()
        out[rank] = (float(X.sum()), t)
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    # rank 0 keeps the shared candidates, rank 1 draws its own
    assert res[0][0] == pytest.approx(12.0)
    assert res[1][0] != pytest.approx(12.0)
    # both ranks see the slowest rank's time
    assert res[0][1] == res[1][1] == 20.0
    assert replicas.evals_per_second(world, 4096, 5, res[0][1]) == pytest.approx(2 * 4096 * 5 / 0.02)


def test_single_process_fallbacks():
    X0 = torch.zeros(2, 2, 2, dtype=torch.float64)
    assert replicas.rank_candidates(X0, 0) is X0
    X1 = replicas.rank_candidates(X0, 1)
    assert X1.shape == X0.shape and torch.equal(X1, replicas.rank_candidates(X0, 1))
    assert replicas.max_over_ranks(3.5) == 3.5
    with pytest.raises(ValueError):
        replicas.evals_per_second(1, 1, 1, 0.0)
