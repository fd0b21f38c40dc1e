"""The oracle against the reference's own property and differential tests.

Restated from test/acquisition/test_monte_carlo.py:98-149 (qEI known answers),
test/acquisition/test_logei.py:103-204 (LogEI bounds) and :513-623 (cached vs
uncached root), test/utils/test_safe_math.py:316-380 (Pareto kernel), plus
central finite differences of the oracle's autograd gradient.
"""

import math

import pytest
import torch

from oracle import safe_math
from oracle.acquisition import (QExpectedImprovement, QLogNoisyExpectedImprovement,
                                qei_from_samples, qlogei_from_samples)
from oracle.gp import ExactGP, NotPSDError, psd_safe_cholesky
from botorch_gb300 import testing as T

F64 = torch.float64


def test_qei_known_answers():
    Y = torch.zeros(2, 1, 1, dtype=F64)
    assert qei_from_samples(Y, 0.0).item() == 0.0
    assert qei_from_samples(Y, -1.0).item() == 1.0
    Yb = torch.zeros(3, 2, 2, dtype=F64)
    Yb[:, 0, 0] = 1.0
    assert qei_from_samples(Yb, 0.0).tolist() == [1.0, 0.0]
    assert qei_from_samples(Yb, -1.0).tolist() == [2.0, 1.0]


def test_qlogei_bounds():
    tau = 1e-6
    Y = torch.zeros(2, 1, 1, dtype=F64)
    v = qlogei_from_samples(Y, torch.tensor(0.0, dtype=F64)).exp().item()
    assert 0 < v <= tau
    v = qlogei_from_samples(Y, torch.tensor(-1.0, dtype=F64)).exp().item()
    assert 1.0 <= v <= 1.0 + tau
    lv = qlogei_from_samples(Y, torch.tensor(1.0, dtype=F64)).item()
    assert 0.0 <= math.exp(lv) <= tau
    assert -100 < lv < -1


def test_pareto_value_and_derivatives_at_zero():
    x = torch.zeros(1, dtype=F64, requires_grad=True)
    p = safe_math.pareto(x, 2.0)
    (g,) = torch.autograd.grad(p.sum(), x, create_graph=True)
    (h,) = torch.autograd.grad(g.sum(), x)
    assert p.item() == 1.0 and g.item() == -1.0 and h.item() == 1.0


def test_fatplus_close_to_relu():
    x = torch.linspace(-5, 5, 101, dtype=F64)
    for tau in (1.0, 1e-2, 1e-6):
        err = (safe_math.fatplus(x, tau) - x.clamp_min(0)).abs().max().item()
        assert err <= tau * (math.log(2) + 0.1) + 1e-15


def test_psd_safe_cholesky_jitter_schedule():
    A = torch.tensor([[1.0, 1.0], [1.0, 1.0]], dtype=F64)  # singular PSD: needs jitter
    L = psd_safe_cholesky(A)
    assert torch.allclose(L @ L.T, A, atol=1e-6)
    with pytest.raises(NotPSDError):
        psd_safe_cholesky(-torch.eye(3, dtype=F64))


def _model(w):
    return ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)


def test_cached_vs_uncached_root():
    w = T.qlognei_diff(b=8, q=3, n=60)
    m = _model(w)
    torch.manual_seed(0)
    a = QLogNoisyExpectedImprovement(m, w.train_X, 64, 0, prune_baseline=False)
    b = QLogNoisyExpectedImprovement(m, w.train_X, 64, 0, prune_baseline=False, cache_root=False)
    va, ga = a.value_and_grad(w.X)
    vb, gb = b.value_and_grad(w.X)
    assert torch.allclose(va, vb, rtol=1e-8, atol=1e-8)
    assert torch.allclose(ga, gb, rtol=1e-6, atol=1e-6)


def test_oracle_gradient_matches_central_differences():
    w = T.qlognei_diff(b=4, q=2, n=80)
    m = _model(w)
    torch.manual_seed(0)
    a = QLogNoisyExpectedImprovement(m, w.train_X, 128, 0)
    _, g = a.value_and_grad(w.X)
    h = 1e-6
    X = w.X.clone()
    fd = torch.zeros_like(X)
    for idx in [(0, 0, 0), (1, 1, 3), (2, 0, 7), (3, 1, 11)]:
        Xp, Xm = X.clone(), X.clone()
        Xp[idx] += h
        Xm[idx] -= h
        fd[idx] = (a(Xp)[idx[0]] - a(Xm)[idx[0]]) / (2 * h)
        assert abs(fd[idx] - g[idx]) <= 1e-5 * max(1.0, abs(g[idx].item())), (idx, fd[idx], g[idx])


def test_qei_oracle_runs_and_is_nonnegative():
    w = T.qei_small(b=32)
    m = _model(w)
    v = QExpectedImprovement(m, w.best_f, w.n_samples, w.seed)(w.X)
    assert v.shape == (32,) and bool((v >= 0).all())


def test_oracle_reproduces_parity_fixtures():
    """The committed parity fixtures are the oracle's output on these inputs."""
    from pathlib import Path

    import numpy as np
    from oracle.acquisition import qei_value_and_grad

    fix = np.load(Path(__file__).resolve().parent / "golden" / "parity_fixtures.npz")
    w = T.qei_small()
    v, g = qei_value_and_grad(QExpectedImprovement(_model(w), w.best_f, w.n_samples, w.seed), w.X)
    assert np.allclose(v.numpy(), fix["qei_small_value"], rtol=1e-12, atol=1e-15)
    assert np.allclose(g.numpy(), fix["qei_small_grad"], rtol=1e-10, atol=1e-13)
    w = T.qlognei_diff()
    torch.manual_seed(0)
    a = QLogNoisyExpectedImprovement(_model(w), w.train_X, w.n_samples, w.seed)
    assert np.array_equal(a.X_baseline.numpy(), fix["qlognei_diff_Xb"])
    v, g = a.value_and_grad(w.X[:32])
    assert np.allclose(v.numpy(), fix["qlognei_diff_value"][:32], rtol=1e-12)
    assert np.allclose(g.numpy(), fix["qlognei_diff_grad"][:32], rtol=1e-9, atol=1e-12)
