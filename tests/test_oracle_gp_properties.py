"""Properties of the exact-GP oracle (oracle/gp.py) that pin its posterior
arithmetic where the reference's own arithmetic (gpytorch, external) cannot be
run here: the kernels' closed forms at known distances, a symmetric positive
semi-definite posterior covariance bounded by the prior, interpolation of
noise-free data, consistency of joint and separate posteriors, the prior far
from the data, and the Standardize transform's effect on the posterior."""

import math

import pytest
import torch

from oracle.gp import ExactGP, kernel_from_sq_dist, kernel_matrix


def _data(n=40, d=3, seed=0):
    g = torch.Generator().manual_seed(seed)
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    y = torch.sin(6 * X).sum(-1, keepdim=True) + 0.3 * torch.randn(n, 1, generator=g, dtype=torch.float64)
    return X, y, g


@pytest.mark.parametrize("kind, f", [
    ("matern52", lambda r: (1 + math.sqrt(5) * r + 5 * r * r / 3) * math.exp(-math.sqrt(5) * r)),
    ("matern32", lambda r: (1 + math.sqrt(3) * r) * math.exp(-math.sqrt(3) * r)),
    ("matern12", lambda r: math.exp(-r)),
    ("rbf", lambda r: math.exp(-0.5 * r * r)),
])
def test_kernel_closed_forms(kind, f):
    for r in (0.0, 0.3, 1.0, 2.5):
        v = float(kernel_from_sq_dist(torch.tensor(r * r, dtype=torch.float64), kind, 1.7))
        assert v == pytest.approx(1.7 * f(r), rel=1e-14, abs=1e-300)
    # ARD scaling: the difference (3, 4) over lengthscales (3, 4) is at distance sqrt(2)
    K = kernel_matrix(torch.tensor([[0.0, 0.0]], dtype=torch.float64),
                      torch.tensor([[3.0, 4.0]], dtype=torch.float64),
                      torch.tensor([3.0, 4.0], dtype=torch.float64), 1.0, kind)
    assert float(K) == pytest.approx(f(math.sqrt(2.0)), rel=1e-14)


@pytest.mark.parametrize("kind", ["matern52", "rbf"])
def test_posterior_covariance_is_psd_and_below_the_prior(kind):
    X, y, g = _data()
    gp = ExactGP(X, y, [0.4, 0.6, 0.5], 1.3, 1e-3, 0.1, kind)
    Xs = torch.rand(5, 6, 3, generator=g, dtype=torch.float64)
    mean, cov = gp.posterior_standardized(Xs)
    assert mean.shape == (5, 6) and cov.shape == (5, 6, 6)
    torch.testing.assert_close(cov, cov.transpose(-1, -2), atol=1e-14, rtol=0)
    assert float(torch.linalg.eigvalsh(cov).min()) > -1e-10
    prior = gp.k(Xs, Xs)
    # prior - posterior = V^T V is positive semi-definite
    assert float(torch.linalg.eigvalsh(prior - cov).min()) > -1e-10
    assert bool((cov.diagonal(dim1=-2, dim2=-1) <= prior.diagonal(dim1=-2, dim2=-1) + 1e-12).all())


def test_noise_free_data_are_interpolated():
    X, y, _ = _data(n=25)
    gp = ExactGP(X, y, [0.3, 0.3, 0.3], 1.0, 1e-9, 0.0, "matern52")
    mean, cov = gp.posterior(X.unsqueeze(0))
    torch.testing.assert_close(mean[0], y.squeeze(-1), atol=1e-5, rtol=0)
    assert float(cov.diagonal(dim1=-2, dim2=-1).max()) < 1e-6


def test_joint_and_separate_posteriors_agree():
    X, y, g = _data()
    gp = ExactGP(X, y, [0.4, 0.6, 0.5], 1.3, 1e-3, 0.1, "matern52")
    A = torch.rand(1, 4, 3, generator=g, dtype=torch.float64)
    B = torch.rand(1, 3, 3, generator=g, dtype=torch.float64)
    mj, cj = gp.posterior(torch.cat([A, B], dim=1))
    ma, ca = gp.posterior(A)
    mb, cb = gp.posterior(B)
    torch.testing.assert_close(mj[:, :4], ma, atol=1e-12, rtol=0)
    torch.testing.assert_close(mj[:, 4:], mb, atol=1e-12, rtol=0)
    torch.testing.assert_close(cj[:, :4, :4], ca, atol=1e-12, rtol=0)
    torch.testing.assert_close(cj[:, 4:, 4:], cb, atol=1e-12, rtol=0)


def test_far_from_the_data_the_prior_returns():
    X, y, _ = _data()
    gp = ExactGP(X, y, [0.2, 0.2, 0.2], 1.3, 1e-3, 0.25, "matern52")
    far = torch.full((1, 2, 3), 50.0, dtype=torch.float64)
    mean, cov = gp.posterior_standardized(far)
    torch.testing.assert_close(mean, torch.full_like(mean, 0.25), atol=1e-12, rtol=0)
    torch.testing.assert_close(cov.diagonal(dim1=-2, dim2=-1), torch.full((1, 2), 1.3, dtype=torch.float64),
                               atol=1e-12, rtol=0)


def test_standardize_scales_the_posterior():
    """With the outcome transform, the posterior equals the untransformed model's
    on the standardised targets, mapped back by mean + std * (.) and std^2 * (.)."""
    X, y, g = _data()
    gp = ExactGP(X, y, [0.4, 0.6, 0.5], 1.3, 1e-3, 0.1, "matern52", standardize=True)
    m, s = float(y.mean()), float(y.std(unbiased=True))
    assert gp.tf.mean == pytest.approx(m) and gp.tf.std == pytest.approx(s)
    plain = ExactGP(X, (y - m) / s, [0.4, 0.6, 0.5], 1.3, 1e-3, 0.1, "matern52", standardize=False)
    Xs = torch.rand(2, 5, 3, generator=g, dtype=torch.float64)
    mean, cov = gp.posterior(Xs)
    pm, pc = plain.posterior(Xs)
    torch.testing.assert_close(mean, m + s * pm, atol=1e-12, rtol=1e-12)
    torch.testing.assert_close(cov, s * s * pc, atol=1e-12, rtol=1e-12)
