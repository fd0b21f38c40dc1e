"""The posterior's sampling surface on the GPU: SobolQMCNormalSampler.forward(posterior)
(botorch/sampling/normal.py:34-50), GPyTorchPosterior.rsample_from_base_samples / rsample
(botorch/posteriors/gpytorch.py:86-127) and posterior(observation_noise=True), against
the float64 oracle's MVN samples: mean + psd_safe_cholesky(covariance) z."""

import pytest
import torch

from botorch_gb300 import SobolQMCNormalSampler
from botorch_gb300 import testing as T
from oracle.gp import psd_safe_cholesky

from tests.test_gpu_parity import gpu_model, oracle_model, rel

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def oracle_samples(mean, cov, Z):
    """S x b x q samples mean + L z with L = psd_safe_cholesky(cov) per batch member."""
    L = psd_safe_cholesky(cov)
    return mean.unsqueeze(0) + torch.einsum("bij,sj->sbi", L, Z)


@pytest.mark.parametrize("batch_shape", [(6,), (2, 3), ()])
def test_sampler_forward_matches_oracle(cuda_lib, batch_shape):
    w = T.qlognei_diff(b=6, q=3, n=150)
    gm, om = gpu_model(w), oracle_model(w)
    X = w.X.reshape(*batch_shape, 3, 12) if batch_shape else w.X[0]
    sampler = SobolQMCNormalSampler(torch.Size([128]), seed=7)
    Y = sampler(gm.posterior(X.to(DEV)))
    assert Y.shape == torch.Size([128, *batch_shape, 3, 1])
    mean, cov = om.posterior(X.reshape(-1, 3, 12))
    ref = oracle_samples(mean, cov, sampler.base_samples(3))
    assert rel(Y.reshape(128, -1, 3), ref) < 1e-9


def test_rsample_from_base_samples_and_observation_noise(cuda_lib):
    w = T.qlognei_diff(b=8, q=4, n=120)
    gm, om = gpu_model(w), oracle_model(w)
    Z = torch.randn(64, 1, 4, 1, dtype=torch.float64, generator=torch.Generator().manual_seed(3))
    mean, cov = om.posterior(w.X)
    for noise in (False, True):
        post = gm.posterior(w.X.to(DEV), observation_noise=noise)
        c = cov + (w.noise * om.tf.std ** 2) * torch.eye(4, dtype=torch.float64) if noise else cov
        assert rel(post.covariance_matrix, c) < 1e-10
        Y = post.rsample_from_base_samples(torch.Size([64]), Z.to(DEV))
        assert Y.shape == torch.Size([64, 8, 4, 1])
        assert rel(Y.squeeze(-1), oracle_samples(mean, c, Z.reshape(64, 4))) < 1e-9
    with pytest.raises(RuntimeError):
        post.rsample_from_base_samples(torch.Size([32]), Z.to(DEV))
    # i.i.d. draws: the sample mean of 20000 draws within 5 standard errors
    Ys = gm.posterior(w.X[:1].to(DEV)).rsample(torch.Size([20000])).reshape(20000, 4).cpu()
    se = cov[0].diagonal().sqrt() / 20000 ** 0.5
    assert bool(((Ys.mean(0) - mean[0]).abs() < 5 * se).all())


def test_rsample_singular_covariance_uses_jitter(cuda_lib):
    """Two identical points make a member's covariance singular: psd_safe_cholesky adds
    jitter for that batch member only, as the oracle does."""
    w = T.qlognei_diff(b=4, q=3, n=100)
    w.X[1, 1] = w.X[1, 0]
    gm, om = gpu_model(w), oracle_model(w)
    sampler = SobolQMCNormalSampler(torch.Size([32]), seed=0)
    Y = sampler(gm.posterior(w.X.to(DEV))).squeeze(-1)
    mean, cov = om.posterior(w.X)
    ref = oracle_samples(mean, cov, sampler.base_samples(3))
    assert rel(Y[:, [0, 2, 3]], ref[:, [0, 2, 3]]) < 1e-9
    # the jittered member: a rank-deficient block amplifies rounding
    assert rel(Y[:, 1], ref[:, 1]) < 1e-6
