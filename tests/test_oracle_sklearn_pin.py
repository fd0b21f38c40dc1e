"""The oracle's exact-GP posterior against an independent implementation of the
same published algorithm: scikit-learn's GaussianProcessRegressor with fixed
hyperparameters (no optimiser).

The reference's posterior arithmetic lives in gpytorch / linear_operator
(exact prediction strategy: mean = m + K(X, Xt) (K + s2 I)^-1 (y - m),
covariance = K(X, X) - K(X, Xt) (K + s2 I)^-1 K(Xt, X), as gpytorch's
ExactGP.__call__ in eval mode), which is not installable here; scikit-learn
computes the same predictive equations (Rasmussen & Williams, Algorithm 2.1)
with its own Cholesky and solves, and its Matern(nu=2.5) and RBF kernels are
the same functions of the lengthscale-scaled distance as gpytorch's
MaternKernel(nu=2.5) and RBFKernel. The comparison runs in the standardised
outcome space of the reference's Standardize transform, with a zero mean
(scikit-learn's prior mean is 0 when normalize_y is off).
"""

import numpy as np
import pytest
import torch

from oracle.gp import ExactGP

sklearn_gp = pytest.importorskip("sklearn.gaussian_process")
kernels = pytest.importorskip("sklearn.gaussian_process.kernels")


def _problem(n, d, seed):
    g = torch.Generator().manual_seed(seed)
    X = torch.rand(n, d, generator=g, dtype=torch.float64)
    y = torch.sin(3 * X).sum(-1, keepdim=True) + 0.05 * torch.randn(n, 1, generator=g,
                                                                     dtype=torch.float64)
    Xq = torch.rand(6, 3, d, generator=g, dtype=torch.float64)
    ls = 0.3 + 0.5 * torch.rand(d, generator=g, dtype=torch.float64)
    return X, y, Xq, ls


@pytest.mark.parametrize("kind", ["matern52", "rbf"])
@pytest.mark.parametrize("n,d", [(40, 3), (200, 6)])
def test_posterior_matches_sklearn(kind, n, d):
    X, y, Xq, ls = _problem(n, d, seed=n + d)
    outputscale, noise = 1.7, 1e-3
    om = ExactGP(X, y, ls, outputscale, noise, mean_constant=0.0, kind=kind)
    ys = om.tf.transform(y).squeeze(-1).numpy()  # the standardised targets the GP sees
    base = (kernels.Matern(length_scale=ls.numpy(), nu=2.5) if kind == "matern52"
            else kernels.RBF(length_scale=ls.numpy()))
    k = kernels.ConstantKernel(outputscale, constant_value_bounds="fixed") * base
    gpr = sklearn_gp.GaussianProcessRegressor(kernel=k, alpha=noise, optimizer=None,
                                              normalize_y=False)
    gpr.fit(X.numpy(), ys)
    mean, cov = om.posterior_standardized(Xq)
    for i in range(Xq.shape[0]):
        m_ref, c_ref = gpr.predict(Xq[i].numpy(), return_cov=True)
        np.testing.assert_allclose(mean[i].numpy(), m_ref, rtol=0, atol=1e-10 * max(1, np.abs(m_ref).max()))
        np.testing.assert_allclose(cov[i].numpy(), c_ref, rtol=0, atol=1e-10 * outputscale)


def test_kernel_matrix_matches_sklearn():
    X, _, Xq, ls = _problem(30, 5, seed=3)
    from oracle.gp import kernel_matrix

    for kind, base in (("matern52", kernels.Matern(length_scale=ls.numpy(), nu=2.5)),
                       ("matern32", kernels.Matern(length_scale=ls.numpy(), nu=1.5)),
                       ("matern12", kernels.Matern(length_scale=ls.numpy(), nu=0.5)),
                       ("rbf", kernels.RBF(length_scale=ls.numpy()))):
        K = kernel_matrix(Xq[0], X, ls, 2.0, kind).numpy()
        K_ref = 2.0 * base(Xq[0].numpy(), X.numpy())
        np.testing.assert_allclose(K, K_ref, rtol=1e-13, atol=1e-15)
