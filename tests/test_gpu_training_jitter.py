"""The training-side psd_safe_cholesky jitter retry on the GPU (bgb_gp_fit,
bgb_psd_safe_cholesky) against the float64 oracle.

linear_operator's psd_safe_cholesky (called for the training covariance by the
exact prediction strategy, settings botorch/__init__.py:51-56) first factors the
matrix as given, then adds jitter 1e-8 x 10^i to the diagonal for i < 6 until
the factorisation succeeds, else raises NotPSDError. The workloads below make
the first attempts fail for a reason far above rounding: an RBF kernel of
lengthscale 5 on 64 points of [0, 1] has numerical rank about 10 (its smallest
eigenvalues sit far below float64 rounding), so with noise 0 the factorisation
meets a non-positive pivot, and with noise -2e-8 so does the first jitter
level; the accepted level leaves a margin of >= 1e-8 over rounding.
"""

import ctypes

import pytest
import torch

from botorch_gb300 import (ConstantMean, GaussianLikelihood, NotPSDError, RBFKernel, ScaleKernel,
                           SingleTaskGP)
from botorch_gb300 import _native as nat
from oracle.gp import ExactGP

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def smooth_problem():
    X = torch.linspace(0, 1, 64, dtype=torch.float64).unsqueeze(-1)
    y = torch.sin(6 * X) + 0.1 * X
    return X, y


def rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float((a - b).norm() / b.norm())


def smooth_model(X, y):
    return SingleTaskGP(X, y, likelihood=GaussianLikelihood(1e-4),
                        covar_module=ScaleKernel(RBFKernel(ard_num_dims=1, lengthscale=5.0), outputscale=1.0),
                        mean_module=ConstantMean(0.0), device=DEV)


@pytest.mark.parametrize("noise,expected", [(0.0, 1e-8), (-2e-8, 1e-7)])
def test_training_jitter_matches_oracle(cuda_lib, noise, expected):
    X, y = smooth_problem()
    model = smooth_model(X, y)
    model.set_hyperparameters(noise=noise)
    om = ExactGP(X, y, torch.tensor([5.0], dtype=torch.float64), 1.0, noise, 0.0, "rbf")
    assert om.jitter == pytest.approx(expected, rel=1e-12)
    assert model.train_jitter == pytest.approx(om.jitter, rel=1e-12)
    # the factor of K + (noise + jitter) I: backward stable, norm-wise close
    assert rel(model.L, om.L) < 1e-9, rel(model.L, om.L)
    # alpha = (K + (noise + jitter) I)^-1 (y - m) at condition ~ 64 / jitter: the
    # oracle's plain Cholesky solve and the library's solve with one refinement step
    # agree to about cond x eps
    assert rel(model.alpha, om.alpha) < 1e-5, rel(model.alpha, om.alpha)
    # backward-stable solve: residual ~ eps ||K|| ||alpha|| / ||y|| (||alpha|| ~ 1e7 here)
    Kj = om.k(om.X, om.X) + (noise + om.jitter) * torch.eye(64, dtype=torch.float64)
    yt = om.tf.transform(y).squeeze(-1)
    a = model.alpha.cpu()
    res = (Kj @ a - yt).norm() / yt.norm()
    bound = 4 * 2.0 ** -52 * float(torch.linalg.matrix_norm(Kj, 2) * a.norm() / yt.norm())
    assert float(res) < bound, (float(res), bound)


def test_training_not_psd_raises(cuda_lib):
    X, y = smooth_problem()
    model = smooth_model(X, y)
    # K - I is indefinite beyond the largest jitter (1e-3): psd_safe_cholesky gives up
    with pytest.raises(NotPSDError):
        model.set_hyperparameters(noise=-1.0)


def test_psd_safe_cholesky_entry_point(cuda_lib):
    """bgb_psd_safe_cholesky directly: jitter levels and the give-up code."""
    stream = nat.stream_handle(DEV)
    n = 4
    ws = torch.empty(cuda_lib.bgb_cholesky_workspace_bytes(n), dtype=torch.uint8, device=DEV)
    L = torch.empty(n, n, dtype=torch.float64, device=DEV)
    jit = ctypes.c_double(-1.0)
    # diag(1, 1, 1, -5e-8): fails plain and at 1e-8, succeeds at 1e-7
    A = torch.eye(n, dtype=torch.float64, device=DEV)
    A[3, 3] = -5e-8
    rc = cuda_lib.bgb_psd_safe_cholesky(A.data_ptr(), n, n, L.data_ptr(), n, 6, 1e-8,
                                        ctypes.byref(jit), ws.data_ptr(), ws.numel(), stream)
    assert rc == nat.BGB_OK and jit.value == pytest.approx(1e-7, rel=1e-12)
    assert float(L[3, 3]) == pytest.approx((1e-7 - 5e-8) ** 0.5, rel=1e-9)
    # -I: no jitter up to 1e-3 helps
    A = -torch.eye(n, dtype=torch.float64, device=DEV)
    rc = cuda_lib.bgb_psd_safe_cholesky(A.data_ptr(), n, n, L.data_ptr(), n, 6, 1e-8,
                                        ctypes.byref(jit), ws.data_ptr(), ws.numel(), stream)
    assert rc == nat.BGB_NOT_PSD
    assert jit.value == pytest.approx(1e-3, rel=1e-12)
