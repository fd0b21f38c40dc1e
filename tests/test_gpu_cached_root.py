"""Cached-root sampling of qLogNEI against joint sampling, on the GPU path.

The reference's differential tests, run through the C ABI:

* ``test_cache_root`` (test/acquisition/test_logei.py:513-623): qLogNEI with
  ``cache_root=True`` and ``cache_root=False`` agree (atol 1e-4 in float64
  there), and breaking the cached root makes the acquisition function fall back
  to standard sampling with one BotorchWarning
  (botorch/acquisition/cached_cholesky.py:143-158);
* ``test_sample_cached_cholesky`` (test/utils/test_low_rank.py:46-175): samples
  from the low-rank update of the cached root equal samples from the joint
  posterior, and so do their gradients.

Here both routes are the library's kernels (BGB_FLAG_JOINT_SAMPLING,
BGB_FLAG_UNCACHED_ROOT), and each is also held to the float64 oracle.
"""

import math
import warnings

import pytest
import torch

from botorch_gb300 import (BotorchWarning, ConstantMean, GaussianLikelihood, MaternKernel, NanError,
                           RBFKernel, ScaleKernel, SingleTaskGP, SobolQMCNormalSampler,
                           qLogNoisyExpectedImprovement)
from botorch_gb300 import _native as nat
from botorch_gb300 import testing as T
from oracle.acquisition import QLogNoisyExpectedImprovement as OQLogNEI
from oracle.gp import ExactGP

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")
TOL = {"fp64": (1e-9, 1e-9), "mixed": (1e-5, 1e-4)}


def rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


def make_pair(X, Y, ls, outputscale, noise, mean, kind, Xb, S, seed, precision, cache_root=True):
    d = X.shape[-1]
    base = RBFKernel(ard_num_dims=d, lengthscale=ls) if kind == "rbf" else \
        MaternKernel(nu=2.5, ard_num_dims=d, lengthscale=ls)
    gm = SingleTaskGP(X, Y, likelihood=GaussianLikelihood(noise),
                      covar_module=ScaleKernel(base, outputscale=outputscale),
                      mean_module=ConstantMean(mean), device=DEV)
    ga = qLogNoisyExpectedImprovement(gm, Xb, sampler=SobolQMCNormalSampler(torch.Size([S]), seed=seed),
                                      prune_baseline=False, cache_root=cache_root, precision=precision)
    om = ExactGP(X, Y, torch.as_tensor(ls, dtype=torch.float64).expand(d), outputscale, noise, mean, kind)
    oa = OQLogNEI(om, Xb, S, seed, prune_baseline=False, cache_root=cache_root)
    return ga, oa


def value_grad(acqf, X):
    Xd = X.to(DEV).requires_grad_(True)
    v = acqf(Xd)
    v.sum().backward()
    return v.detach().cpu(), Xd.grad.cpu()


def oracle_value_grad(oa, X):
    X3 = X.reshape(-1, *X.shape[-2:])
    v, g = oa.value_and_grad(X3)
    return v.reshape(X.shape[:-2]), g.reshape(X.shape)


def cache_root_problem():
    """The setup of test_cache_root (test/acquisition/test_logei.py:517-573): 3 training
    points in [0,1]^2, y = sin(2 pi x_1) + N(0, 1), standardised; the hyperparameters of
    its state dict that the default SingleTaskGP has (noise 0.0895, constant mean
    -0.4545); the default RBF kernel at its initial lengthscale, the mode of
    LogNormal(sqrt(2) + log(2) / 2, sqrt(3)) (models/utils/gpytorch_modules.py:100-133)."""
    torch.manual_seed(1234)
    train_X = torch.rand(3, 2, dtype=torch.float64)
    train_Y = (torch.sin(train_X * 2 * math.pi) + torch.randn(3, 2, dtype=torch.float64))[..., :1]
    train_Y = (train_Y - train_Y.mean(0)) / train_Y.std(0)
    ls = math.exp(math.sqrt(2) + 0.5 * math.log(2) - 3.0)
    return train_X, train_Y, ls


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cache_root_matches_uncached(cuda_lib, precision):
    train_X, train_Y, ls = cache_root_problem()
    args = (train_X, train_Y, ls, 1.0, 0.0895, -0.4545, "rbf", train_X, 5, 0, precision)
    cached, o_cached = make_pair(*args, cache_root=True)
    uncached, o_uncached = make_pair(*args, cache_root=False)
    tv, tg = TOL[precision]
    g = torch.Generator().manual_seed(0)
    for q in (1, 3):
        for batch_shape in (torch.Size([]), torch.Size([3]), torch.Size([4, 3])):
            X = 0.3 + 0.05 * torch.randn(*batch_shape, q, 2, generator=g, dtype=torch.float64)
            v1, g1 = value_grad(cached, X)
            v2, g2 = value_grad(uncached, X)
            # the reference's bound between the two routes (float64): atol 1e-4 on exp(value)
            assert torch.allclose(v1.exp(), v2.exp(), atol=1e-4, rtol=0)
            assert torch.allclose(g1, g2, atol=1e-4 * max(1.0, float(g1.abs().max())), rtol=0)
            # each route against the oracle's route of the same name
            ov1, og1 = oracle_value_grad(o_cached, X)
            ov2, og2 = oracle_value_grad(o_uncached, X)
            assert rel(v1, ov1) < tv and rel(v2, ov2) < tv, (rel(v1, ov1), rel(v2, ov2))
            if precision == "fp64":
                assert rel(g1, og1) < tg and rel(g2, og2) < tg, (rel(g1, og1), rel(g2, og2))
            else:
                # the mixed path's per-sample float32 terms (log_fatplus, its derivative and
                # the smooth maxima with fast intrinsics) are averaged over only 5 samples
                # here: gradient within 5e-4 (the reference's own float32 version of this
                # test allows atol 1e-1)
                assert rel(g1, og1) < 5e-4 and rel(g2, og2) < 5e-4, (rel(g1, og1), rel(g2, og2))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_broken_cached_root_falls_back_to_joint_sampling(cuda_lib, precision):
    """As the reference's test, break the cached root (here its inverse: NaN) so the
    low-rank update yields non-finite samples: one warning, then joint sampling with the
    cached incumbent, equal to the oracle taking the same fallback."""
    w = T.qlognei_diff(b=16, q=3, n=200)
    args = (w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel,
            w.train_X[:40], w.n_samples, w.seed, precision)
    ga, oa = make_pair(*args)
    v0, g0 = value_grad(ga, w.X)  # the cached route, before breaking it
    ga._Lb_inv.fill_(float("nan"))
    oa.baseline_L = torch.zeros_like(oa.baseline_L)
    with warnings.catch_warnings(record=True) as ws:
        warnings.simplefilter("always")
        v, g = value_grad(ga, w.X)
    assert sum(issubclass(x.category, BotorchWarning) for x in ws) == 1
    with warnings.catch_warnings(record=True):
        warnings.simplefilter("always")
        ov, og = oracle_value_grad(oa, w.X)
    tv, tg = TOL[precision]
    assert rel(v, ov) < tv and rel(g, og) < tg, (rel(v, ov), rel(g, og))
    # joint sampling of a well-conditioned problem equals the cached route (to the
    # rounding of the precision)
    ev, eg = (1e-9, 1e-8) if precision == "fp64" else (1e-5, 1e-4)
    assert rel(v, v0) < ev and rel(g, g0) < eg, (rel(v, v0), rel(g, g0))


def test_joint_sampling_equals_cached_root_sampling(cuda_lib):
    """test_sample_cached_cholesky's setup: 10 training points in [0,1]^2, the baseline
    all but the last q, the new points the last q (over several t-batch shapes): the
    cached-root route and the joint route give the same values and gradients."""
    torch.manual_seed(0)
    train_X = torch.rand(10, 2, dtype=torch.float64)
    train_Y = torch.randn(10, 1, dtype=torch.float64)
    for q in (1, 3, 9):
        ga, _ = make_pair(train_X, train_Y, 0.5, 1.0, 1e-2, 0.0, "matern52", train_X[:-q], 64, 0, "fp64")
        for shape in (torch.Size([]), torch.Size([4]), torch.Size([4, 2])):
            X = train_X[-q:].expand(*shape, q, 2).contiguous()
            v1, g1 = value_grad(ga, X)
            Xd = X.reshape(-1, q, 2).to(DEV)
            acq, wsb = ga._call_struct(q, nat.BGB_FLAG_JOINT_SAMPLING)
            v2, g2, st = ga._native_call(Xd, True, acq, wsb)
            assert int(st.max()) == 0
            assert torch.allclose(v1.reshape(-1), v2.cpu(), rtol=1e-9, atol=1e-12)
            assert torch.allclose(g1.reshape(-1, q, 2), g2.cpu(), rtol=1e-7, atol=1e-9)


def test_joint_sampling_nan_candidates_raise(cuda_lib):
    """NaN candidates: the cached route fails, the joint route's psd_safe_cholesky
    meets NaN and raises NanError, as the reference's does."""
    w = T.qlognei_diff(b=4, q=2, n=100)
    ga, _ = make_pair(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant,
                      w.kernel, w.train_X[:20], 64, 0, "fp64")
    X = w.X.clone()
    X[1, 0, 0] = float("nan")
    with warnings.catch_warnings(record=True) as ws:
        warnings.simplefilter("always")
        with pytest.raises(NanError):
            ga(X.to(DEV))
    assert sum(issubclass(x.category, BotorchWarning) for x in ws) == 1
