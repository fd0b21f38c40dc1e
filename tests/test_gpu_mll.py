"""Exact MLL and its gradient on the GPU against the float64 oracle."""

import pytest
import torch

from botorch_gb300 import testing as T
from botorch_gb300.mll import exact_marginal_log_likelihood
from oracle.mll import exact_mll

from tests.test_gpu_parity import gpu_model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["matern52", "matern32", "matern12", "rbf"])
def test_mll_matches_oracle(cuda_lib, kind):
    w = T.qlognei_branin(n=300, b=1, q=1, d=7)
    w.kernel = kind
    w.mean_constant = 0.15
    gm = gpu_model(w)
    v, g = exact_marginal_log_likelihood(gm)
    y = gm.train_targets.cpu()
    ov, og = exact_mll(w.train_X, y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, kind)
    assert abs(v - ov) <= 1e-9 * abs(ov)
    assert float((g["lengthscale"] - og["lengthscale"]).norm() / og["lengthscale"].norm()) < 1e-9
    for name in ("outputscale", "noise", "mean_constant"):
        assert abs(g[name] - og[name]) <= 1e-9 * max(abs(og[name]), 1e-12), name


def test_mll_ragged_sizes(cuda_lib):
    # n not a multiple of the 32-point tiles, d spanning two buckets
    for n, d in ((33, 3), (95, 17)):
        g = torch.Generator().manual_seed(n)
        w = T.qlognei_branin(n=n, b=1, q=1, d=d, seed=n)
        gm = gpu_model(w)
        v, gr = exact_marginal_log_likelihood(gm)
        ov, og = exact_mll(w.train_X, gm.train_targets.cpu(), w.lengthscale, w.outputscale, w.noise,
                           w.mean_constant, w.kernel)
        assert abs(v - ov) <= 1e-9 * abs(ov)
        assert float((gr["lengthscale"] - og["lengthscale"]).norm() / og["lengthscale"].norm()) < 1e-9
