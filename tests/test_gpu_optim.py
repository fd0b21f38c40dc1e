"""Raw samples -> restarts -> L-BFGS-B on the CUDA acquisition path."""

import pytest
import torch

from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement
from botorch_gb300 import testing as T
from botorch_gb300.optim import draw_sobol_samples, evaluate_raw, gen_candidates_scipy, optimize_acqf

from tests.test_gpu_parity import DEV, gpu_model, rel

pytestmark = pytest.mark.gpu


def _acqf(gm, w, precision):
    torch.manual_seed(0)
    return qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(
        torch.Size([256]), seed=0), precision=precision)


def test_optimize_acqf_improves_and_agrees_with_fp64(cuda_lib):
    w = T.qlognei_diff(b=1, q=2, n=128)
    gm = gpu_model(w)
    acqf, a64 = _acqf(gm, w, "mixed"), _acqf(gm, w, "fp64")
    d = w.train_X.shape[-1]
    bounds = torch.stack([torch.zeros(d), torch.ones(d)]).double().to(DEV)
    X, v = optimize_acqf(acqf, bounds, q=2, num_restarts=4, raw_samples=128,
                         options={"maxiter": 30}, seed=0)
    info = gen_candidates_scipy.last_info
    assert info["mode"] == "per-restart"  # the default, as the reference's
    assert info["f"] <= info["f0"]  # the summed restart objective decreased
    assert X.shape == (2, d) and bool(((X >= 0) & (X <= 1)).all())
    v_raw = evaluate_raw(acqf, draw_sobol_samples(bounds.cpu(), 128, 2, seed=0))
    assert float(v) >= float(v_raw.max()) - 1e-6
    v64, _ = a64.value_and_grad_raw(X.unsqueeze(0).contiguous(), False)
    assert rel(v.reshape(1), v64) < 1e-5
    # the graph-replayed and eager objectives give the same optimisation
    X2, v2 = optimize_acqf(acqf, bounds, q=2, num_restarts=4, raw_samples=128,
                           options={"maxiter": 30}, seed=0, use_graph=False)
    assert torch.allclose(X, X2) and float(v) == float(v2)


def test_per_restart_and_aggregated_modes(cuda_lib):
    """The per-restart mode (the reference's fast path and the default): every
    restart's own value does not decrease; the aggregated mode decreases the summed
    objective; both stay in the box."""
    w = T.qlognei_diff(b=1, q=2, n=128)
    gm = gpu_model(w)
    acqf = _acqf(gm, w, "mixed")
    d = w.train_X.shape[-1]
    X0 = draw_sobol_samples(torch.stack([torch.zeros(d), torch.ones(d)]).double(), 6, 2, seed=1).to(DEV)
    v0, _ = acqf.value_and_grad_raw(X0.contiguous(), False)
    v0 = v0.clone()
    X, v = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": 20}, use_parallel_mode=True)
    info = gen_candidates_scipy.last_info
    assert info["mode"] == "per-restart" and len(info["nit_per_restart"]) == 6
    assert bool((v >= v0 - 1e-9).all()), (v, v0)
    assert bool(((X >= 0) & (X <= 1)).all())
    Xa, va = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": 20}, use_parallel_mode=False)
    assert gen_candidates_scipy.last_info["mode"] == "aggregated"
    assert float(va.sum()) >= float(v0.sum()) - 1e-9


@pytest.mark.parametrize("n,q,d,seed", [(1, 2, 3, 0), (257, 16, 50, 0), (1000, 3, 7, 11)])
def test_device_sobol_samples_equal_the_host_engine(cuda_lib, n, q, d, seed):
    """The raw samples drawn on the device are, bit for bit, torch's SobolEngine
    draw mapped to the box on the host (the reference's draw_sobol_samples)."""
    g = torch.Generator().manual_seed(seed + 1)
    lo = -torch.rand(d, generator=g, dtype=torch.float64)
    hi = lo + 0.5 + torch.rand(d, generator=g, dtype=torch.float64)
    bounds = torch.stack([lo, hi])
    host = draw_sobol_samples(bounds, n, q, seed=seed)
    dev = draw_sobol_samples(bounds.to(DEV), n, q, seed=seed)
    assert dev.device.type == "cuda" and dev.shape == (n, q, d)
    assert torch.equal(dev.cpu(), host)
