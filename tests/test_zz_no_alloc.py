"""bgb_acq_forward_backward_noalloc through the C ABI.

The no-allocation entry point keeps its scratch in one fixed device array that
every call shares. It must return what bgb_acq_forward_backward returns with a
caller-supplied workspace, call after call. The file name sorts last, so in a
full run these tests also run after every other GPU test of the process.
"""

import ctypes

import pytest
import torch

from botorch_gb300 import (ConstantMean, GaussianLikelihood, MaternKernel, ScaleKernel,
                           SingleTaskGP, SobolQMCNormalSampler, qLogNoisyExpectedImprovement)
from botorch_gb300 import _native as nat
from botorch_gb300 import testing as T

DEV = torch.device("cuda:0")


def rel(a, b):
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


def make_acqf(w, precision):
    d = w.train_X.shape[-1]
    model = SingleTaskGP(w.train_X, w.train_Y, likelihood=GaussianLikelihood(w.noise),
                         covar_module=ScaleKernel(MaternKernel(nu=2.5, ard_num_dims=d,
                                                               lengthscale=w.lengthscale),
                                                  outputscale=w.outputscale),
                         mean_module=ConstantMean(w.mean_constant), device=DEV)
    torch.manual_seed(0)
    return qLogNoisyExpectedImprovement(model, w.train_X, sampler=SobolQMCNormalSampler(
        torch.Size([w.n_samples]), seed=w.seed), precision=precision)


def outputs(b, q, d):
    value = torch.full((b,), float("nan"), dtype=torch.float64, device=DEV)
    grad = torch.full((b, q, d), float("nan"), dtype=torch.float64, device=DEV)
    status = torch.full((b,), -7, dtype=torch.int32, device=DEV)
    return value, grad, status


def with_workspace(lib, acq, X):
    """The existing entry point, scratch from a caller-owned workspace."""
    b, q, d = X.shape
    value, grad, status = outputs(b, q, d)
    nbytes = lib.bgb_acq_workspace_bytes(ctypes.byref(acq), b)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=DEV)
    rc = lib.bgb_acq_forward_backward(ctypes.byref(acq), nat.ptr(X), b, nat.ptr(value),
                                      nat.ptr(grad), nat.ptr(status), nat.ptr(ws), nbytes,
                                      nat.stream_handle(DEV))
    assert rc == nat.BGB_OK, rc
    torch.cuda.synchronize()
    return value, grad, status


def no_alloc(lib, acq, X):
    b, q, d = X.shape
    value, grad, status = outputs(b, q, d)
    rc = lib.bgb_acq_forward_backward_noalloc(ctypes.byref(acq), nat.ptr(X), b, nat.ptr(value),
                                              nat.ptr(grad), nat.ptr(status),
                                              nat.stream_handle(DEV))
    assert rc == nat.BGB_OK, rc
    torch.cuda.synchronize()
    return value, grad, status


# (workload, precision, value bound, gradient bound): the float64 bar of the
# parity tests, and the mixed bar (1e-5 value, 1e-4 gradient) on a headline-shaped
# workload (d=20, q=8, n=4096) in the tensor-core form.
CASES = [
    pytest.param(lambda: T.qlognei_diff(b=96, q=4, n=1024), "fp64", 1e-9, 1e-9, id="fp64_n1024_q4"),
    pytest.param(lambda: T.qlognei_branin(n=4096, b=128, q=8, d=20), "mixed", 1e-5, 1e-4,
                 id="mixed_tc_n4096_q8"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("make,precision,tv,tg", CASES)
def test_no_alloc_matches_workspace_entry_point(cuda_lib, make, precision, tv, tg):
    w = make()
    acqf = make_acqf(w, precision)
    q, d = w.X.shape[-2], w.X.shape[-1]
    acq = acqf._acq_struct(q)
    half = w.X.shape[0] // 2
    # two calls in a row on different t-batches, then the workspace entry point on each
    X1 = w.X[:half].to(DEV).contiguous()
    X2 = w.X[half:].to(DEV).contiguous()
    got = [no_alloc(cuda_lib, acq, X1), no_alloc(cuda_lib, acq, X2)]
    want = [with_workspace(cuda_lib, acq, X1), with_workspace(cuda_lib, acq, X2)]
    for (gv, gg, gs), (wv, wg, ws) in zip(got, want):
        assert torch.equal(gs, ws) and int(ws.abs().max()) == 0
        assert rel(gv, wv) < tv, rel(gv, wv)
        assert rel(gg, wg) < tg, rel(gg, wg)
    # and the same t-batches again: nothing left over in the shared array changes them
    again = no_alloc(cuda_lib, acq, X1)
    assert rel(again[0], got[0][0]) < tv and rel(again[1], got[0][1]) < tg


@pytest.mark.gpu
def test_no_alloc_rejects_calls_beyond_its_scratch(cuda_lib):
    w = T.qlognei_branin(n=4096, b=2048, q=8, d=20)
    acqf = make_acqf(w, "mixed")
    acq = acqf._acq_struct(8)
    X = w.X.to(DEV).contiguous()
    b = X.shape[0]
    assert cuda_lib.bgb_acq_workspace_bytes(ctypes.byref(acq), b) > nat.BGB_NOALLOC_SCRATCH_BYTES
    value, grad, status = outputs(b, 8, 20)
    rc = cuda_lib.bgb_acq_forward_backward_noalloc(ctypes.byref(acq), nat.ptr(X), b,
                                                   nat.ptr(value), nat.ptr(grad), nat.ptr(status),
                                                   nat.stream_handle(DEV))
    assert rc == nat.BGB_ERR_SCRATCH_LIMIT
    torch.cuda.synchronize()
    assert bool(torch.isnan(value).all()) and int(status.min()) == -7   # nothing launched
    with pytest.raises(RuntimeError, match="no-allocation scratch"):
        nat.check(rc, "qLogNEI")
    # a slice that fits runs
    fit = 64
    assert cuda_lib.bgb_acq_workspace_bytes(ctypes.byref(acq), fit) <= nat.BGB_NOALLOC_SCRATCH_BYTES
    v, g, s = no_alloc(cuda_lib, acq, X[:fit].contiguous())
    assert int(s.abs().max()) == 0 and bool(torch.isfinite(v).all())
