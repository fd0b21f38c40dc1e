"""CUDA-graph replay of the acquisition call against the eager call."""

import pytest
import torch

from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement
from botorch_gb300 import testing as T

from tests.test_gpu_parity import DEV, gpu_model, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_replay_matches_eager(cuda_lib, precision):
    w = T.qlognei_branin(n=1024, b=96, q=8, d=20)
    gm = gpu_model(w)
    torch.manual_seed(0)
    acqf = qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(
        torch.Size([256]), seed=0), precision=precision)
    X1 = w.X[:48].to(DEV).contiguous()
    X2 = w.X[48:].to(DEV).contiguous()
    e1 = [t.clone() for t in acqf.value_and_grad_raw(X1, True)]
    e2 = [t.clone() for t in acqf.value_and_grad_raw(X2, True)]
    for _ in range(2):  # capture, then replays with different inputs
        g1 = [t.clone() for t in acqf.graphed_value_and_grad(X1, True)]
        g2 = [t.clone() for t in acqf.graphed_value_and_grad(X2, True)]
        for (gv, gg), (ev, eg) in (((g1[0], g1[1]), (e1[0], e1[1])), ((g2[0], g2[1]), (e2[0], e2[1]))):
            assert rel(gv, ev) < 1e-12 and rel(gg, eg) < 1e-12
    assert acqf.graph_launches(48, 8) >= 8


def test_public_forward_with_graphs(cuda_lib):
    w = T.qlognei_branin(n=512, b=32, q=4, d=20)
    gm = gpu_model(w)
    torch.manual_seed(0)
    acqf = qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(
        torch.Size([128]), seed=0), precision="mixed")
    X = w.X.to(DEV)
    ref = acqf(X).detach().clone()
    acqf.use_cuda_graphs = True
    outs = []
    for _ in range(3):
        Xg = X.clone().requires_grad_(True)
        v = acqf(Xg)
        v.sum().backward()
        outs.append((v.detach(), Xg.grad))
    # results returned earlier are not overwritten by later replays
    assert all(rel(o[0], ref) < 1e-12 for o in outs)
    assert rel(outs[0][1], outs[2][1]) < 1e-12
