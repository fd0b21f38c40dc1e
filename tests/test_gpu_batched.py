"""Many GPs of uneven size in one CUDA-graph launch, against each model's own call."""

import pytest
import torch

from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement
from botorch_gb300 import testing as T
from botorch_gb300.batched import Autotuner, ModelBatch

from tests.test_gpu_parity import DEV, gpu_model, rel

pytestmark = pytest.mark.gpu


def test_model_batch_matches_individual_calls(cuda_lib):
    works = T.many_gps(6, restarts=64, seed=1, n_range=(100, 1500))
    acqfs, Xs = [], []
    for w in works:
        gm = gpu_model(w)
        torch.manual_seed(0)
        acqfs.append(qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(
            torch.Size([w.n_samples]), seed=w.seed), precision="mixed"))
        Xs.append(w.X.to(DEV).contiguous())
    tuner = Autotuner(repeats=1)
    mb = ModelBatch(acqfs, [tuple(x.shape) for x in Xs], n_streams=3, tuner=tuner)
    g = torch.Generator().manual_seed(7)
    for step in range(2):
        if step == 1:  # replay with new candidates
            Xs = [torch.rand(x.shape, generator=g, dtype=torch.float64).to(DEV) for x in Xs]
        outs = [(v.clone(), gr.clone()) for v, gr in mb.value_and_grad(Xs)]
        for a, x, (v, gr) in zip(acqfs, Xs, outs):  # each acqf carries its tuned schedule
            ev, eg = a.value_and_grad_raw(x.contiguous(), True)
            assert rel(v, ev) < 1e-12 and rel(gr, eg) < 1e-12
    assert mb.launches >= 6 * 8
    assert len(tuner.choice) >= 1 and all(len(t) >= 2 for t in tuner.timings.values())
    assert sorted(i for lane in mb.lanes for i in lane) == list(range(6))


def _group_problems(n_models, restarts, seed, n_range, q=2):
    works = T.many_gps(n_models, restarts=restarts, seed=seed, n_range=n_range, q=q)
    acqfs, Xs = [], []
    for w in works:
        gm = gpu_model(w)
        torch.manual_seed(0)
        acqfs.append(qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(
            torch.Size([w.n_samples]), seed=w.seed), precision="mixed"))
        Xs.append(w.X.to(DEV).contiguous())
    return acqfs, Xs


@pytest.mark.parametrize("q", [2, 5])
def test_model_group_matches_individual_calls(cuda_lib, q):
    """One launch per stage for all problems (bgb_group_*): the same values and
    gradients as each problem's own call, over uneven n (100..2500) and d, for
    two candidate sets."""
    from botorch_gb300.batched import ModelGroup

    acqfs, Xs = _group_problems(7, 64, 3, (100, 2500), q=q)
    shapes = [tuple(x.shape) for x in Xs]
    assert ModelGroup.supported(acqfs, shapes)
    mg = ModelGroup(acqfs, shapes)
    assert 8 <= mg.launches <= 22  # 7 stages + one adjoint (and finish) per d bucket
    g = torch.Generator().manual_seed(11)
    for step in range(2):
        if step == 1:
            Xs = [torch.rand(x.shape, generator=g, dtype=torch.float64).to(DEV) for x in Xs]
        outs = [(v.clone(), gr.clone()) for v, gr in mg.value_and_grad(Xs)]
        for a, x, (v, gr) in zip(acqfs, Xs, outs):
            ev, eg = a.value_and_grad_raw(x.contiguous(), True)
            assert torch.isfinite(v).all() and torch.isfinite(gr).all()
            assert rel(v, ev) < 1e-12 and rel(gr, eg) < 1e-12, (rel(v, ev), rel(gr, eg))


def test_model_group_rejects_unsupported_members(cuda_lib):
    """A member on the FFMA GEMMs (or float64, or joint sampling) is outside the grouped path."""
    from botorch_gb300.batched import ModelGroup
    from botorch_gb300.exceptions import UnsupportedError

    acqfs, Xs = _group_problems(2, 16, 5, (100, 300))
    acqfs[1].use_tensor_cores = False
    shapes = [tuple(x.shape) for x in Xs]
    assert not ModelGroup.supported(acqfs, shapes)
    with pytest.raises(UnsupportedError):
        ModelGroup(acqfs, shapes)
