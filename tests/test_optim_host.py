"""Raw-sample initialisation host logic (no GPU)."""

import pytest
import torch

from botorch_gb300.optim import draw_sobol_samples, initialize_q_batch


def test_draw_sobol_samples_in_box_and_reproducible():
    bounds = torch.tensor([[-1.0, 0.0, 2.0], [1.0, 0.5, 3.0]], dtype=torch.float64)
    X = draw_sobol_samples(bounds, 64, 4, seed=3)
    assert X.shape == (64, 4, 3)
    assert bool((X >= bounds[0]).all() and (X <= bounds[1]).all())
    assert torch.equal(X, draw_sobol_samples(bounds, 64, 4, seed=3))
    # same point set as the engine over q * d dimensions, scaled into the box
    raw = torch.quasirandom.SobolEngine(12, scramble=True, seed=3).draw(64, dtype=torch.float64)
    assert torch.allclose(X, bounds[0] + (bounds[1] - bounds[0]) * raw.view(64, 4, 3))


def test_initialize_q_batch_keeps_the_best_and_is_without_replacement():
    g = torch.Generator().manual_seed(0)
    X = torch.rand(200, 2, 3, generator=g, dtype=torch.float64)
    v = torch.randn(200, generator=g, dtype=torch.float64)
    for seed in range(5):
        Xs, vs = initialize_q_batch(X, v, 10, eta=1.0, generator=torch.Generator().manual_seed(seed))
        assert Xs.shape == (10, 2, 3)
        assert float(vs.max()) == float(v.max())
        rows = {tuple(x.flatten().tolist()) for x in Xs}
        assert len(rows) == 10


def test_initialize_q_batch_edge_cases():
    X = torch.rand(8, 1, 2, dtype=torch.float64)
    assert initialize_q_batch(X, torch.zeros(8, dtype=torch.float64), 8)[0] is X
    Xs, _ = initialize_q_batch(X, torch.ones(8, dtype=torch.float64), 3)  # equal values: random pick
    assert Xs.shape == (3, 1, 2)
    with pytest.raises(RuntimeError):
        initialize_q_batch(X, torch.zeros(8, dtype=torch.float64), 9)
    # large eta with extreme values: the temperature is lowered until weights are finite
    v = torch.tensor([0.0] * 7 + [1e6], dtype=torch.float64)
    Xs, vs = initialize_q_batch(X, v, 2, eta=1e4)
    assert float(vs.max()) == 1e6
