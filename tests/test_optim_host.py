"""Raw-sample initialisation host logic (no GPU)."""

import platform
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


class _FakeAcqf:
    """Independent concave objectives per t-batch on the CPU:
    value_i = -sum (w_i (X_i - c)^2 + (X_i - c)^4), w_i anisotropic and uneven."""

    device = torch.device("cpu")

    def __init__(self, b, q, d, fail_at=None):
        g = torch.Generator().manual_seed(4)
        self.w = 0.5 + 20 * torch.rand(b, q, d, generator=g, dtype=torch.float64) ** 3
        self.c = 0.2 + 0.6 * torch.rand(1, q, d, generator=g, dtype=torch.float64)
        self.calls = 0
        self.fail_at = fail_at

    def value_and_grad_raw(self, X, need_grad, **kw):
        self.calls += 1
        if self.fail_at is not None and self.calls >= self.fail_at:
            raise ValueError("planted failure")
        return self.rows(X, self.w[:X.shape[0]], need_grad)

    def rows(self, X, w, need_grad):
        r = X - self.c
        return -(w * r * r + r ** 4).sum((1, 2)), (-(2 * w * r + 4 * r ** 3) if need_grad else None)


def test_per_restart_mode_equals_independent_runs():
    """Each restart's own L-BFGS-B with batched rounds gives exactly the result of
    running scipy on that restart alone (the rows do not interact)."""
    import numpy as np
    from scipy.optimize import minimize

    from botorch_gb300.optim import gen_candidates_scipy

    b, q, d = 7, 2, 3
    acqf = _FakeAcqf(b, q, d)
    X0 = torch.rand(b, q, d, generator=torch.Generator().manual_seed(9), dtype=torch.float64)
    X, v = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": 50}, use_parallel_mode=True)
    info = gen_candidates_scipy.last_info
    assert info["mode"] == "per-restart" and len(set(info["nit_per_restart"])) > 1
    for i in range(b):
        def f(x, i=i):  # restart i alone
            vv, gg = acqf.rows(torch.from_numpy(x.reshape(1, q, d)), acqf.w[i:i + 1], True)
            return -float(vv[0]), -gg.numpy().reshape(-1)
        res = minimize(f, X0[i].numpy().reshape(-1), method="L-BFGS-B", jac=True,
                       bounds=[(0.0, 1.0)] * (q * d), options={"maxiter": 50})
        assert np.array_equal(res.x, X[i].numpy().reshape(-1)), i
    assert torch.allclose(X, acqf.c.expand(b, q, d), atol=1e-3)
    assert info["nfev"] >= max(info["nit_per_restart"])  # one round per evaluation of the slowest restart


@pytest.mark.timeout(60)
def test_per_restart_mode_raises_without_hanging():
    from botorch_gb300.optim import gen_candidates_scipy

    acqf = _FakeAcqf(5, 2, 2, fail_at=4)
    X0 = torch.rand(5, 2, 2, dtype=torch.float64)
    with pytest.raises(RuntimeError, match="batched acquisition evaluation failed"):
        gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": 50}, use_parallel_mode=True)


@pytest.mark.timeout(120)
def test_per_restart_drivers_agree(monkeypatch):
    """scipy's reverse-communication routine stepped per restart (used where it passes
    its self-test) and one scipy optimiser per host thread (the fallback) give the
    same restarts bit for bit."""
    import numpy as np

    import botorch_gb300.optim as O

    b, q, d = 6, 2, 3
    X0 = torch.rand(b, q, d, generator=torch.Generator().manual_seed(13), dtype=torch.float64)
    X_rc, _ = O.gen_candidates_scipy(X0, _FakeAcqf(b, q, d), 0.0, 1.0, {"maxiter": 40}, use_parallel_mode=True)
    info_rc = O.gen_candidates_scipy.last_info
    monkeypatch.setattr(O, "_lbfgsb_rc", lambda: None)
    X_th, _ = O.gen_candidates_scipy(X0, _FakeAcqf(b, q, d), 0.0, 1.0, {"maxiter": 40}, use_parallel_mode=True)
    info_th = O.gen_candidates_scipy.last_info
    assert info_th["driver"] == "threads"
    if info_rc["driver"] == "reverse communication":
        assert np.array_equal(X_rc.numpy(), X_th.numpy())
        assert info_rc["nit_per_restart"] == info_th["nit_per_restart"] and info_rc["nfev"] == info_th["nfev"]


@pytest.mark.timeout(60)
def test_per_restart_thread_driver_raises_without_hanging(monkeypatch):
    import botorch_gb300.optim as O

    monkeypatch.setattr(O, "_lbfgsb_rc", lambda: None)
    with pytest.raises(RuntimeError, match="batched acquisition evaluation failed"):
        O.gen_candidates_scipy(torch.rand(5, 2, 2, dtype=torch.float64), _FakeAcqf(5, 2, 2, fail_at=4), 0.0, 1.0,
                               {"maxiter": 50}, use_parallel_mode=True)


def test_batched_lbfgsb_reproduces_the_reference_batched_driver():
    """botorch_gb300.optim.batched_lbfgsb against the reference's fmin_l_bfgs_b_batched
    (botorch/optim/batched_lbfgs_b.py:169) on the objective of
    tests/golden/make_lbfgsb_golden.py: the same per-row iterates (bit for bit with the
    scipy version the fixture was made with, to 1e-10 with another)."""
    from pathlib import Path

    import numpy as np
    import pytest
    import scipy

    from botorch_gb300.optim import _lbfgsb_rc, batched_lbfgsb
    from tests.golden.make_lbfgsb_golden import fg_batched, problem

    if _lbfgsb_rc() is None:
        pytest.skip("scipy's reverse-communication L-BFGS-B is not available")
    fx = np.load(Path(__file__).resolve().parent / "golden" / "lbfgsb_golden.npz")
    c, w, x0, lo, hi = problem()
    assert np.array_equal(x0, fx["x0"])
    res = batched_lbfgsb(lambda X, rows: fg_batched(X, rows, c, w), x0, lo, hi, {"maxiter": 40})
    xs = np.stack([r["x"] for r in res])
    nit = np.array([r["nit"] for r in res])
    # bit for bit where scipy's compiled routine is the fixture's (same version, x86-64);
    # another build of it rounds differently
    if str(fx["scipy_version"]) == scipy.__version__ and platform.machine() == "x86_64":
        assert np.array_equal(xs, fx["x"]) and np.array_equal(nit, fx["nit"])
    else:
        assert np.allclose(xs, fx["x"], rtol=0, atol=1e-10)
