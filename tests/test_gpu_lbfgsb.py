"""The device L-BFGS-B (bgb_lbfgsb_*, one CTA per restart) against scipy's own
L-BFGS-B routine, the optimiser the reference's batched driver steps per
restart (botorch/optim/batched_lbfgs_b.py:169-636; botorch/generation/gen.py:226-247).

Lock-step: each side evaluates the same host objective at its own points every
round. The device sums its O(m n) dot products as CTA reductions, so the
points may differ from scipy's by rounding; the iteration and evaluation
counts and the stop reasons must be the same."""

import numpy as np
import pytest
import torch

from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement
from botorch_gb300 import testing as T
from botorch_gb300._lbfgsb_rc import _RCRestart, lbfgsb_rc
from botorch_gb300.lbfgsb import DeviceLbfgsb, minimize_batched
from botorch_gb300.optim import draw_sobol_samples, gen_candidates_scipy

from tests.test_gpu_parity import DEV, gpu_model
from tests.test_lbfgsb_emu import ref_code, rosen

pytestmark = pytest.mark.gpu


def device_lockstep(fg, x0, lo, hi, m=10, maxiter=200, maxls=20, ftol=2.220446049250313e-09, gtol=1e-5,
                    maxfun=15000):
    if lbfgsb_rc() is None:
        pytest.skip("scipy's reverse-communication L-BFGS-B (scipy >= 1.15) is not available")
    R, n = x0.shape
    X = torch.from_numpy(x0.copy()).to(DEV).contiguous()
    lb = DeviceLbfgsb(X, torch.from_numpy(lo), torch.from_numpy(hi), maxcor=m, ftol=ftol, gtol=gtol, maxls=maxls,
                      maxiter=maxiter, maxfun=maxfun)
    opts = dict(maxcor=m, maxiter=maxiter, maxls=maxls, ftol=ftol, gtol=gtol, maxfun=maxfun)
    sts = [_RCRestart(*lbfgsb_rc(), x0[i], lo, hi, opts) for i in range(R)]
    act = [s.advance() for s in sts]
    diffs = []
    while True:
        Xh = X.cpu().numpy()
        vals, grads = np.zeros(R), np.zeros((R, n))
        for i in range(R):
            vals[i], grads[i] = fg(Xh[i])
        lb.step(torch.from_numpy(vals).to(DEV), torch.from_numpy(grads).to(DEV))
        summary = lb.summary.cpu().tolist()
        for i in range(R):
            if act[i]:
                sts[i].f, sts[i].g = fg(sts[i].x)
                sts[i].nfev += 1
                act[i] = sts[i].advance()
        Xh = X.cpu().numpy()
        diffs.append(max(float(np.abs(Xh[i] - sts[i].x).max()) for i in range(R)))
        if summary[0] == 0 and not any(act):
            break
        assert len(diffs) < 3000
    res = lb.results()
    return dict(X=X.cpu().numpy(), res=res, ref=[s.result() for s in sts], diffs=diffs)


def assert_same_counts(out, x_tol):
    assert max(out["diffs"]) <= x_tol, max(out["diffs"])
    for i, ref in enumerate(out["ref"]):
        assert int(out["res"]["nit"][i]) == ref["nit"] and int(out["res"]["nfev"][i]) == ref["nfev"], (i, ref)
        assert out["res"]["code"][i] == ref_code(ref["message"]), (out["res"]["code"][i], ref["message"])
        if ref_code(ref["message"]) != 3:  # (scipy's driver reports the last trial's f after a failed search)
            assert abs(float(out["res"]["fun"][i]) - ref["fun"]) <= 1e-12 * max(1.0, abs(ref["fun"]))


def test_bounded_quadratic_matches_scipy(cuda_lib):
    rng = np.random.default_rng(0)
    n = 12
    A, c = rng.uniform(0.5, 4, n), rng.uniform(-0.5, 1.5, n)

    def fg(x):
        return float(np.sum(A * (x - c) ** 2) + 0.3 * np.sum(np.sin(3 * x))), 2 * A * (x - c) + 0.9 * np.cos(3 * x)

    assert_same_counts(device_lockstep(fg, rng.uniform(0, 1, (8, n)), np.zeros(n), np.ones(n)), 1e-12)


def test_bounded_rosenbrock_history_wrap_matches_scipy(cuda_lib):
    rng = np.random.default_rng(1)
    n = 20
    out = device_lockstep(rosen, rng.uniform(-1.5, 0.8, (6, n)), np.full(n, -1.5), np.full(n, 0.8), m=5,
                          maxiter=500)
    assert_same_counts(out, 1e-8)


def test_config_size_landscape_matches_scipy(cuda_lib):
    """64 restarts of n = 800 (q = 16 x d = 50) in [0, 1]: the shape of the
    optimisation configuration; several breakpoint walks per restart."""
    rng = np.random.default_rng(3)
    n = 800
    W = rng.normal(size=(64, n)) / np.sqrt(n)
    b = rng.uniform(0, 6, 64)

    def fg(x):
        u = W @ x * 4 + b
        return (-float(np.sum(np.cos(u))) / 8 + 0.5 * float(np.sum((x - 0.5) ** 2)),
                (W.T @ np.sin(u)) * 0.5 + (x - 0.5))

    out = device_lockstep(fg, rng.uniform(0, 1, (64, n)), np.zeros(n), np.ones(n), maxiter=100)
    # line-search trial points amplify the reduction-order rounding; the end points agree closely
    assert_same_counts(out, 1e-8)
    assert out["diffs"][-1] <= 1e-11


def test_mixed_bounds_and_line_search_failure(cuda_lib):
    rng = np.random.default_rng(2)
    n = 30
    lo = rng.uniform(-1, 0, n)
    hi = lo + rng.uniform(0.5, 2, n)
    lo[::5] = -np.inf
    hi[1::5] = np.inf
    hi[2::7] = lo[2::7]
    lo[4], hi[4] = -np.inf, np.inf
    A, c = rng.uniform(0.5, 4, n), rng.uniform(-2, 2, n)

    def fg(x):
        nb = np.r_[x[1:], 0] + np.r_[0, x[:-1]]
        f = np.sum(A * (x - c) ** 2) + 0.5 * np.sum(np.sin(2 * x) ** 2) + 0.1 * np.sum(x[:-1] * x[1:])
        return float(f), 2 * A * (x - c) + 2 * np.sin(2 * x) * np.cos(2 * x) + 0.1 * nb

    assert_same_counts(device_lockstep(fg, rng.uniform(-3, 3, (5, n)), lo, hi, m=4), 1e-8)

    def wrong(x):
        return float(np.sum((x - 0.3) ** 2)), -0.5 * (x - 0.3) + 0.01

    out = device_lockstep(wrong, rng.uniform(0, 1, (3, 8)), np.zeros(8), np.ones(8))
    assert_same_counts(out, 1e-13)
    assert set(out["res"]["code"]) == {3}


def test_status_holds_the_round_and_non_finite_stops(cuda_lib):
    R, n = 3, 4
    X = torch.full((R, n), 0.5, dtype=torch.float64, device=DEV)
    lb = DeviceLbfgsb(X, torch.zeros(n), torch.ones(n), maxcor=5)
    vals = torch.tensor([1.0, float("nan"), 2.0], dtype=torch.float64, device=DEV)
    grads = torch.ones(R, n, dtype=torch.float64, device=DEV)
    status = torch.tensor([0, 2, 0], dtype=torch.int32, device=DEV)
    X0 = X.clone()
    lb.step(vals, grads, status=status)
    assert lb.summary.cpu().tolist() == [3, 3, 0, 0]
    assert torch.equal(X, X0)
    lb.step(vals, grads, status=status, ignore_status=True)
    assert lb.summary.cpu().tolist() == [2, 0, 1, 1]
    assert torch.equal(X[1], X0[1])
    assert lb.results()["code"] == [0, 6, 0]


def test_minimize_batched_on_a_device_objective(cuda_lib):
    """A torch objective evaluated on the device every round; each row ends at
    scipy's minimum of the same function. (The device's sin and the host's
    round differently, so the two runs are not in lock-step: the end values
    and points agree to the accuracy the stopping rules allow, ftol = 2.2e-9
    relative reduction of f.)"""
    from scipy.optimize import minimize

    g = torch.Generator().manual_seed(7)
    R, n = 16, 40
    A = (0.5 + 3 * torch.rand(n, generator=g, dtype=torch.float64)).to(DEV)
    c = (-0.5 + 2 * torch.rand(n, generator=g, dtype=torch.float64)).to(DEV)

    def objective(X):
        v = (A * (X - c) ** 2).sum(-1) + 0.2 * torch.sin(4 * X).sum(-1)
        return v, 2 * A * (X - c) + 0.8 * torch.cos(4 * X)

    X0 = torch.rand(R, n, generator=g, dtype=torch.float64).to(DEV)
    X, res = minimize_batched(objective, X0, 0.0, 1.0, {"maxiter": 200})
    Ah, ch = A.cpu().numpy(), c.cpu().numpy()
    for i in range(R):
        ref = minimize(lambda x: (float(np.sum(Ah * (x - ch) ** 2) + 0.2 * np.sum(np.sin(4 * x))),
                                  2 * Ah * (x - ch) + 0.8 * np.cos(4 * x)),
                       X0[i].cpu().numpy(), jac=True, method="L-BFGS-B", bounds=[(0.0, 1.0)] * n,
                       options={"maxiter": 200})
        assert abs(float(res["fun"][i]) - ref.fun) <= 1e-8 * max(1.0, abs(ref.fun))
        assert np.abs(X[i].cpu().numpy() - ref.x).max() <= 1e-4


def test_gen_candidates_device_and_scipy_drivers_agree(cuda_lib):
    """The acquisition optimisation in the per-restart mode: the device driver
    (the default on CUDA) and scipy's routine stepped on the host give the same
    candidates on the float64 acquisition path."""
    w = T.qlognei_diff(b=1, q=2, n=128)
    gm = gpu_model(w)
    torch.manual_seed(0)
    acqf = qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(torch.Size([256]), seed=0),
                                        precision="fp64")
    d = w.train_X.shape[-1]
    X0 = draw_sobol_samples(torch.stack([torch.zeros(d), torch.ones(d)]).double(), 6, 2, seed=1).to(DEV)
    Xd, vd = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": 40})
    info_d = gen_candidates_scipy.last_info
    assert info_d["driver"] == "device"
    Xs, vs = gen_candidates_scipy(X0, acqf, 0.0, 1.0, {"maxiter": 40}, lbfgsb="scipy")
    info_s = gen_candidates_scipy.last_info
    assert info_s["driver"] == "reverse communication"
    assert info_d["nit_per_restart"] == info_s["nit_per_restart"]
    assert float((Xd - Xs).abs().max()) <= 1e-8
    assert float(((vd - vs).abs() / vs.abs().clamp_min(1.0)).max()) <= 1e-10
    # the mixed path, eager and graph-replayed rounds give the same optimisation
    acqm = qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(torch.Size([256]), seed=0),
                                        precision="mixed")
    Xg, vg = gen_candidates_scipy(X0, acqm, 0.0, 1.0, {"maxiter": 40})
    Xe, ve = gen_candidates_scipy(X0, acqm, 0.0, 1.0, {"maxiter": 40}, use_graph=False)
    assert torch.equal(Xg, Xe) and torch.equal(vg, ve)


def test_device_driver_groups_agree(cuda_lib):
    """Restarts cut into stream groups (one group's step overlapping the other's
    evaluation) reach the same candidates as one group: the restarts are
    independent, the grouping changes only the rounding of batched sums."""
    from botorch_gb300.optim import _per_restart_device

    w = T.qlognei_diff(b=1, q=2, n=128)
    gm = gpu_model(w)
    torch.manual_seed(0)
    acqf = qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(torch.Size([256]), seed=0),
                                        precision="fp64")
    d = w.train_X.shape[-1]
    X0 = draw_sobol_samples(torch.stack([torch.zeros(d), torch.ones(d)]).double().to(DEV), 20, 2, seed=3)
    lo, hi = np.zeros(d), np.ones(d)
    X1, r1, _ = _per_restart_device(acqf, X0, lo, hi, 30, {}, True, groups=1)
    X2, r2, _ = _per_restart_device(acqf, X0, lo, hi, 30, {}, True, groups=2)
    assert [int(v) for v in r1["nit"]] == [int(v) for v in r2["nit"]]
    assert float((X1 - X2).abs().max()) <= 1e-8
    assert float((r1["fun"] - r2["fun"]).abs().max()) <= 1e-10


class _FlakyObjective:
    """A stand-in acquisition function (a smooth bowl) whose batched call
    reports a failed t-batch in chosen rounds; its checked call (the fallback
    route) returns the same, correct values."""

    def __init__(self, bad_calls):
        self.device = DEV
        self.bad_calls = set(bad_calls)
        self.calls = 0
        self.checked = 0

    def value_and_grad_raw(self, Xd, need_grad, check=None, out=None, ws=None):
        w = torch.arange(1, Xd.shape[-1] + 1, dtype=torch.float64, device=Xd.device) ** 2
        v = -(w * (Xd - 0.3) ** 2 + 0.05 * torch.sin(7 * Xd)).sum((-1, -2))
        g = -(2.0 * w * (Xd - 0.3) + 0.35 * torch.cos(7 * Xd))
        if out is None:
            if need_grad:
                self.checked += 1
            return v, (g if need_grad else None)
        value, grad, status = out
        value.copy_(v)
        grad.copy_(g)
        status.zero_()
        if self.calls in self.bad_calls:
            status[0] = 1  # the batched call failed for one t-batch
            value[0] = float("nan")
        self.calls += 1
        return value, grad


def test_device_driver_reevaluates_held_rounds(cuda_lib):
    """A round whose batched evaluation reports a failed t-batch is held back,
    evaluated again through the checked call, and then consumed: the optimisation
    ends where the one without failures ends."""
    from botorch_gb300.optim import _per_restart_device

    g = torch.Generator().manual_seed(2)
    X0 = torch.rand(5, 2, 3, generator=g, dtype=torch.float64).to(DEV)
    lo, hi = np.zeros(3), np.ones(3)
    clean = _FlakyObjective([])
    Xc, rc, nc = _per_restart_device(clean, X0, lo, hi, 50, {}, False)
    assert nc >= 4
    flaky = _FlakyObjective([0, 1, 3])
    Xf, rf, nf = _per_restart_device(flaky, X0, lo, hi, 50, {}, False)
    assert flaky.checked == 3  # each held round evaluated once more through the checked call
    assert nf == nc and torch.equal(Xf, Xc)
    assert [int(v) for v in rf["nit"]] == [int(v) for v in rc["nit"]]
