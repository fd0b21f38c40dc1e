"""The device L-BFGS-B's state machine (botorch_gb300/csrc/lbfgsb_core.cuh),
built for the host with one thread per restart, stepped in lock-step with
scipy's own L-BFGS-B routine (the optimiser the reference's batched driver
steps per restart, botorch/optim/batched_lbfgs_b.py:169-636) on the CPU.

Each side evaluates the same objective at its own points, so any difference
in the algorithm shows as a difference in the points. The host build sums in
the same order as a serial loop; the device build differs only in its
reduction order (tests/test_gpu_lbfgsb.py)."""

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from botorch_gb300._lbfgsb_rc import _RCRestart, lbfgsb_rc

ROOT = Path(__file__).resolve().parents[1]
EPS = float(np.finfo(float).eps)


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    if lbfgsb_rc() is None:
        pytest.skip("scipy's reverse-communication L-BFGS-B (scipy >= 1.15) is not available")
    so = tmp_path_factory.mktemp("lbemu") / "lbemu.so"
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "botorch_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "lbfgsb_emu.cpp"), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    vp, ll, i32, f64 = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_double
    lib.emu_workspace_bytes.restype = ll
    lib.emu_workspace_bytes.argtypes = [ll, ll, i32]
    lib.emu_init.argtypes = [ll, i32, i32, vp, vp, vp, vp]
    lib.emu_step.argtypes = [ll, i32, i32, i32, ll, ll, f64, f64, vp, vp, f64, vp, vp, i32, vp, vp]
    lib.emu_results.argtypes = [ll, i32, i32, vp, vp, vp, vp, vp]
    return lib


def P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lockstep(lib, fg, x0, lo, hi, m=10, maxiter=200, maxls=20, ftol=2.220446049250313e-09, gtol=1e-5,
             maxfun=15000):
    """Run both optimisers to the end; returns per-round max point differences and
    both sides' results."""
    R, n = x0.shape
    ws = np.zeros(lib.emu_workspace_bytes(R, n, m), np.uint8)
    X = np.ascontiguousarray(x0.copy())
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    lib.emu_init(R, n, m, P(X), P(lo), P(hi), P(ws))
    opts = dict(maxcor=m, maxiter=maxiter, maxls=maxls, ftol=ftol, gtol=gtol, maxfun=maxfun)
    sts = [_RCRestart(*lbfgsb_rc(), x0[i], lo, hi, opts) for i in range(R)]
    act = [s.advance() for s in sts]
    summary = np.zeros(4, np.int32)
    diffs = []
    rounds = 0
    while True:
        vals, grads = np.zeros(R), np.zeros((R, n))
        for i in range(R):
            vals[i], grads[i] = fg(X[i])
        lib.emu_step(R, n, m, maxls, maxiter, maxfun, ftol / EPS, gtol, P(X), P(vals), 1.0, P(grads), None, 1,
                     P(ws), P(summary))
        for i in range(R):
            if act[i]:
                sts[i].f, sts[i].g = fg(sts[i].x)
                sts[i].nfev += 1
                act[i] = sts[i].advance()
        rounds += 1
        diffs.append(max(float(np.abs(X[i] - sts[i].x).max()) for i in range(R)))
        if summary[0] == 0 and not any(act):
            break
        assert rounds < 5000
    f = np.zeros(R)
    nit = np.zeros(R, np.int64)
    nfev = np.zeros(R, np.int64)
    code = np.zeros(R, np.int32)
    lib.emu_results(R, n, m, P(ws), P(f), P(nit), P(nfev), P(code))
    return dict(X=X, f=f, nit=nit, nfev=nfev, code=code, ref=[s.result() for s in sts], diffs=diffs)


def ref_code(msg: str) -> int:
    """scipy's stop message as a BGB_LBFGSB_* code."""
    for key, code in (("PROJECTED GRADIENT", 1), ("REDUCTION OF F", 2), ("ABNORMAL", 3),
                      ("ITERATIONS REACHED", 4), ("EVALUATIONS EXCEEDS", 5)):
        if key in msg.upper():
            return code
    return -1


def assert_same_run(out, x_tol=1e-12):
    R = len(out["ref"])
    assert max(out["diffs"]) <= x_tol, out["diffs"]
    for i in range(R):
        ref = out["ref"][i]
        assert out["nit"][i] == ref["nit"] and out["nfev"][i] == ref["nfev"], (i, out["nit"][i], ref)
        if ref_code(ref["message"]) != 3:
            # (after a failed line search scipy's driver reports the last trial's f
            # beside the restored x; the device keeps f at x)
            assert abs(out["f"][i] - ref["fun"]) <= 1e-13 * max(1.0, abs(ref["fun"]))
        assert out["code"][i] == ref_code(ref["message"]), (out["code"][i], ref["message"])


def rosen(x):
    f = np.sum(100 * (x[1:] - x[:-1] ** 2) ** 2 + (1 - x[:-1]) ** 2)
    g = np.zeros_like(x)
    g[:-1] = -400 * x[:-1] * (x[1:] - x[:-1] ** 2) - 2 * (1 - x[:-1])
    g[1:] += 200 * (x[1:] - x[:-1] ** 2)
    return float(f), g


def test_bounded_quadratic_with_active_bounds(emu):
    rng = np.random.default_rng(0)
    n = 12
    A, c = rng.uniform(0.5, 4, n), rng.uniform(-0.5, 1.5, n)

    def fg(x):
        return float(np.sum(A * (x - c) ** 2) + 0.3 * np.sum(np.sin(3 * x))), 2 * A * (x - c) + 0.9 * np.cos(3 * x)

    assert_same_run(lockstep(emu, fg, rng.uniform(0, 1, (4, n)), np.zeros(n), np.ones(n)))


def test_bounded_rosenbrock_wraps_the_history(emu):
    """m = 5 over ~40 iterations: the circular S, Y columns and the shifted S^T S,
    S^T Y are exercised many times."""
    rng = np.random.default_rng(1)
    n = 20
    out = lockstep(emu, rosen, rng.uniform(-1.5, 0.8, (6, n)), np.full(n, -1.5), np.full(n, 0.8), m=5, maxiter=500)
    assert max(out["nit"]) > 15
    assert_same_run(out, x_tol=1e-9)


def test_mixed_bounds_fixed_variables_and_starts_outside_the_box(emu):
    rng = np.random.default_rng(2)
    n = 30
    lo = rng.uniform(-1, 0, n)
    hi = lo + rng.uniform(0.5, 2, n)
    lo[::5] = -np.inf  # upper bound only
    hi[1::5] = np.inf  # lower bound only
    hi[2::7] = lo[2::7]  # fixed
    lo[4], hi[4] = -np.inf, np.inf  # unbounded
    A, c = rng.uniform(0.5, 4, n), rng.uniform(-2, 2, n)

    def fg(x):
        nb = np.r_[x[1:], 0] + np.r_[0, x[:-1]]
        f = np.sum(A * (x - c) ** 2) + 0.5 * np.sum(np.sin(2 * x) ** 2) + 0.1 * np.sum(x[:-1] * x[1:])
        return float(f), 2 * A * (x - c) + 2 * np.sin(2 * x) * np.cos(2 * x) + 0.1 * nb

    # trial points of long line-search steps amplify rounding to ~1e-10; the
    # accepted iterates and the end points agree to ~1e-14
    out = lockstep(emu, fg, rng.uniform(-3, 3, (5, n)), lo, hi, m=4)
    assert_same_run(out, x_tol=1e-9)
    assert out["diffs"][-1] <= 1e-12


def test_acquisition_like_landscape_at_config_size(emu):
    """n = 800 (q = 16 x d = 50), the restarts of the optimisation configuration."""
    rng = np.random.default_rng(3)
    n = 800
    W = rng.normal(size=(64, n)) / np.sqrt(n)
    b = rng.uniform(0, 6, 64)

    def fg(x):
        u = W @ x * 4 + b
        return (-float(np.sum(np.cos(u))) / 8 + 0.5 * float(np.sum((x - 0.5) ** 2)),
                (W.T @ np.sin(u)) * 0.5 + (x - 0.5))

    assert_same_run(lockstep(emu, fg, rng.uniform(0, 1, (3, n)), np.zeros(n), np.ones(n), maxiter=100),
                    x_tol=1e-11)


def test_unbounded_problem_reaches_the_same_minimum(emu):
    """Without bounds the Cauchy step is skipped after the first iteration. On
    Rosenbrock's valley the two runs separate by rounding after ~40 rounds, so
    the check is on the minimum: the early rounds agree to 1e-12."""
    rng = np.random.default_rng(4)
    n = 20
    out = lockstep(emu, rosen, rng.uniform(-1, 1, (3, n)), np.full(n, -np.inf), np.full(n, np.inf), m=7,
                   maxiter=500)
    assert max(out["diffs"][:15]) <= 1e-12
    for i in range(3):
        assert abs(out["f"][i] - out["ref"][i]["fun"]) <= 1e-8
        assert np.abs(out["X"][i] - out["ref"][i]["x"]).max() <= 1e-4


@pytest.mark.parametrize("limit", ["maxiter", "maxfun"])
def test_iteration_and_evaluation_limits(emu, limit):
    rng = np.random.default_rng(5)
    n = 20
    kw = {"maxiter": 7} if limit == "maxiter" else {"maxfun": 9}
    out = lockstep(emu, rosen, rng.uniform(-1, 0.8, (3, n)), np.full(n, -1.5), np.full(n, 0.8), **kw)
    assert_same_run(out, x_tol=1e-13)
    assert set(out["code"].tolist()) == {4 if limit == "maxiter" else 5}


def test_wrong_gradient_ends_in_the_same_line_search_failure(emu):
    """A gradient that does not match f makes the line search fail; with no
    history left both give up with the previous point."""
    rng = np.random.default_rng(6)
    n = 8

    def fg(x):
        return float(np.sum((x - 0.3) ** 2)), -0.5 * (x - 0.3) + 0.01

    out = lockstep(emu, fg, rng.uniform(0, 1, (3, n)), np.zeros(n), np.ones(n))
    assert_same_run(out, x_tol=1e-13)
    assert set(out["code"].tolist()) == {3}


def test_non_finite_values_stop_the_restart_and_status_holds_the_round(emu):
    n, R, m = 4, 3, 5
    lo, hi = np.zeros(n), np.ones(n)
    X = np.full((R, n), 0.5)
    ws = np.zeros(emu.emu_workspace_bytes(R, n, m), np.uint8)
    emu.emu_init(R, n, m, P(X), P(lo), P(hi), P(ws))
    summary = np.zeros(4, np.int32)
    vals = np.array([1.0, np.nan, 2.0])
    grads = np.ones((R, n))
    status = np.array([0, 2, 0], np.int32)
    X0 = X.copy()
    # a bad status anywhere holds every restart back: nothing consumed, nothing moved
    emu.emu_step(R, n, m, 20, 100, 100, 1e7, 1e-5, P(X), P(vals), 1.0, P(grads), P(status), 0, P(ws), P(summary))
    assert summary.tolist() == [3, 3, 0, 0]
    assert np.array_equal(X, X0)
    emu.emu_step(R, n, m, 20, 100, 100, 1e7, 1e-5, P(X), P(vals), 1.0, P(grads), P(status), 1, P(ws), P(summary))
    assert summary.tolist() == [2, 0, 1, 1]
    assert np.array_equal(X[1], X0[1])  # the stopped restart keeps its point
    code = np.zeros(R, np.int32)
    emu.emu_results(R, n, m, P(ws), P(np.zeros(R)), P(np.zeros(R, np.int64)), P(np.zeros(R, np.int64)), P(code))
    assert code.tolist() == [0, 6, 0]


@pytest.mark.parametrize("case", ["scalar", "history_one", "history_twenty", "one_trial", "all_fixed",
                                  "start_on_bounds", "zero_gradient"])
def test_edge_cases_match_scipy(emu, case):
    """Edge cases of the sizes, the options and the starting points."""
    rng = np.random.default_rng(7)
    opts = {}
    if case == "scalar":
        n = 1
        lo, hi = np.array([-2.0]), np.array([3.0])

        def fg(x):
            return float((x[0] - 1.3) ** 4 + np.cos(3 * x[0])), np.array([4 * (x[0] - 1.3) ** 3 - 3 * np.sin(3 * x[0])])

        x0 = rng.uniform(-2, 3, (4, n))
    else:
        n = 24
        lo, hi = np.zeros(n), np.ones(n)
        A, c = rng.uniform(0.5, 4, n), rng.uniform(-0.5, 1.5, n)

        def fg(x):
            return (float(np.sum(A * (x - c) ** 2) + 0.2 * np.sum(np.sin(5 * x))),
                    2 * A * (x - c) + np.cos(5 * x))

        x0 = rng.uniform(0, 1, (4, n))
        if case == "history_one":
            opts["m"] = 1
        elif case == "history_twenty":
            opts["m"] = 20
        elif case == "one_trial":
            opts["maxls"] = 1
        elif case == "all_fixed":
            hi = lo.copy()
        elif case == "start_on_bounds":
            x0 = np.where(rng.uniform(size=x0.shape) < 0.5, 0.0, 1.0)
        elif case == "zero_gradient":
            def fg(x):  # noqa: F811 - flat objective
                return 1.5, np.zeros_like(x)
    out = lockstep(emu, fg, x0, lo, hi, **opts)
    assert_same_run(out, x_tol=1e-10)


@pytest.mark.parametrize("seed", range(10))
def test_random_sizes_histories_and_bound_kinds_match_scipy(emu, seed):
    """Seeded sweep over the sizes, the history length and the kind of each
    variable's bounds (both, lower only, upper only, none, fixed), with starts
    inside and outside the box, on strongly convex objectives (one minimum, so
    the runs cannot part at a saddle): every combination of free, active and
    entering/leaving variables the subspace matrix's updates meet."""
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 80))
    m = int(rng.integers(1, 13))
    lo = rng.uniform(-1, 0.5, n)
    hi = lo + rng.uniform(0.2, 2, n)
    kind = rng.choice(5, size=n, p=[0.5, 0.15, 0.15, 0.1, 0.1])
    lo[kind == 2] = -np.inf  # upper bound only
    hi[kind == 1] = np.inf  # lower bound only
    lo[kind == 3], hi[kind == 3] = -np.inf, np.inf  # unbounded
    hi[kind == 4] = lo[kind == 4]  # fixed
    A, c = rng.uniform(0.5, 4, n), rng.uniform(-2, 2, n)

    def fg(x):
        # second derivative >= 2 A - 0.9 - 0.2 > 0
        nb = np.r_[x[1:], 0] + np.r_[0, x[:-1]]
        f = np.sum(A * (x - c) ** 2) + 0.1 * np.sum(np.sin(3 * x)) + 0.1 * np.sum(x[:-1] * x[1:])
        return float(f), 2 * A * (x - c) + 0.3 * np.cos(3 * x) + 0.1 * nb

    # (half or more of the variables end on a bound; the runs agree to ~1e-14,
    # 2.6e-12 at worst over these seeds)
    out = lockstep(emu, fg, rng.uniform(-2.5, 2.5, (4, n)), lo, hi, m=m)
    assert_same_run(out, x_tol=1e-10)
    assert out["diffs"][-1] <= 1e-12
