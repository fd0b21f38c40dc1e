"""Acquisition optimisation around the CUDA acquisition path.

The caller side of the path: raw-sample initialisation and multi-start
L-BFGS-B on the acquisition value and its gradient, with the reference's
argument meanings.

* ``draw_sobol_samples``: scrambled Sobol q-batches in a box
  (botorch/utils/sampling.py:74-111).
* ``initialize_q_batch``: Boltzmann selection of restart points from the raw
  samples, keeping the best raw sample (botorch/optim/initializers.py:959-1042,
  botorch/utils/sampling.py:1084-1115).
* ``gen_candidates_scipy``: L-BFGS-B on the restarts, in either of the
  reference's two modes. By default (``use_parallel_mode`` None or True, the
  reference's fast path, botorch/generation/gen.py:226-247 with
  botorch/optim/batched_lbfgs_b.py) every restart runs its own L-BFGS-B on
  minus its own value, the objectives of all restarts evaluated in one call
  per round. For an acquisition function on a CUDA device the restarts'
  L-BFGS-B states live on the device (``botorch_gb300.lbfgsb``): a round is
  the evaluation, one step launch and a four-integer summary read by the
  host, captured in one CUDA graph. ``lbfgsb="scipy"`` instead steps scipy's
  reverse-communication routine for every restart on the calling thread, as
  the reference does (scipy >= 1.15, checked bit for bit against scipy's own
  ``minimize`` in a self-test; else one scipy optimiser per restart in its own
  host thread); each evaluation then copies the points to the device and the
  values and gradients back through pinned buffers (the f / grad wrapper of
  gen.py:423-487). With ``use_parallel_mode=False`` the restarts are
  aggregated into one problem whose objective is minus the sum of the values
  (the reference's aggregated mode, gen.py:249-395).
* ``optimize_acqf``: raw samples -> restarts -> L-BFGS-B -> the best restart
  (botorch/optim/optimize.py:619, ``return_best_only=True``).
"""

from __future__ import annotations

import numpy as np
import torch
from torch import Tensor

from botorch_gb300 import _native as nat
from botorch_gb300._lbfgsb_rc import _RCRestart  # noqa: F401
from botorch_gb300._lbfgsb_rc import lbfgsb_rc as _lbfgsb_rc


def draw_sobol_samples(bounds: Tensor, n: int, q: int, seed: int | None = None) -> Tensor:
    """``n x q x d`` scrambled-Sobol points in the box ``bounds`` (2 x d), on
    ``bounds``' device (botorch/utils/sampling.py:74-111).

    The engine is torch's ``SobolEngine(q * d, scramble=True, seed)``. For
    float64 bounds on a CUDA device its state is built on the host and the
    points are generated and mapped to the box on the device (``bgb_sobol_box``),
    bit for bit what the engine's draw and the elementwise map give on the host."""
    d = bounds.shape[-1]
    engine = torch.quasirandom.SobolEngine(q * d, scramble=True, seed=seed)
    lo, hi = bounds[0], bounds[1]
    if bounds.device.type == "cuda" and bounds.dtype == torch.float64 and n > 0:
        dev = bounds.device
        state = engine.sobolstate.to(dev).contiguous()
        shift = engine.shift.to(dev).contiguous()
        first_point = engine._first_point.to(torch.float64).reshape(-1).to(dev).contiguous()
        lo_d, hi_d = lo.contiguous(), hi.contiguous()
        out = torch.empty(n, q, d, dtype=torch.float64, device=dev)
        with torch.cuda.device(dev):
            nat.check(nat.lib().bgb_sobol_box(nat.ptr(state), nat.ptr(shift), nat.ptr(first_point), q * d,
                                              engine.MAXBIT, 0, n, nat.ptr(lo_d), nat.ptr(hi_d), d, nat.ptr(out),
                                              nat.stream_handle(dev)), "bgb_sobol_box")
        return out
    raw = engine.draw(n, dtype=bounds.dtype).view(n, q, d).to(bounds.device)
    return lo + (hi - lo) * raw


def _standardize(y: Tensor) -> Tensor:
    s = y.std()
    s = s if s >= 1e-9 else torch.ones_like(s)
    return (y - y.mean()) / s


def initialize_q_batch(X: Tensor, acq_vals: Tensor, n: int, eta: float = 1.0,
                       generator: torch.Generator | None = None) -> tuple[Tensor, Tensor]:
    """Pick ``n`` of the ``b`` raw q-batches ``X`` (b x q x d) without replacement with
    probability proportional to exp(eta * standardised value), always keeping the
    best one. Equal or non-finite values: a random choice."""
    b = X.shape[0]
    if n > b:
        raise RuntimeError(f"n ({n}) cannot be larger than the number of provided samples ({b})")
    if n == b:
        return X, acq_vals
    ystd = acq_vals.std()
    if ystd == 0 or not torch.isfinite(ystd):
        idx = torch.randperm(b, device=X.device, generator=generator)[:n]
        return X[idx], acq_vals[idx]
    z = _standardize(acq_vals)
    weights = torch.exp(eta * z)
    while torch.isinf(weights).any():
        eta *= 0.5
        weights = torch.exp(eta * z)
    idx = torch.multinomial(weights, n, replacement=False, generator=generator)
    best = torch.argmax(acq_vals)
    if not bool((idx == best).any()):
        idx[-1] = best
    return X[idx], acq_vals[idx]


def evaluate_raw(acqf, X: Tensor, batch_limit: int = 4096) -> Tensor:
    """Acquisition values (no gradient) of ``b x q x d`` raw q-batches, ``batch_limit``
    q-batches per call."""
    out = []
    Xd = X.to(acqf.device, torch.float64)
    for i in range(0, X.shape[0], batch_limit):
        v, _ = acqf.value_and_grad_raw(Xd[i:i + batch_limit].contiguous(), False)
        out.append(v.clone())
    return torch.cat(out)


class _Objective:
    """f(x) = -sum_i acq(X_i) and its gradient for L-BFGS-B, x the flattened restarts.

    The restarts are evaluated in one call per objective evaluation; x and the
    gradient cross the host boundary through pinned buffers."""

    def __init__(self, acqf, shape: tuple[int, int, int], use_graph: bool = True) -> None:
        self.acqf = acqf
        self.shape = shape
        self.use_graph = use_graph
        self.host_x = torch.empty(shape, dtype=torch.float64).pin_memory()
        self.host_v = torch.empty(shape[0], dtype=torch.float64).pin_memory()
        self.host_g = torch.empty(shape, dtype=torch.float64).pin_memory()
        self.dev_x = torch.empty(shape, dtype=torch.float64, device=acqf.device)
        self.calls = 0

    def __call__(self, x: np.ndarray) -> tuple[float, np.ndarray]:
        if np.isnan(x).any():
            raise RuntimeError(f"{int(np.isnan(x).sum())} elements of x are NaN")
        self.host_x.numpy().reshape(-1)[:] = x
        self.dev_x.copy_(self.host_x, non_blocking=True)
        if self.use_graph:
            v, g = self.acqf.graphed_value_and_grad(self.dev_x, True)
        else:
            v, g = self.acqf.value_and_grad_raw(self.dev_x, True)
        self.host_v.copy_(v, non_blocking=True)
        self.host_g.copy_(g, non_blocking=True)
        torch.cuda.current_stream(self.acqf.device).synchronize()
        self.calls += 1
        gn = self.host_g.numpy().reshape(-1)
        if np.isnan(gn).any():
            raise RuntimeError(f"{int(np.isnan(gn).sum())} elements of the gradient are NaN")
        return -float(self.host_v.numpy().sum()), -gn.astype(np.float64, copy=True)


class _RestartRounds:
    """Batched objective for restarts that each run their own L-BFGS-B.

    Every restart's optimiser runs in its own host thread and hands its point
    to ``evaluate``. The threads pass a baton, so that exactly one of them, or
    the serving thread, runs at a time (no contention for the interpreter
    lock): a restart that has handed in its point wakes the next restart
    waiting for the last round's result (or starts the next thread that has
    not begun); the last one wakes the serving thread (``serve``), which
    evaluates all b points in one call (a CUDA graph replay at fixed shape,
    through pinned buffers; only this thread touches the GPU) and wakes the
    first restart. Rows of restarts that have finished keep their last point
    and their values are ignored. The value of a t-batch does not depend on
    the other rows, so each restart's path is that of its own run alone.
    (The reference reaches the same per-restart semantics by stepping scipy's
    internal L-BFGS-B routine for every restart in one loop,
    botorch/optim/batched_lbfgs_b.py:169-636.)"""

    def __init__(self, acqf, shape: tuple[int, int, int], use_graph: bool = True) -> None:
        import collections
        import threading

        self.acqf = acqf
        self.use_graph = use_graph
        self.cuda = torch.device(acqf.device).type == "cuda"
        b = shape[0]

        def host(*sz):
            t = torch.empty(sz, dtype=torch.float64)
            return t.pin_memory() if self.cuda else t

        self.host_x, self.host_v, self.host_g = host(*shape), host(b), host(*shape)
        self.dev_x = torch.empty(shape, dtype=torch.float64, device=acqf.device)
        self.sems = [threading.Semaphore(0) for _ in range(b)]
        self.server = threading.Semaphore(0)
        self.unstarted: collections.deque = collections.deque()
        self.queue: collections.deque = collections.deque()
        self.active = b
        self.pending: list[int] = []
        self.calls = 0
        self.error: BaseException | None = None
        self.fv = np.zeros(b)
        self.fg = np.zeros((b, shape[1] * shape[2]))

    def _next(self) -> None:
        """Hand the baton on: a thread not yet started, else the next restart
        waiting for its result, else the serving thread."""
        if self.unstarted:
            self.unstarted.popleft().start()
        elif self.queue:
            self.sems[self.queue.popleft()].release()
        else:
            self.server.release()

    def _run(self) -> None:
        """One batched evaluation (serving thread)."""
        try:
            self.dev_x.copy_(self.host_x, non_blocking=True)
            if self.use_graph and self.cuda:
                v, g = self.acqf.graphed_value_and_grad(self.dev_x, True)
            else:
                v, g = self.acqf.value_and_grad_raw(self.dev_x, True)
            self.host_v.copy_(v, non_blocking=True)
            self.host_g.copy_(g, non_blocking=True)
            if self.cuda:
                torch.cuda.current_stream(self.dev_x.device).synchronize()
            self.fv = -self.host_v.numpy().copy()
            self.fg = -self.host_g.numpy().reshape(self.fv.shape[0], -1).copy()
            self.calls += 1
        except BaseException as e:  # handed to every waiting restart
            self.error = e

    def serve(self, threads) -> None:
        """Run the restart threads and evaluate rounds until all have finished."""
        self.unstarted.extend(threads)
        self._next()
        while True:
            self.server.acquire()
            if self.active == 0:
                return
            # every running restart has handed in its point
            self.queue.extend(self.pending)
            self.pending = []
            self._run()
            self._next()

    def evaluate(self, i: int, x: np.ndarray) -> tuple[float, np.ndarray]:
        """Restart i's objective (its own thread, holding the baton)."""
        if np.isnan(x).any():
            raise RuntimeError(f"{int(np.isnan(x).sum())} elements of x are NaN")
        if self.error is not None:
            raise RuntimeError("batched acquisition evaluation failed") from self.error
        self.host_x.numpy()[i].reshape(-1)[:] = x
        self.pending.append(i)
        self._next()
        self.sems[i].acquire()
        if self.error is not None:
            raise RuntimeError("batched acquisition evaluation failed") from self.error
        f, g = float(self.fv[i]), self.fg[i].copy()
        if np.isnan(g).any():
            raise RuntimeError(f"{int(np.isnan(g).sum())} elements of the gradient are NaN")
        return f, g

    def done(self, i: int) -> None:
        """Restart i has finished (holding the baton): the rounds no longer wait for it."""
        self.active -= 1
        self._next()


def batched_lbfgsb(fg_batched, x0: np.ndarray, lo: np.ndarray, hi: np.ndarray, options: dict,
                   rc=None) -> list[dict]:
    """Independent L-BFGS-B runs, one per row of x0 (b x n), through scipy's
    reverse-communication routine: every round, the rows that ask for f and g are
    evaluated in one call ``fg_batched(X_rows, rows) -> (f, g)`` (X_rows k x n).
    The semantics of the reference's batched driver ``fmin_l_bfgs_b_batched``
    (botorch/optim/batched_lbfgs_b.py:169-636); per row, the same iterates as
    scipy's ``minimize(method="L-BFGS-B")``. Needs the routine (``_lbfgsb_rc()``)."""
    rc = rc if rc is not None else _lbfgsb_rc()
    if rc is None:
        raise RuntimeError("scipy's reverse-communication L-BFGS-B (scipy >= 1.15) is not available")
    b = x0.shape[0]
    states = [_RCRestart(*rc, x0[i], lo, hi, options) for i in range(b)]
    active = [i for i in range(b) if states[i].advance()]
    while active:
        for i in active:
            if np.isnan(states[i].x).any():
                raise RuntimeError(f"{int(np.isnan(states[i].x).sum())} elements of x are NaN")
        f, g = fg_batched(np.stack([states[i].x for i in active]), active)
        for k, i in enumerate(active):
            gi = np.array(g[k], dtype=np.float64)
            if np.isnan(gi).any():
                raise RuntimeError(f"{int(np.isnan(gi).sum())} elements of the gradient are NaN")
            states[i].f, states[i].g = float(f[k]), gi
            states[i].nfev += 1
        active = [i for i in active if states[i].advance()]
    return [s.result() for s in states]


def _per_restart_rc(acqf, x0: np.ndarray, lo: np.ndarray, hi: np.ndarray, shape, maxiter: int,
                    options: dict, use_graph: bool, rc):
    """Each restart's own L-BFGS-B (``batched_lbfgsb``), all restarts that need f and g
    evaluated in one acquisition call per round, on this thread. Returns per-restart
    results and the rounds."""
    b, q, d = shape
    rounds = _RestartRounds(acqf, shape, use_graph)

    def fg(X_rows: np.ndarray, rows: list[int]):
        for k, i in enumerate(rows):
            rounds.host_x.numpy()[i].reshape(-1)[:] = X_rows[k]
        rounds._run()
        if rounds.error is not None:
            raise RuntimeError("batched acquisition evaluation failed") from rounds.error
        return rounds.fv[rows], rounds.fg[rows]

    results = batched_lbfgsb(fg, x0, np.tile(lo, q), np.tile(hi, q), {**options, "maxiter": maxiter}, rc)
    return results, rounds.calls


_DEVICE_LBFGSB_OPTIONS = ("maxcor", "ftol", "gtol", "maxls", "maxfun")


def _per_restart_device(acqf, X0: Tensor, lo: np.ndarray, hi: np.ndarray, maxiter: int, options: dict,
                        use_graph: bool, groups: int | None = None):
    """Each restart's own L-BFGS-B with its state on the device (``DeviceLbfgsb``):
    a round is one batched evaluation of the restarts, one step launch and a
    four-integer summary read by the host (the round captured in one CUDA graph).
    ``groups`` > 1 cuts the restarts into groups whose rounds run on their own
    streams, so that one group's L-BFGS-B step (one CTA per restart) can overlap
    another's evaluation; restarts are independent, so each one's path does not
    depend on the grouping beyond rounding. (At 64 restarts of q = 16 two
    groups gave 0.887 ms per round against 0.873 ms for one: the default is
    one.) A group whose evaluation reports a failed t-batch is evaluated again
    through the acquisition function's checked call (its fallback route, or its
    error) before its restarts consume it. Returns the points, the per-restart
    results and the rounds."""
    from botorch_gb300.lbfgsb import DeviceLbfgsb

    b, q, d = X0.shape
    dev = X0.device
    X = X0.reshape(b, q * d).to(torch.float64).contiguous().clone()
    ng = groups if groups is not None else 1
    ng = max(1, min(ng, b))
    bounds_lo, bounds_hi = torch.from_numpy(np.tile(lo, q)), torch.from_numpy(np.tile(hi, q))
    lb_opts = {k: options[k] for k in _DEVICE_LBFGSB_OPTIONS if k in options}
    cut = [b * g // ng for g in range(ng + 1)]
    G = []
    for g in range(ng):
        Xg = X[cut[g]:cut[g + 1]]
        bg = cut[g + 1] - cut[g]
        G.append(dict(Xv=Xg.view(bg, q, d), lb=DeviceLbfgsb(Xg, bounds_lo, bounds_hi, maxiter=maxiter, **lb_opts),
                      value=torch.empty(bg, dtype=torch.float64, device=dev),
                      grad=torch.empty(bg, q, d, dtype=torch.float64, device=dev),
                      status=torch.zeros(bg, dtype=torch.int32, device=dev), ws=nat.Workspace(dev),
                      host=torch.zeros(4, dtype=torch.int32).pin_memory(),
                      stream=torch.cuda.Stream(dev) if ng > 1 else torch.cuda.current_stream(dev),
                      graph=None, active=True))

    def round_body(gr):
        acqf.value_and_grad_raw(gr["Xv"], True, check=False, out=(gr["value"], gr["grad"], gr["status"]),
                                ws=gr["ws"])
        gr["lb"].step(gr["value"], gr["grad"], sign=-1.0, status=gr["status"])
        gr["host"].copy_(gr["lb"].summary, non_blocking=True)

    main = torch.cuda.current_stream(dev)
    for gr in G:
        gr["stream"].wait_stream(main)
    if use_graph:
        for gr in G:
            # set up the acquisition's state for this shape, then capture one round
            side = torch.cuda.Stream(dev)
            side.wait_stream(main)
            with torch.cuda.stream(side):
                acqf.value_and_grad_raw(gr["Xv"], True, check=False, out=(gr["value"], gr["grad"], gr["status"]),
                                        ws=gr["ws"])
            main.wait_stream(side)
            torch.cuda.synchronize(dev)
            gr["graph"] = torch.cuda.CUDAGraph()
            with torch.cuda.graph(gr["graph"]):
                round_body(gr)
    rounds = 0
    while any(gr["active"] for gr in G):
        live = [gr for gr in G if gr["active"]]
        for gr in live:
            with torch.cuda.stream(gr["stream"]):
                if gr["graph"] is not None:
                    gr["graph"].replay()
                else:
                    round_body(gr)
        for gr in live:
            gr["stream"].synchronize()
        rounds += 1
        for gr in live:
            host = gr["host"]
            act, held, nonfin = int(host[0]), int(host[1]), int(host[2])
            if held:
                with torch.cuda.stream(gr["stream"]):
                    v, g = acqf.value_and_grad_raw(gr["Xv"], True)
                    gr["lb"].step(v.contiguous(), g.contiguous(), sign=-1.0, ignore_status=True)
                    host.copy_(gr["lb"].summary, non_blocking=True)
                gr["stream"].synchronize()
                act, nonfin = int(host[0]), int(host[2])
            if nonfin:
                raise RuntimeError("the acquisition value or its gradient is not finite "
                                   "(NaN elements of the gradient)")
            gr["active"] = act > 0
    for gr in G:
        main.wait_stream(gr["stream"])
    res = [gr["lb"].results() for gr in G]
    merged = {"fun": torch.cat([r["fun"] for r in res]), "nit": torch.cat([r["nit"] for r in res]),
              "nfev": torch.cat([r["nfev"] for r in res]), "code": sum((r["code"] for r in res), []),
              "message": sum((r["message"] for r in res), [])}
    return X.view(b, q, d), merged, rounds


def _per_restart_lbfgsb(acqf, x0: np.ndarray, lo: np.ndarray, hi: np.ndarray, shape, maxiter: int,
                        options: dict, use_graph: bool):
    """Each restart's own L-BFGS-B (scipy, one host thread each), objectives batched
    per round on the calling thread. Returns the scipy results and the rounds."""
    import threading

    from scipy.optimize import minimize

    b, q, d = shape
    rounds = _RestartRounds(acqf, shape, use_graph)
    bounds = list(zip(np.tile(lo, q), np.tile(hi, q)))
    results: list = [None] * b
    errors: list = [None] * b

    def run(i: int) -> None:
        try:
            results[i] = minimize(lambda x: rounds.evaluate(i, x), x0[i], method="L-BFGS-B", jac=True,
                                  bounds=bounds, options={"maxiter": maxiter, **options})
        except BaseException as e:
            errors[i] = e
        finally:
            rounds.done(i)

    threads = [threading.Thread(target=run, args=(i,), daemon=True) for i in range(b)]
    rounds.serve(threads)
    for t in threads:
        t.join()
    for e in errors:
        if e is not None:
            raise e
    return results, rounds.calls


def gen_candidates_scipy(initial_conditions: Tensor, acquisition_function, lower_bounds: float | Tensor,
                         upper_bounds: float | Tensor, options: dict | None = None,
                         use_graph: bool = True,
                         use_parallel_mode: bool | None = None,
                         lbfgsb: str | None = None) -> tuple[Tensor, Tensor]:
    """L-BFGS-B from the ``b x q x d`` initial conditions on the box; returns the
    candidates and their acquisition values.

    ``use_parallel_mode`` None (the default) or True: the reference's fast path
    (botorch/generation/gen.py:226-247, taken unless use_parallel_mode is False):
    every restart runs its own L-BFGS-B on minus its own value, with one batched
    evaluation per round. False: one L-BFGS-B on minus the sum of all restarts'
    values (the reference's aggregated mode, gen.py:249-395).

    ``lbfgsb`` (per-restart mode): "device" (the default for an acquisition
    function on a CUDA device) keeps every restart's L-BFGS-B state on the
    device (``botorch_gb300.lbfgsb``; the same algorithm as scipy's routine,
    iterates equal to rounding); "scipy" steps scipy's own routine per restart
    on the host (``batched_lbfgsb``; scipy's iterates bit for bit)."""
    from scipy.optimize import minimize

    options = dict(options or {})
    maxiter = int(options.pop("maxiter", 2000))
    X0 = initial_conditions.detach().to(torch.float64)
    b, q, d = X0.shape
    lo = torch.as_tensor(lower_bounds, dtype=torch.float64).expand(d).cpu().numpy()
    hi = torch.as_tensor(upper_bounds, dtype=torch.float64).expand(d).cpu().numpy()
    x0 = np.clip(X0.cpu().numpy(), lo, hi).reshape(-1)
    if use_parallel_mode is not False:
        v0, _ = acquisition_function.value_and_grad_raw(
            torch.from_numpy(x0.reshape(b, q, d)).to(acquisition_function.device), False)
        f0 = -float(v0.sum())
        on_cuda = torch.device(acquisition_function.device).type == "cuda"
        which = lbfgsb or ("device" if on_cuda else "scipy")
        if which not in ("device", "scipy"):
            raise ValueError(f"lbfgsb must be 'device' or 'scipy', got {lbfgsb!r}")
        if which == "device":
            X, res, calls = _per_restart_device(
                acquisition_function, torch.from_numpy(x0.reshape(b, q, d)).to(acquisition_function.device),
                lo, hi, maxiter, options, use_graph)
            v, _ = acquisition_function.value_and_grad_raw(X.contiguous(), False)
            nits = [int(t) for t in res["nit"]]
            info = {"mode": "per-restart", "driver": "device", "nit": max(nits), "nfev": int(calls),
                    "nit_per_restart": nits, "message": str(res["message"][0]),
                    "messages": list(res["message"]), "f0": f0, "f": -float(v.sum())}
            gen_candidates_scipy.last_info = info
            return X, v.clone()
        rc = _lbfgsb_rc()
        if rc is not None:
            results, calls = _per_restart_rc(acquisition_function, x0.reshape(b, -1), lo, hi, (b, q, d),
                                             maxiter, options, use_graph, rc)
        else:
            results, calls = _per_restart_lbfgsb(acquisition_function, x0.reshape(b, -1), lo, hi,
                                                 (b, q, d), maxiter, options, use_graph)
        xs = np.stack([r["x"] for r in results]).reshape(b, q, d)
        X = torch.from_numpy(np.clip(xs, lo, hi)).to(acquisition_function.device)
        v, _ = acquisition_function.value_and_grad_raw(X.contiguous(), False)
        info = {"mode": "per-restart", "driver": "reverse communication" if rc is not None else "threads",
                "nit": max(int(r["nit"]) for r in results), "nfev": int(calls),
                "nit_per_restart": [int(r["nit"]) for r in results],
                "message": str(results[0]["message"]), "f0": f0, "f": -float(v.sum())}
        gen_candidates_scipy.last_info = info
        return X, v.clone()
    bounds = list(zip(np.tile(lo, b * q), np.tile(hi, b * q)))
    obj = _Objective(acquisition_function, (b, q, d), use_graph)
    f0 = obj(x0)[0]
    res = minimize(obj, x0, method="L-BFGS-B", jac=True, bounds=bounds,
                   options={"maxiter": maxiter, **options})
    X = torch.from_numpy(np.clip(res.x.reshape(b, q, d), lo, hi)).to(acquisition_function.device)
    v, _ = acquisition_function.value_and_grad_raw(X.contiguous(), False)
    info = {"mode": "aggregated", "nit": int(res.nit), "nfev": int(obj.calls), "message": str(res.message),
            "f0": f0, "f": float(res.fun)}
    gen_candidates_scipy.last_info = info
    return X, v.clone()


def optimize_acqf(acq_function, bounds: Tensor, q: int, num_restarts: int, raw_samples: int,
                  options: dict | None = None, seed: int | None = None,
                  use_graph: bool = True, use_parallel_mode: bool | None = None,
                  lbfgsb: str | None = None) -> tuple[Tensor, Tensor]:
    """Raw samples -> Boltzmann-selected restarts -> L-BFGS-B -> the best restart.

    options: ``batch_limit`` (raw-sample evaluation chunk, 4096), ``eta`` (1.0),
    ``maxiter`` (2000) and further L-BFGS-B options."""
    options = dict(options or {})
    batch_limit = int(options.pop("batch_limit", 4096))
    eta = float(options.pop("eta", 1.0))
    bounds = bounds.to(torch.float64)
    X_raw = draw_sobol_samples(bounds.to(acq_function.device), raw_samples, q, seed=seed)
    v_raw = evaluate_raw(acq_function, X_raw, batch_limit)
    g = None if seed is None else torch.Generator(device=v_raw.device).manual_seed(seed)
    X0, _ = initialize_q_batch(X_raw.to(v_raw.device), v_raw, num_restarts, eta=eta, generator=g)
    X, v = gen_candidates_scipy(X0, acq_function, bounds[0], bounds[1], options, use_graph,
                                use_parallel_mode, lbfgsb)
    best = int(torch.argmax(v))
    return X[best], v[best]
