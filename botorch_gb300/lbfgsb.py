"""Batched L-BFGS-B whose state stays on the device.

The per-restart optimiser of the reference's fast path: every restart runs its
own L-BFGS-B (botorch/generation/gen.py:226-247 drives
``fmin_l_bfgs_b_batched``, botorch/optim/batched_lbfgs_b.py:169-636, which
steps scipy's routine once per restart and round), with the objectives of all
restarts evaluated in one batched call per round. Here one CTA per restart
advances that restart's L-BFGS-B 3.0 state machine (``bgb_lbfgsb_step``) in
HBM between two evaluations, so a round is the evaluation, one step launch and
a four-integer summary read by the host; the points, gradients and
limited-memory pairs never leave the device.

``DeviceLbfgsb`` is the reverse-communication object (what scipy's routine is
for one restart, for all of them); ``minimize_batched`` runs it against a
batched objective on the device.
"""

from __future__ import annotations

import ctypes
from typing import Callable

import numpy as np
import torch
from torch import Tensor

from botorch_gb300 import _native as nat
from botorch_gb300.exceptions import UnsupportedError

EPS = float(np.finfo(float).eps)


class DeviceLbfgsb:
    """L-BFGS-B state of ``X.shape[0]`` independent restarts over ``X.shape[1]``
    variables, the box ``lower <= x <= upper`` shared (+-inf: unbounded).

    ``X`` (float64, CUDA, contiguous) is both the restarts' current points and
    the points to evaluate next: ``init`` projects it onto the box; every
    ``step(value, grad)`` consumes f = sign * value[r], g = sign * grad[r] for
    each restart waiting for them, and writes the next point into its row.
    The options mean what they mean for ``scipy.optimize.minimize(method=
    "L-BFGS-B")``: maxcor, ftol, gtol, maxls, maxiter, maxfun."""

    def __init__(self, X: Tensor, lower: Tensor, upper: Tensor, maxcor: int = 10, ftol: float = 2.2204460492503131e-09,
                 gtol: float = 1e-5, maxls: int = 20, maxiter: int = 15000, maxfun: int = 15000) -> None:
        if X.dtype != torch.float64 or X.device.type != "cuda" or X.dim() != 2 or not X.is_contiguous():
            raise ValueError("X must be a contiguous 2-d float64 CUDA tensor")
        R, n = X.shape
        self.X = X
        self.device = X.device
        self.opts = nat.BgbLbfgsbOpts(restarts=R, n=n, m=int(maxcor), maxls=int(maxls), maxiter=int(maxiter),
                                      maxfun=int(maxfun), factr=float(ftol) / EPS, pgtol=float(gtol))
        lib = nat.lib()
        self.ws_bytes = int(lib.bgb_lbfgsb_workspace_bytes(ctypes.byref(self.opts)))
        if self.ws_bytes == 0:
            raise UnsupportedError(f"device L-BFGS-B supports 1 <= n <= 8192 variables and maxcor <= 20 "
                                   f"(got n={n}, maxcor={maxcor})")
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        self.lower = torch.as_tensor(lower, dtype=torch.float64, device=self.device).expand(n).contiguous()
        self.upper = torch.as_tensor(upper, dtype=torch.float64, device=self.device).expand(n).contiguous()
        self.summary = torch.zeros(4, dtype=torch.int32, device=self.device)
        with torch.cuda.device(self.device):
            nat.check(lib.bgb_lbfgsb_init(ctypes.byref(self.opts), nat.ptr(X), nat.ptr(self.lower),
                                          nat.ptr(self.upper), nat.ptr(self.ws), self.ws_bytes,
                                          nat.stream_handle(self.device)), "bgb_lbfgsb_init")

    def step(self, value: Tensor, grad: Tensor, sign: float = 1.0, status: Tensor | None = None,
             ignore_status: bool = False) -> None:
        """Consume the objective at ``X`` and advance (one launch plus the summary's);
        capturable in a CUDA graph. ``status`` (int32 per row, 0 = good): unless
        ``ignore_status``, a nonzero entry anywhere holds every restart back (the
        summary's second count) so the caller can re-evaluate first."""
        if value.device != self.device or grad.device != self.device or (
                status is not None and status.device != self.device):
            raise ValueError("value, grad and status must be on the optimiser's device")
        with torch.cuda.device(self.device):
            nat.check(nat.lib().bgb_lbfgsb_step(ctypes.byref(self.opts), nat.ptr(self.X), nat.ptr(value),
                                                float(sign), nat.ptr(grad), nat.ptr(status),
                                                int(bool(ignore_status)), nat.ptr(self.ws), self.ws_bytes,
                                                nat.ptr(self.summary), nat.stream_handle(self.device)),
                      "bgb_lbfgsb_step")

    def results(self) -> dict:
        """Per restart: f at its row of X, iterations, evaluations, stop code and message."""
        R = self.X.shape[0]
        f = torch.empty(R, dtype=torch.float64, device=self.device)
        nit = torch.empty(R, dtype=torch.int64, device=self.device)
        nfev = torch.empty(R, dtype=torch.int64, device=self.device)
        code = torch.empty(R, dtype=torch.int32, device=self.device)
        with torch.cuda.device(self.device):
            nat.check(nat.lib().bgb_lbfgsb_results(ctypes.byref(self.opts), nat.ptr(self.ws), self.ws_bytes,
                                                   nat.ptr(f), nat.ptr(nit), nat.ptr(nfev), nat.ptr(code),
                                                   nat.stream_handle(self.device)), "bgb_lbfgsb_results")
        codes = code.cpu().tolist()
        return {"fun": f.cpu(), "nit": nit.cpu(), "nfev": nfev.cpu(), "code": codes,
                "message": [nat.BGB_LBFGSB_MESSAGES.get(c, str(c)) for c in codes]}


def minimize_batched(objective: Callable[[Tensor], tuple[Tensor, Tensor]], X0: Tensor, lower, upper,
                     options: dict | None = None, sign: float = 1.0) -> tuple[Tensor, dict]:
    """Minimise ``sign * objective`` for every row of ``X0`` (R x n) with its own
    L-BFGS-B; ``objective(X) -> (value (R,), grad (R, n))`` is evaluated on the
    device once per round for all rows. Returns the final points and the
    per-restart results (the reference's ``fmin_l_bfgs_b_batched`` contract,
    botorch/optim/batched_lbfgs_b.py:169)."""
    opts = dict(options or {})
    X = X0.detach().to(torch.float64).contiguous().clone()
    lb = DeviceLbfgsb(X, lower, upper, **opts)
    host = torch.zeros(4, dtype=torch.int32).pin_memory()
    rounds = 0
    while True:
        value, grad = objective(X)
        lb.step(value.contiguous(), grad.contiguous(), sign=sign)
        host.copy_(lb.summary, non_blocking=True)
        torch.cuda.current_stream(X.device).synchronize()
        rounds += 1
        if int(host[2]) > 0:
            raise RuntimeError("the objective or its gradient is not finite at a restart's point")
        if int(host[0]) == 0:
            break
    out = lb.results()
    out["rounds"] = rounds
    return X, out
