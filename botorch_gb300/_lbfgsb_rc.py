"""L-BFGS-B restarts stepped through scipy's reverse-communication routine.

``_RCRestart`` advances one restart exactly as scipy's own driver loop does;
the batched driver (``botorch_gb300.optim.batched_lbfgsb``) steps every
restart in one host loop, as the reference does
(botorch/optim/batched_lbfgs_b.py:169-636). This file imports only numpy and
scipy.
"""

from __future__ import annotations

import numpy as np

class _RCRestart:
    """One restart's L-BFGS-B state for scipy's reverse-communication routine
    ``setulb`` (scipy >= 1.15), advanced exactly as scipy's own driver loop
    advances it (scipy.optimize._lbfgsb_py._minimize_lbfgsb): task 3 asks for
    f and g at x, task 1 starts a new iteration, anything else stops."""

    def __init__(self, setulb, int_dtype, x0: np.ndarray, lo: np.ndarray, hi: np.ndarray, opts: dict):
        n = x0.size
        self.setulb = setulb
        self.m = int(opts.get("maxcor", 10))
        self.factr = float(opts.get("ftol", 2.2204460492503131e-09)) / np.finfo(float).eps
        self.pgtol = float(opts.get("gtol", 1e-5))
        self.maxls = int(opts.get("maxls", 20))
        self.maxiter = int(opts.get("maxiter", 15000))
        self.maxfun = int(opts.get("maxfun", 15000))
        self.nbd = np.zeros(n, dtype=int_dtype)
        self.low = np.zeros(n, dtype=np.float64)
        self.up = np.zeros(n, dtype=np.float64)
        for i in range(n):  # scipy's bound codes: 0 none, 1 lower, 2 both, 3 upper
            has_lo, has_up = not np.isinf(lo[i]), not np.isinf(hi[i])
            if has_lo:
                self.low[i] = lo[i]
            if has_up:
                self.up[i] = hi[i]
            self.nbd[i] = {(False, False): 0, (True, False): 1, (True, True): 2, (False, True): 3}[has_lo, has_up]
        self.x = np.clip(np.asarray(x0, dtype=np.float64), lo, hi)
        self.f = np.array(0.0, dtype=np.float64)
        self.g = np.zeros(n, dtype=np.float64)
        m = self.m
        self.wa = np.zeros(2 * m * n + 5 * n + 11 * m * m + 8 * m, np.float64)
        self.iwa = np.zeros(3 * n, dtype=int_dtype)
        self.task = np.zeros(2, dtype=int_dtype)
        self.ln_task = np.zeros(2, dtype=int_dtype)
        self.lsave = np.zeros(4, dtype=int_dtype)
        self.isave = np.zeros(44, dtype=int_dtype)
        self.dsave = np.zeros(29, dtype=np.float64)
        self.nit = 0
        self.nfev = 0

    def advance(self) -> bool:
        """Run the routine until it asks for f and g (True) or stops (False)."""
        while True:
            self.g = self.g.astype(np.float64)
            self.setulb(self.m, self.x, self.low, self.up, self.nbd, self.f, self.g, self.factr,
                        self.pgtol, self.wa, self.iwa, self.task, self.lsave, self.isave, self.dsave,
                        self.maxls, self.ln_task)
            if self.task[0] == 3:
                return True
            if self.task[0] == 1:
                self.nit += 1
                if self.nit >= self.maxiter:
                    self.task[0], self.task[1] = 5, 504
                elif self.nfev > self.maxfun:
                    self.task[0], self.task[1] = 5, 502
            else:
                return False

    def result(self) -> dict:
        from scipy.optimize import _lbfgsb_py

        msg = (_lbfgsb_py.status_messages[int(self.task[0])] + ": "
               + _lbfgsb_py.task_messages[int(self.task[1])])
        return {"x": self.x.copy(), "fun": float(self.f), "nit": self.nit, "nfev": self.nfev, "message": msg}


_RC: dict = {}


def lbfgsb_rc():
    """(setulb, int dtype) of scipy's reverse-communication L-BFGS-B when it is the
    interface this driver follows (scipy >= 1.15) and reproduces scipy's own
    ``minimize`` bit for bit on a small bounded problem; else None (the per-restart
    mode then runs one scipy optimiser per host thread)."""
    if "rc" in _RC:
        return _RC["rc"]
    rc = None
    try:
        import scipy
        from scipy.optimize import _lbfgsb, _lbfgsb_py, minimize

        major, minor = (int(v) for v in scipy.__version__.split(".")[:2])
        if (major, minor) >= (1, 15) and hasattr(_lbfgsb_py, "HAS_ILP64"):
            cand = (_lbfgsb.setulb, np.int64 if _lbfgsb_py.HAS_ILP64 else np.int32)
            w = np.array([3.0, 0.5, 7.0, 1.5])
            c = np.array([0.3, 1.2, -0.4, 0.8])

            def fg(x):
                r = x - c
                return float(np.sum(w * r * r + r ** 4)), 2 * w * r + 4 * r ** 3

            lo, hi = np.array([0.0, 0.0, -1.0, 0.0]), np.array([1.0, 1.0, 1.0, 0.5])
            x0 = np.array([0.9, 0.1, 0.5, 0.2])
            ref = minimize(fg, x0, method="L-BFGS-B", jac=True, bounds=list(zip(lo, hi)),
                           options={"maxiter": 30})
            st = _RCRestart(*cand, x0, lo, hi, {"maxiter": 30})
            while st.advance():
                st.f, st.g = fg(st.x)
                st.nfev += 1
            if np.array_equal(st.x, ref.x) and st.nit == ref.nit:
                rc = cand
    except Exception:
        rc = None
    _RC["rc"] = rc
    return rc
