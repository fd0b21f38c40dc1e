"""Generate tests/golden/lbfgsb_golden.npz: iterates of the reference's batched L-BFGS-B.

Runs ``fmin_l_bfgs_b_batched`` (botorch/optim/batched_lbfgs_b.py:169) of the
reference checkout given as argument 1 on a deterministic batched objective and
stores, per row, the start, the final point, value and iteration count. The module is loaded from the reference tree
under bare package stubs (``botorch``, ``botorch.optim``), because
``botorch/__init__.py`` needs gpytorch, which is absent here; its one package
import, ``check_scipy_version_at_least`` (botorch/optim/utils/common.py:65-78),
is supplied by a stub module with the same one-line comparison. No reference
source is copied.

Objective, row i of x (b = 6 rows, n = 8): f(x) = sum_j w_j (x_j - c_ij)^2
+ (x_j - c_ij)^4 + 0.3 sin(3 x_j) x_{j+1}, box [-1, 1.5], with c, w seeded.
"""

from __future__ import annotations

import importlib.util
import sys
import types
from pathlib import Path

import numpy as np
import scipy

OUT = Path(__file__).resolve().parent / "lbfgsb_golden.npz"
B, N = 6, 8


def problem():
    rng = np.random.default_rng(3)
    c = rng.uniform(-1.2, 1.6, size=(B, N))
    w = rng.uniform(0.5, 3.0, size=N)
    x0 = rng.uniform(-1.0, 1.5, size=(B, N))
    return c, w, x0, np.full(N, -1.0), np.full(N, 1.5)


def fg_batched(X: np.ndarray, rows, c, w):
    """(f, g) of the rows of X (k x n) for objective rows ``rows``."""
    C = c[rows]
    r = X - C
    s = np.sin(3 * X[:, :-1]) * X[:, 1:]
    f = (w * r * r + r ** 4).sum(1) + 0.3 * s.sum(1)
    g = 2 * w * r + 4 * r ** 3
    g[:, :-1] += 0.3 * 3 * np.cos(3 * X[:, :-1]) * X[:, 1:]
    g[:, 1:] += 0.3 * np.sin(3 * X[:, :-1])
    return f, g


def load_reference(root: Path):
    for name, path in (("botorch", root / "botorch"), ("botorch.optim", root / "botorch" / "optim")):
        mod = types.ModuleType(name)
        mod.__path__ = [str(path)]
        sys.modules[name] = mod
    utils = types.ModuleType("botorch.optim.utils")
    utils.check_scipy_version_at_least = (
        lambda minor, major=1: tuple(map(int, scipy.__version__.split(".")[:2])) >= (major, minor))
    sys.modules["botorch.optim.utils"] = utils
    spec = importlib.util.spec_from_file_location(
        "botorch.optim.batched_lbfgs_b", root / "botorch" / "optim" / "batched_lbfgs_b.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def main(root: str) -> None:
    ref = load_reference(Path(root))
    c, w, x0, lo, hi = problem()

    def func(X, batch_indices):
        return fg_batched(X, batch_indices, c, w)

    xs, fs, results = ref.fmin_l_bfgs_b_batched(func, x0, bounds=list(zip(lo, hi)), maxiter=40,
                                                pass_batch_indices=True)
    out = {"x0": x0, "x": xs, "f": fs, "nit": np.array([r["nit"] for r in results]),
           "scipy_version": np.array(scipy.__version__)}
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: nit {out['nit'].tolist()}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_lbfgsb_golden.py <root of the reference checkout>")
    main(sys.argv[1])
