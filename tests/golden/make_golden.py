"""Generate tests/golden/reference_golden.npz from the reference's own modules.

Run in a container that has the BoTorch sources; argument 1 is the root of
that checkout (required). gpytorch and
linear_operator are not importable there, so ``botorch/__init__.py`` cannot
run; the modules below only need torch, numpy and scipy, and are loaded by
registering bare package stubs whose ``__path__`` points at the reference
tree (no reference source is copied).

Fixtures:
* safe_math: cauchy, fatplus, log_fatplus (tau 1e-6 and 1), _pareto (alpha 2),
  fatmax (tau 1e-2, with -inf/+inf rows), logmeanexp (with -inf rows),
  logsumexp;
* the qLogNEI per-sample utility log_fatplus(Y - best_f) composed as in
  botorch/acquisition/logei.py:688-715;
* Sobol normal base samples: draw_sobol_normal_samples(d, n, seed) for
  several (d, n, seed), bit-exact targets.
"""

from __future__ import annotations

import importlib
import sys
import types
from pathlib import Path

import numpy as np
import torch

OUT = Path(__file__).resolve().parent / "reference_golden.npz"


def load_reference(ref_root: str):
    for name, sub in (("botorch", "botorch"), ("botorch.utils", "botorch/utils"),
                      ("botorch.sampling", "botorch/sampling")):
        mod = types.ModuleType(name)
        mod.__path__ = [f"{ref_root}/{sub}"]
        sys.modules[name] = mod
    sm = importlib.import_module("botorch.utils.safe_math")
    us = importlib.import_module("botorch.utils.sampling")
    return sm, us


def main(ref_root: str) -> None:
    sm, us = load_reference(ref_root)
    g = torch.Generator().manual_seed(1234)
    f64 = torch.float64
    out: dict[str, np.ndarray] = {}
    # smooth nonlinearities over a wide range, including the far tails
    x = torch.cat([torch.linspace(-50, 50, 2001, dtype=f64), torch.tensor([-1e3, -1e2, 1e2, 1e3], dtype=f64),
                   torch.logspace(-9, 3, 200, dtype=f64), -torch.logspace(-9, 3, 200, dtype=f64)])
    out["x"] = x.numpy()
    out["cauchy"] = sm.cauchy(x).numpy()
    out["fatplus_tau1"] = sm.fatplus(x, tau=1.0).numpy()
    out["log_fatplus_tau1"] = sm.log_fatplus(x, tau=1.0).numpy()
    xs = x * 1e-5
    out["x_small"] = xs.numpy()
    out["log_fatplus_tau1e-6"] = sm.log_fatplus(xs, tau=1e-6).numpy()
    xp = torch.linspace(0, 100, 1001, dtype=f64)
    out["x_pareto"] = xp.numpy()
    out["pareto2"] = sm._pareto(xp, alpha=2.0).numpy()
    # fatmax over q with inf rows
    F = torch.randn(64, 8, generator=g, dtype=f64) * 3
    F[5] = -torch.inf
    F[6, 3] = torch.inf
    F[7, :2] = -torch.inf
    out["fatmax_in"] = F.numpy()
    out["fatmax_tau1e-2"] = sm.fatmax(F, dim=-1, tau=1e-2).numpy()
    out["fatmax_tau1"] = sm.fatmax(F, dim=-1, tau=1.0).numpy()
    Lm = torch.randn(512, 6, generator=g, dtype=f64) * 10
    Lm[:, 3] = -torch.inf
    out["lme_in"] = Lm.numpy()
    out["logmeanexp"] = sm.logmeanexp(Lm, dim=0).numpy()
    out["logsumexp"] = sm.logsumexp(Lm, dim=0).numpy()
    # qLogNEI per-sample utility and reductions on synthetic samples
    Y = 100 + 3 * torch.randn(256, 8, 4, generator=g, dtype=f64)
    best_f = 102 + torch.randn(256, generator=g, dtype=f64)
    li = sm.log_fatplus(Y - best_f.unsqueeze(-1).unsqueeze(-1), tau=1e-6)
    out["qlognei_Y"] = Y.numpy()
    out["qlognei_best_f"] = best_f.numpy()
    out["qlognei_li"] = li.numpy()
    out["qlognei_value"] = sm.logmeanexp(sm.fatmax(li, dim=-1, tau=1e-2), dim=0).numpy()
    # Sobol normal base samples (bit-exact)
    for d, n, seed in ((4, 256, 0), (6, 256, 0), (10, 512, 0), (12, 512, 0), (2, 16, 12345), (22, 64, 7)):
        out[f"sobol_normal_d{d}_n{n}_s{seed}"] = us.draw_sobol_normal_samples(d, n, dtype=f64, seed=seed).numpy()
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_golden.py <root of the reference checkout>")
    main(sys.argv[1])
