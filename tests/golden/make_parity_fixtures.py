"""Generate tests/golden/parity_fixtures.npz: float64 oracle outputs for the GPU parity tests.

The oracle (oracle/, the CPU float64 restatement of the reference path) is run
here, on the x86 host the golden vectors were pinned on, so the GPU tests do
not depend on the CPU arithmetic of the machine that hosts the GPU. Cases:

* qei_small:      qEI, d=6, n=64, b=512, q=4, 256 Sobol samples (seed 0):
                  value and gradient of all 512 t-batches;
* qlognei_diff:   qLogNEI, d=12, n=1024, q=4, 512 samples: the pruned baseline
                  (prune seed from torch.manual_seed(0)) and value + gradient of
                  the first 256 of the 2048 t-batches;
* qlognei_branin: qLogNEI, d=20, n=4096, q=8, 512 samples: pruned baseline and
                  value + gradient of every 64th of the 4096 t-batches.

A checksum of each candidate tensor is stored so that a test can verify that
the seeded generator reproduced the same inputs on the GPU host. For the qLogNEI
cases, ``*_sens_v`` / ``*_sens_g`` hold each t-batch's sensitivity to a 1e-6
shift of the standardised posterior mean (oracle/sensitivity.py), which bounds
the mixed path's error where float32 rounding of the mean is amplified.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from botorch_gb300 import testing as T  # noqa: E402
from oracle.acquisition import (QExpectedImprovement, QLogNoisyExpectedImprovement,  # noqa: E402
                                qei_value_and_grad)
from oracle.gp import ExactGP  # noqa: E402
from oracle.sensitivity import mean_sensitivity  # noqa: E402

OUT = Path(__file__).resolve().parent / "parity_fixtures.npz"


def model(w):
    return ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)


def checksum(t: torch.Tensor) -> np.ndarray:
    return np.array([float(t.sum()), float((t * t).sum()), float(t.reshape(-1)[::97].sum())])


def main() -> None:
    torch.set_num_threads(max(1, torch.get_num_threads()))
    out: dict[str, np.ndarray] = {}
    w = T.qei_small()
    v, g = qei_value_and_grad(QExpectedImprovement(model(w), w.best_f, w.n_samples, w.seed), w.X)
    out.update({"qei_small_value": v.numpy(), "qei_small_grad": g.numpy(), "qei_small_Xsum": checksum(w.X)})

    w = T.qlognei_diff()
    torch.manual_seed(0)
    a = QLogNoisyExpectedImprovement(model(w), w.train_X, w.n_samples, w.seed)
    idx = torch.arange(0, 256)
    v, g = a.value_and_grad(w.X[idx])
    sv, sg = mean_sensitivity(a, w.X[idx], v, g)
    out.update({"qlognei_diff_idx": idx.numpy(), "qlognei_diff_value": v.numpy(),
                "qlognei_diff_grad": g.numpy(), "qlognei_diff_Xb": a.X_baseline.numpy(),
                "qlognei_diff_Xsum": checksum(w.X), "qlognei_diff_sens_v": sv.numpy(),
                "qlognei_diff_sens_g": sg.numpy()})

    w = T.qlognei_branin(n=4096, b=4096, q=8, d=20)
    torch.manual_seed(0)
    a = QLogNoisyExpectedImprovement(model(w), w.train_X, w.n_samples, w.seed)
    idx = torch.arange(0, 4096, 64)
    v, g = a.value_and_grad(w.X[idx])
    sv, sg = mean_sensitivity(a, w.X[idx], v, g)
    out.update({"qlognei_branin_idx": idx.numpy(), "qlognei_branin_value": v.numpy(),
                "qlognei_branin_grad": g.numpy(), "qlognei_branin_Xb": a.X_baseline.numpy(),
                "qlognei_branin_Xsum": checksum(w.X), "qlognei_branin_sens_v": sv.numpy(),
                "qlognei_branin_sens_g": sg.numpy()})
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
