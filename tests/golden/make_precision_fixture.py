"""Generate tests/golden/precision_n8192.npz: the float64 oracle on the large-n
precision workload (SingleTaskGP d=20, n=8192, Branin-sum targets, ARD
lengthscales ~ U[0.2, 1.0]; qLogNEI with q=8, 512 Sobol samples, b=4096
t-batches).

The oracle (oracle/, the CPU float64 restatement of the reference path) runs
here, on the x86 host the other fixtures were pinned on, so the GPU tests
compare per output against it without depending on the CPU arithmetic of the
GPU host. Stored per t-batch, for all 4096 t-batches:

* value and gradient of qLogNEI (pruned baseline from torch.manual_seed(0));
* the model's posterior at the t-batch's 8 points: mean (8) and the lower
  triangle of the covariance (36 values, row-major);
* the sensitivity of value and gradient to a 1e-6 shift of the standardised
  posterior mean of the t-batch's points (oracle/sensitivity.py);

plus the pruned baseline and a checksum of the candidates, which the test uses
to check that the seeded generator reproduced the inputs. About ten minutes on
8 host cores.
"""

from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from botorch_gb300 import testing as T  # noqa: E402
from oracle.acquisition import QLogNoisyExpectedImprovement  # noqa: E402
from oracle.gp import ExactGP  # noqa: E402
from oracle.sensitivity import mean_sensitivity  # noqa: E402
from tests.golden.make_parity_fixtures import checksum  # noqa: E402

OUT = Path(__file__).resolve().parent / "precision_n8192.npz"
N, B, Q, D = 8192, 4096, 8, 20


def main() -> None:
    t0 = time.perf_counter()
    w = T.qlognei_branin(n=N, b=B, q=Q, d=D)
    om = ExactGP(w.train_X, w.train_Y, w.lengthscale, w.outputscale, w.noise, w.mean_constant, w.kernel)
    torch.manual_seed(0)
    a = QLogNoisyExpectedImprovement(om, w.train_X, w.n_samples, w.seed)
    print(f"init {time.perf_counter() - t0:.1f} s, r = {a.X_baseline.shape[0]}", flush=True)
    vals, grads, means, covs, svs, sgs = [], [], [], [], [], []
    tri = torch.tril_indices(Q, Q)
    for i in range(0, B, 256):
        v, g = a.value_and_grad(w.X[i:i + 256])
        sv, sg = mean_sensitivity(a, w.X[i:i + 256], v, g)
        with torch.no_grad():
            m, c = om.posterior(w.X[i:i + 256])
        vals.append(v)
        grads.append(g)
        svs.append(sv)
        sgs.append(sg)
        means.append(m)
        covs.append(c[:, tri[0], tri[1]])
        print(f"{i + 256} / {B} t-batches, {time.perf_counter() - t0:.1f} s", flush=True)
    np.savez_compressed(OUT, value=torch.cat(vals).numpy(), grad=torch.cat(grads).numpy(),
                        post_mean=torch.cat(means).numpy(), post_cov_tril=torch.cat(covs).numpy(),
                        sens_v=torch.cat(svs).numpy(), sens_g=torch.cat(sgs).numpy(),
                        Xb=a.X_baseline.numpy(), Xsum=checksum(w.X))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
