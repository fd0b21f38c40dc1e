"""Write tests/golden/log_areas_golden.npz: inputs and outputs of the reference's
own fused qLogEHVI kernel (botorch/csrc/logei_fused.cpp, compiled from the
reference checkout by oracle/build.py into oracle/_ref/).

Cases (float64 and float32):
* the branch cases of the reference's test_fused_kernel_branch_coverage
  (test/acquisition/multi_objective/test_logei.py:349-415): one cell
  [0, 0] x [3, 3]; q=2 objectives placed in the three softplus regimes, and
  q=1 (fatmin over one element);
* log_fatplus underflow (tau * fatplus == 0 -> -1e30) and the fatmin
  shortcut below -1e29;
* unbounded cells (upper = inf, clamped);
* seeded random shapes: shared (nc, m) and batched (B, nc, m) cells, subset
  sizes across the GPU kernel's register buckets (1, 3, 4, 5, 8, 9, 16, 17,
  32) and m from 1 to 8.

Run from the repository root:  python tests/golden/make_log_areas_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.build import build_reference  # noqa: E402

TAU_RELU, TAU_MAX = 1e-6, 1e-2


def cases(dtype: torch.dtype):
    g = torch.Generator().manual_seed(20240611)
    big_neg = -1e155 if dtype == torch.float64 else -1e15  # tau * fatplus underflows to 0
    cell_lo = torch.tensor([[0.0, 0.0]], dtype=torch.float64)
    cell_up = torch.tensor([[3.0, 3.0]], dtype=torch.float64)
    yield "branch_q2", torch.tensor([[[[0.000005, 4.0], [-6.0, 0.00001]]]]), cell_lo, cell_up
    yield "branch_q1", torch.tensor([[[[5.0, 3.0]]]]), cell_lo, cell_up
    yield ("underflow", torch.tensor([[[[big_neg, 1.0], [0.5, 2.0]], [[1.5, 1.2], [0.5, 2.0]],
                                       [[big_neg, big_neg], [2.0, 2.5]]]]),
           torch.tensor([[0.0, 0.0], [1.0, -1.0]]), torch.tensor([[3.0, 3.0], [float("inf"), 4.0]]))
    for name, B, n_sub, isz, m, nc, batched in [
            ("r1", 7, 4, 1, 2, 5, False), ("r3", 5, 3, 3, 3, 6, True), ("r4", 4, 6, 4, 2, 9, False),
            ("r5", 3, 5, 5, 4, 4, True), ("r8", 3, 2, 8, 2, 33, False), ("r9", 2, 3, 9, 5, 3, True),
            ("r16", 2, 2, 16, 1, 7, False), ("r17", 2, 1, 17, 6, 4, True), ("r32", 2, 1, 32, 8, 3, False),
            ("r_many_cells", 3, 6, 2, 2, 70, False)]:
        obj = torch.randn(B, n_sub, isz, m, generator=g, dtype=torch.float64)
        # a third of the entries near the cell corners (|obj - lower| ~ tau_relu)
        near = torch.rand(obj.shape, generator=g) < 0.3
        obj = torch.where(near, obj * 1e-5, obj)
        lo = torch.randn(B if batched else 1, nc, m, generator=g, dtype=torch.float64) - 0.5
        up = lo + torch.rand(lo.shape, generator=g, dtype=torch.float64) * 2.0 + 1e-3
        up[..., 0, :] = float("inf")
        if not batched:
            lo, up = lo[0], up[0]
        yield name, obj, lo, up


def main(root: str) -> None:
    ref = build_reference(root)
    if ref is None:
        raise SystemExit("the reference checkout is not present: cannot generate the fixtures")
    out = {}
    for dtype, tag in ((torch.float64, "f64"), (torch.float32, "f32")):
        g = torch.Generator().manual_seed(7)
        for name, obj, lo, up in cases(dtype):
            obj, lo, up = obj.to(dtype), lo.to(dtype), up.to(dtype)
            val = ref.forward(obj, lo, up, TAU_RELU, TAU_MAX)
            go = torch.randn(val.shape, generator=g, dtype=torch.float64).to(dtype)
            grad = ref.backward(go, obj, lo, up, TAU_RELU, TAU_MAX)
            key = f"{tag}_{name}"
            for part, t in (("obj", obj), ("lower", lo), ("upper", up), ("value", val), ("grad_out", go),
                            ("grad", grad)):
                out[f"{key}__{part}"] = t.numpy()
    np.savez_compressed(Path(__file__).with_name("log_areas_golden.npz"), tau_relu=TAU_RELU,
                        tau_max=TAU_MAX, **out)
    print(f"wrote {len(out) // 6} cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_log_areas_golden.py <root of the reference checkout>")
    main(sys.argv[1])
