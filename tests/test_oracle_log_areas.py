"""Oracle of the fused qLogEHVI log-areas against the reference's own kernel
(golden fixtures from botorch/csrc/logei_fused.cpp, and the live kernel when the
reference checkout is present), against the reference's unfused Python path,
and the host-side argument checks of botorch_gb300.logei_fused (no GPU)."""

import math
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import log_areas as ola
from oracle.build import build_reference

GOLDEN = Path(__file__).parent / "golden" / "log_areas_golden.npz"


def golden_cases():
    z = np.load(GOLDEN)
    keys = sorted({k.split("__")[0] for k in z.files if "__" in k})
    for key in keys:
        yield key, {p: torch.from_numpy(z[f"{key}__{p}"]) for p in
                    ("obj", "lower", "upper", "value", "grad_out", "grad")}, float(z["tau_relu"]), float(z["tau_max"])


def _close(a, b, tol):
    return bool(((a - b).abs() <= tol * (1 + b.abs())).all()) and torch.equal(torch.isfinite(a), torch.isfinite(b))


def test_golden_fixture_has_all_cases():
    names = [k for k, *_ in golden_cases()]
    assert len(names) == 26
    for tag in ("f64", "f32"):
        for c in ("branch_q1", "branch_q2", "underflow", "r32", "r_many_cells"):
            assert f"{tag}_{c}" in names


@pytest.mark.parametrize("threads", [1, 3])
def test_oracle_matches_reference_golden(threads):
    for key, c, tr, tm in golden_cases():
        tol = 1e-14 if key.startswith("f64") else 1e-6
        v = ola.forward(c["obj"], c["lower"], c["upper"], tr, tm, threads=threads)
        g = ola.backward(c["grad_out"], c["obj"], c["lower"], c["upper"], tr, tm, threads=threads)
        assert _close(v, c["value"], tol), key
        assert _close(g, c["grad"], tol), key


def test_golden_branches_are_exercised():
    z = {k: c for k, c, *_ in golden_cases()}
    # tau * fatplus underflow -> -1e30 and the fatmin shortcut: exact -1e30 / -2e30 areas
    v = z["f64_underflow"]["value"]
    assert float(v[0, 0, 0]) == -1e30 and float(v[0, 0, 2]) == -2e30
    assert bool((z["f64_underflow"]["grad"][0, 2] == 0).all())
    # q = 1: fatmin over one element is the identity
    assert z["f64_branch_q1"]["obj"].shape[2] == 1


def test_oracle_matches_unfused_python_path():
    """The fused kernel equals steps 1-4 of the reference's unfused path
    (the reference's own test compares them at atol 1e-6, rtol 1e-6)."""
    for key, c, tr, tm in golden_cases():
        if not key.startswith("f64") or key.endswith("underflow"):
            continue  # the unfused path gives -inf where the fused one gives -1e30
        x = c["obj"].clone().requires_grad_(True)
        p = ola.python_path_log_areas(x, c["lower"], c["upper"], tr, tm)
        (p * c["grad_out"]).sum().backward()
        v = ola.forward(c["obj"], c["lower"], c["upper"], tr, tm)
        g = ola.backward(c["grad_out"], c["obj"], c["lower"], c["upper"], tr, tm)
        torch.testing.assert_close(v, p.detach(), atol=1e-6, rtol=1e-6, msg=key)
        torch.testing.assert_close(g, x.grad, atol=1e-6, rtol=1e-6, msg=key)


def test_oracle_matches_live_reference_kernel():
    ref = build_reference()
    if ref is None:
        pytest.skip("the reference kernel was not built here (no reference checkout)")
    g = torch.Generator().manual_seed(3)
    for dtype in (torch.float64, torch.float32):
        for B, n_sub, isz, m, nc, batched in [(4, 6, 2, 2, 5, False), (3, 4, 7, 3, 6, True), (2, 1, 32, 8, 2, False)]:
            obj = (torch.randn(B, n_sub, isz, m, generator=g, dtype=torch.float64) * 0.5).to(dtype)
            lo = torch.randn(B if batched else 1, nc, m, generator=g, dtype=torch.float64)
            up = (lo + 1.5).to(dtype)
            lo = lo.to(dtype)
            if not batched:
                lo, up = lo[0], up[0]
            go = torch.randn(B, nc, n_sub, generator=g, dtype=torch.float64).to(dtype)
            assert torch.equal(ola.forward(obj, lo, up, 1e-6, 1e-2), ref.forward(obj, lo, up, 1e-6, 1e-2))
            assert torch.equal(ola.backward(go, obj, lo, up, 1e-6, 1e-2, threads=2),
                               ref.backward(go, obj, lo, up, 1e-6, 1e-2))


def test_host_argument_checks_without_gpu():
    from botorch_gb300 import logei_fused as lf

    obj = torch.zeros(2, 3, 2, 2, dtype=torch.float64)
    cells = torch.zeros(4, 2, dtype=torch.float64)
    with pytest.raises(RuntimeError, match="obj_subsets must be 4-D"):
        lf.forward(obj[0], cells, cells, 1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="cell bounds must be 2-D or 3-D"):
        lf.forward(obj, cells[0], cells[0], 1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="subset_size or m too large"):
        lf.forward(torch.zeros(1, 1, 33, 2, dtype=torch.float64), cells, cells, 1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="subset_size or m too large"):
        lf.forward(torch.zeros(1, 1, 2, 9, dtype=torch.float64), torch.zeros(4, 9), torch.zeros(4, 9),
                   1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="CUDA tensors"):
        lf.forward(obj, cells, cells, 1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="CUDA tensors"):
        lf.backward(torch.zeros(2, 4, 3, dtype=torch.float64), obj, cells, cells, 1e-6, 1e-2)


def test_log_areas_workload_is_well_formed():
    """The benchmark workload: q-subsets of each size are the combinations of the q
    objective samples, cells are non-empty boxes above the front, the outer ones
    unbounded above."""
    import itertools

    from botorch_gb300.testing import log_areas_workload

    w = log_areas_workload(mc=2, restarts=3)
    assert w.B == 6 and w.nc == 64 and len(w.obj_subsets) == w.q == 4
    assert w.areas_per_step() == 6 * 64 * sum(math.comb(4, i) for i in range(1, 5))
    for i, o in enumerate(w.obj_subsets, start=1):
        combos = list(itertools.combinations(range(4), i))
        assert o.shape == (6, len(combos), i, 2)
        assert torch.equal(o[:, 0, 0], w.obj_subsets[0][:, combos[0][0], 0])  # first element of the first subset
    assert bool((w.cell_upper > w.cell_lower).all())
    assert bool(torch.isinf(w.cell_upper[:, 1]).all()) and bool(torch.isinf(w.cell_upper[-1, 0]))


def test_fused_log_areas_host_reshaping(monkeypatch):
    """FusedLogAreas's batch flattening, batched-cell reshape and gradient routing,
    with the C oracle standing in for the kernels (recompute route), against
    autograd through the reference's unfused steps."""
    from botorch_gb300 import logei_fused as lf

    monkeypatch.setattr(lf, "JACOBIAN_BUDGET_BYTES", 0)
    monkeypatch.setattr(lf, "forward", lambda o, cl, cu, tr, tm: ola.forward(o, cl, cu, tr, tm))
    monkeypatch.setattr(lf, "backward", lambda go, o, cl, cu, tr, tm: ola.backward(go, o, cl, cu, tr, tm))
    g = torch.Generator().manual_seed(8)
    obj = torch.randn(4, 3, 6, 2, 2, generator=g, dtype=torch.float64)   # (mc, batch, n_sub, i, m)
    lo = torch.randn(4, 3, 7, 2, generator=g, dtype=torch.float64) - 0.5  # batched cells
    up = lo + 1.0
    w = torch.randn(4, 3, 7, 6, generator=g, dtype=torch.float64)
    for cells in ((lo, up), (lo[0, 0], up[0, 0])):                       # batched and shared cells
        x = obj.clone().requires_grad_(True)
        out = lf.FusedLogAreas.apply(x, cells[0], cells[1], 1e-6, 1e-2)
        assert out.shape == (4, 3, 7, 6)
        (out * w).sum().backward()
        xr = obj.clone().requires_grad_(True)
        cl = cells[0].reshape(-1, 7, 2) if cells[0].dim() > 2 else cells[0]
        cu = cells[1].reshape(-1, 7, 2) if cells[1].dim() > 2 else cells[1]
        ref = ola.python_path_log_areas(xr.reshape(12, 6, 2, 2), cl, cu, 1e-6, 1e-2).reshape(4, 3, 7, 6)
        (ref * w).sum().backward()
        torch.testing.assert_close(out.detach(), ref.detach(), atol=1e-6, rtol=1e-6)
        torch.testing.assert_close(x.grad, xr.grad, atol=1e-6, rtol=1e-6)
