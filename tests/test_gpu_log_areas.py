"""Fused qLogEHVI log-areas on the GPU (bgb_log_areas_forward / _backward)
against the reference kernel's golden outputs and the C oracle.

Tolerances: float64 |gpu - ref| <= 1e-12 (1 + |ref|) (CUDA's and the host
libm's exp / log / log1p differ in the last bits). float32 results are held
to the float64 oracle on the same inputs: the GPU's float32 error
max |gpu - exact| / (1 + |exact|) must be within 4x the reference's own
float32 error, or below 2e-5. (The gradient weights of the smooth minimum
amplify last-bit differences of the log improvements by |li| / tau_max, so
two correct float32 implementations can differ by ~1e-4 there.) The -1e30
underflow values match exactly."""

import pytest
import torch

from botorch_gb300 import logei_fused as lf
from oracle import log_areas as ola

from tests.test_oracle_log_areas import golden_cases

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
TOL = {torch.float64: 1e-12, torch.float32: 2e-5}


def _err(a, b):
    return ((a.double() - b.double()).abs() / (1 + b.double().abs())).max().item() if b.numel() else 0.0


def _assert_close(gpu, ref, tol, what, exact=None):
    """float64: |gpu - ref| within tol. float32 (exact = float64 oracle on the same
    inputs): the GPU's error from exact within 4x the reference's own, or below tol."""
    gpu = gpu.cpu()
    assert gpu.shape == ref.shape, what
    if exact is None:
        err = _err(gpu, ref)
        assert err <= tol, f"{what}: {err:.3e} > {tol:.1e}"
    else:
        keep = ref > -1e29  # float32-only underflow sentinels are compared exactly below
        e_gpu, e_ref = _err(gpu[keep], exact[keep]), _err(ref[keep], exact[keep])
        assert e_gpu <= max(4 * e_ref, tol), f"{what}: float32 error {e_gpu:.3e} vs reference's {e_ref:.3e}"
    # exact sentinels
    assert torch.equal(gpu[ref <= -1e29], ref[ref <= -1e29]), what


def _exact(obj, lo, up, go):
    """float64 oracle on float32 inputs (upcast); None for float64 inputs."""
    if obj.dtype == torch.float64:
        return None, None
    d = lambda t: t.double()  # noqa: E731
    return (ola.forward(d(obj), d(lo), d(up), 1e-6, 1e-2),
            ola.backward(d(go), d(obj), d(lo), d(up), 1e-6, 1e-2))


def test_golden_reference_cases(cuda_lib):
    for key, c, tr, tm in golden_cases():
        dtype = c["obj"].dtype
        obj, lo, up = (c[k].to(DEV) for k in ("obj", "lower", "upper"))
        v = lf.forward(obj, lo, up, tr, tm)
        g = lf.backward(c["grad_out"].to(DEV), obj, lo, up, tr, tm)
        ev, eg = _exact(c["obj"], c["lower"], c["upper"], c["grad_out"])
        _assert_close(v, c["value"], TOL[dtype], key + " value", ev)
        _assert_close(g, c["grad"], TOL[dtype], key + " grad", eg)


def _random_case(g, B, n_sub, isz, m, nc, batched, dtype):
    obj = torch.randn(B, n_sub, isz, m, generator=g, dtype=torch.float64)
    near = torch.rand(obj.shape, generator=g) < 0.25
    obj = torch.where(near, obj * 1e-5, obj)
    lo = torch.randn(B if batched else 1, nc, m, generator=g, dtype=torch.float64) - 0.5
    up = lo + torch.rand(lo.shape, generator=g, dtype=torch.float64) * 2 + 1e-3
    if nc > 0:
        up[..., 0, :] = float("inf")
    if not batched:
        lo, up = lo[0], up[0]
    go = torch.randn(B, nc, n_sub, generator=g, dtype=torch.float64)
    return obj.to(dtype), lo.to(dtype), up.to(dtype), go.to(dtype)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_random_shapes_against_oracle(cuda_lib, dtype):
    g = torch.Generator().manual_seed(11)
    shapes = [(1, 1, 1, 1, 1, False), (9, 4, 1, 2, 5, False), (7, 6, 2, 2, 40, True),
              (5, 4, 3, 3, 17, False), (3, 1, 4, 4, 64, True), (4, 10, 5, 2, 3, False),
              (2, 8, 8, 3, 100, False), (3, 3, 9, 2, 6, True), (2, 2, 16, 8, 5, False),
              (2, 1, 17, 2, 33, True), (2, 1, 32, 8, 4, False), (64, 6, 2, 2, 1, False)]
    for B, n_sub, isz, m, nc, batched in shapes:
        obj, lo, up, go = _random_case(g, B, n_sub, isz, m, nc, batched, dtype)
        rv = ola.forward(obj, lo, up, 1e-6, 1e-2)
        rg = ola.backward(go, obj, lo, up, 1e-6, 1e-2)
        v = lf.forward(obj.to(DEV), lo.to(DEV), up.to(DEV), 1e-6, 1e-2)
        gr = lf.backward(go.to(DEV), obj.to(DEV), lo.to(DEV), up.to(DEV), 1e-6, 1e-2)
        what = f"{dtype} B={B} n_sub={n_sub} i={isz} m={m} nc={nc} batched={batched}"
        ev, eg = _exact(obj, lo, up, go)
        _assert_close(v, rv, TOL[dtype], what + " value", ev)
        _assert_close(gr, rg, TOL[dtype], what + " grad", eg)


def test_empty_inputs(cuda_lib):
    d = dict(dtype=torch.float64, device=DEV)
    cells = torch.zeros(3, 2, **d)
    assert lf.forward(torch.zeros(0, 4, 2, 2, **d), cells, cells + 1, 1e-6, 1e-2).shape == (0, 3, 4)
    assert lf.forward(torch.zeros(2, 0, 2, 2, **d), cells, cells + 1, 1e-6, 1e-2).shape == (2, 3, 0)
    empty_cells = torch.zeros(0, 2, **d)
    obj = torch.randn(2, 3, 2, 2, **d)
    assert lf.forward(obj, empty_cells, empty_cells, 1e-6, 1e-2).shape == (2, 0, 3)
    g = lf.backward(torch.zeros(2, 0, 3, **d), obj, empty_cells, empty_cells, 1e-6, 1e-2)
    assert g.shape == obj.shape and bool((g == 0).all())


def test_argument_errors(cuda_lib):
    d = dict(dtype=torch.float64, device=DEV)
    cells = torch.zeros(3, 2, **d)
    with pytest.raises(RuntimeError, match="subset_size or m too large"):
        lf.forward(torch.zeros(1, 1, 33, 2, **d), cells, cells + 1, 1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="one batch per obj_subsets batch"):
        lf.forward(torch.zeros(4, 1, 2, 2, **d), torch.zeros(3, 3, 2, **d), torch.ones(3, 3, 2, **d),
                   1e-6, 1e-2)
    with pytest.raises(RuntimeError, match="invalid argument"):
        lf.forward(torch.zeros(1, 1, 2, 2, **d), cells, cells + 1, 0.0, 1e-2)


def test_autograd_function_matches_unfused_path(cuda_lib):
    """FusedLogAreas with t-batch dims and batched cells against autograd through
    the reference's unfused steps (the reference's own test: atol 1e-6, rtol 1e-6)."""
    g = torch.Generator().manual_seed(5)
    obj = torch.randn(4, 3, 6, 2, 2, generator=g, dtype=torch.float64)  # (mc, batch, n_sub, i, m)
    lo = torch.randn(4, 3, 7, 2, generator=g, dtype=torch.float64) - 0.5
    up = lo + 1.0
    x = obj.to(DEV).requires_grad_(True)
    out = lf.FusedLogAreas.apply(x, lo.to(DEV), up.to(DEV), 1e-6, 1e-2)
    assert out.shape == (4, 3, 7, 6)
    w = torch.randn(out.shape, generator=g, dtype=torch.float64)
    (out * w.to(DEV)).sum().backward()
    xr = obj.clone().requires_grad_(True)
    ref = ola.python_path_log_areas(xr.reshape(12, 6, 2, 2), lo.reshape(12, 7, 2), up.reshape(12, 7, 2),
                                    1e-6, 1e-2).reshape(4, 3, 7, 6)
    (ref * w).sum().backward()
    torch.testing.assert_close(out.detach().cpu(), ref.detach(), atol=1e-6, rtol=1e-6)
    torch.testing.assert_close(x.grad.cpu(), xr.grad, atol=1e-6, rtol=1e-6)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_benchmark_size_rows_against_oracle(cuda_lib, dtype):
    """At the benchmark's size (B = 32768 sample-batches, q = 4, m = 2, 64 cells) the
    rows are independent: a seeded sample of rows matches the oracle on those rows."""
    from botorch_gb300.testing import log_areas_workload

    w = log_areas_workload(dtype=dtype, device=DEV)
    g = torch.Generator().manual_seed(2)
    rows = torch.randint(0, w.B, (48,), generator=g)
    for obj in w.obj_subsets:
        v = lf.forward(obj, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
        go = torch.ones_like(v)
        gr = lf.backward(go, obj, w.cell_lower, w.cell_upper, w.tau_relu, w.tau_max)
        sub = obj[rows.to(DEV)].cpu()
        cl, cu = w.cell_lower.cpu(), w.cell_upper.cpu()
        gsub = go[rows.to(DEV)].cpu()
        rv = ola.forward(sub, cl, cu, w.tau_relu, w.tau_max)
        rg = ola.backward(gsub, sub, cl, cu, w.tau_relu, w.tau_max)
        ev, eg = _exact(sub, cl, cu, gsub)
        _assert_close(v[rows.to(DEV)], rv, TOL[dtype], f"i={obj.shape[2]} value", ev)
        _assert_close(gr[rows.to(DEV)], rg, TOL[dtype], f"i={obj.shape[2]} grad", eg)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_jacobian_route_matches_recompute_route(cuda_lib, dtype):
    """forward_with_jacobian's areas equal forward's, and the Jacobian contraction
    equals the recomputing backward (float64 1e-12; float32 held to the float64
    oracle as above)."""
    g = torch.Generator().manual_seed(23)
    for B, n_sub, isz, m, nc, batched in [(9, 4, 1, 2, 5, False), (7, 6, 2, 2, 40, True),
                                          (4, 10, 5, 3, 3, False), (2, 1, 17, 2, 33, True),
                                          (2, 1, 32, 8, 4, False)]:
        obj, lo, up, go = _random_case(g, B, n_sub, isz, m, nc, batched, dtype)
        od, ld, ud, gd = obj.to(DEV), lo.to(DEV), up.to(DEV), go.to(DEV)
        v, jac = lf.forward_with_jacobian(od, ld, ud, 1e-6, 1e-2)
        assert jac.shape == (B, nc, n_sub, isz, m)
        v0 = lf.forward(od, ld, ud, 1e-6, 1e-2)
        torch.testing.assert_close(v, v0, atol=0, rtol=1e-14 if dtype == torch.float64 else 1e-6)
        gj = lf.backward_from_jacobian(gd, jac)
        rg = ola.backward(go, obj, lo, up, 1e-6, 1e-2)
        _, eg = _exact(obj, lo, up, go)
        _assert_close(gj, rg, TOL[dtype], f"{dtype} B={B} i={isz} m={m} nc={nc} jacobian grad", eg)


def test_autograd_routes(cuda_lib, monkeypatch):
    """FusedLogAreas keeps the Jacobian when the input needs a gradient and it fits the
    budget, and recomputes otherwise; both give the same gradient."""
    g = torch.Generator().manual_seed(31)
    obj, lo, up, _ = _random_case(g, 6, 6, 2, 2, 12, False, torch.float64)
    w = torch.randn(6, 12, 6, generator=g, dtype=torch.float64).to(DEV)
    grads = []
    for budget in (lf.JACOBIAN_BUDGET_BYTES, 0):
        monkeypatch.setattr(lf, "JACOBIAN_BUDGET_BYTES", budget)
        x = obj.to(DEV).requires_grad_(True)
        out = lf.FusedLogAreas.apply(x, lo.to(DEV), up.to(DEV), 1e-6, 1e-2)
        assert out.grad_fn is not None
        (out * w).sum().backward()
        grads.append(x.grad.clone())
    torch.testing.assert_close(grads[0], grads[1], atol=0, rtol=1e-12)
    with torch.no_grad():  # no gradient wanted: the plain forward
        v = lf.FusedLogAreas.apply(obj.to(DEV), lo.to(DEV), up.to(DEV), 1e-6, 1e-2)
    torch.testing.assert_close(v, lf.forward(obj.to(DEV), lo.to(DEV), up.to(DEV), 1e-6, 1e-2), atol=0, rtol=0)
