"""Float64 dense routines of the training side on the GPU: the in-place
lower-triangular inverse (bgb_tri_inverse) at sizes that exercise every shape
of its recursion (a single diagonal block, ragged last blocks, ragged last
pairs at several levels) against a LAPACK triangular solve on the host.

The reference computes L^-1 implicitly through linear_operator's triangular
solves (gpytorch exact prediction strategy); the product path keeps L^-1
explicitly, so its accuracy is checked here directly.
"""

import pytest
import torch

from botorch_gb300 import _native as nat

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def lower_factor(n: int, seed: int) -> torch.Tensor:
    """Cholesky factor of a well-conditioned SPD matrix (condition ~1e3)."""
    g = torch.Generator().manual_seed(seed)
    A = torch.randn(n, n, generator=g, dtype=torch.float64)
    Q, _ = torch.linalg.qr(A)
    ev = torch.logspace(0, 3, n, dtype=torch.float64)
    return torch.linalg.cholesky((Q * ev) @ Q.T)


@pytest.mark.parametrize("n", [1, 37, 64, 65, 128, 200, 383, 1000, 1500, 2048])
def test_tri_inverse_matches_host(n):
    lib = nat.lib()
    Lh = lower_factor(n, seed=n)
    # junk above the diagonal: the routine must ignore it and leave zeros there
    L = torch.tril(Lh.to(DEV)) + torch.rand(n, n, dtype=torch.float64, device=DEV).triu(1)
    wsb = lib.bgb_tri_inverse_workspace_bytes(n)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=DEV)
    rc = lib.bgb_tri_inverse(nat.ptr(L), n, n, nat.ptr(ws), wsb, nat.stream_handle(DEV))
    torch.cuda.synchronize()
    assert rc == 0
    ref = torch.linalg.solve_triangular(Lh, torch.eye(n, dtype=torch.float64), upper=False)
    out = L.cpu()
    assert bool((out.triu(1) == 0).all())
    assert float((out - ref).norm() / ref.norm()) < 1e-12
    # residual of the inverse itself: ||L X - I|| relative to ||L|| ||X||
    res = (Lh @ out - torch.eye(n, dtype=torch.float64)).norm() / (Lh.norm() * out.norm())
    assert float(res) < 1e-14


def test_tri_inverse_strided_rows():
    """lda > n: the routine works on the leading n x n block and leaves the rest."""
    lib = nat.lib()
    n, lda = 300, 320
    Lh = lower_factor(n, seed=7)
    big = torch.full((n, lda), 3.25, dtype=torch.float64)
    big[:, :n] = Lh
    L = big.to(DEV).contiguous()
    wsb = lib.bgb_tri_inverse_workspace_bytes(n)
    ws = torch.empty(wsb, dtype=torch.uint8, device=DEV)
    rc = lib.bgb_tri_inverse(nat.ptr(L), n, lda, nat.ptr(ws), wsb, nat.stream_handle(DEV))
    torch.cuda.synchronize()
    assert rc == 0
    out = L.cpu()
    ref = torch.linalg.solve_triangular(Lh, torch.eye(n, dtype=torch.float64), upper=False)
    assert float((out[:, :n] - ref).norm() / ref.norm()) < 1e-12
    assert bool((out[:, n:] == 3.25).all())
