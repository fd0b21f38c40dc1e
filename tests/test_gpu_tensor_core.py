"""The tcgen05 float16-split cross-covariance GEMM through the C ABI.

Float32 accuracy is the bar: ||C - C_ref|| / ||C_ref|| below 5e-6 against a
float64 product of the operands the float16 hi/lo splits represent.
"""

import ctypes

import pytest
import torch

from botorch_gb300 import _native as nat

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def pow2_scale(m: torch.Tensor) -> torch.Tensor:
    """2^(14 - e) with m = f 2^e, f in [0.5, 1): brings m to at most 2^14 (1 for m = 0)."""
    _, e = torch.frexp(m)
    return torch.where(m > 0, torch.exp2(14.0 - e.double()), torch.ones_like(m))


def split16(x: torch.Tensor, scale: torch.Tensor):
    """Row-scaled float16 split: hi = f16(s x), lo = f16(s x - hi), rows scaled by `scale`."""
    xs = x * scale[:, None]
    hi = xs.half()
    lo = (xs - hi.double()).half()
    return hi, lo


@pytest.mark.parametrize("M,N,K", [(300, 512, 384), (128, 256, 32), (1000, 777, 777), (64, 64, 64)])
@pytest.mark.parametrize("kmode", [0, 1, 3])
def test_tc_gemm_matches_float64(cuda_lib, M, N, K, kmode):
    g = torch.Generator().manual_seed(M + N + K + kmode)
    A = (torch.rand(M, K, generator=g, dtype=torch.float64) - 0.3) * torch.exp2(
        torch.randint(-12, 12, (M, 1), generator=g).double())
    Bs = torch.randn(N, K, generator=g, dtype=torch.float64) * torch.exp2(
        torch.randint(-12, 12, (N, 1), generator=g).double())
    jj, kk = torch.meshgrid(torch.arange(N), torch.arange(K), indexing="ij")
    if kmode == 3:    # op(B) upper triangular: op(B)[k][j] = Bs[j][k] != 0 only for k <= j
        Bs = Bs * (kk <= jj)
    elif kmode == 1:  # op(B) lower triangular: k >= j
        Bs = Bs * (kk >= jj)
    lda = (K + 7) // 8 * 8
    ldc = (N + 7) // 8 * 8
    sa, sb = pow2_scale(A.abs().amax(1)), pow2_scale(Bs.abs().amax(1))
    Ahi, Alo = split16(A, sa)
    Bhi, Blo = split16(Bs, sb)
    pad = lambda t, ld: torch.nn.functional.pad(t, (0, ld - t.shape[1])).contiguous().to(DEV)  # noqa: E731
    Ahi_d, Alo_d, Bhi_d, Blo_d = pad(Ahi, lda), pad(Alo, lda), pad(Bhi, lda), pad(Blo, lda)
    row_mul = (1.0 / sa).float().to(DEV)
    col_mul = (1.0 / sb).float().to(DEV)
    C = torch.full((M, ldc), float("nan"), dtype=torch.float32, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    rc = cuda_lib.bgb_crosscov_gemm_f16x3(M, N, K, Ahi_d.data_ptr(), Alo_d.data_ptr(), lda,
                                          Bhi_d.data_ptr(), Blo_d.data_ptr(), lda, C.data_ptr(), ldc,
                                          row_mul.data_ptr(), 0.0, col_mul.data_ptr(), kmode,
                                          err.data_ptr(), nat.stream_handle(DEV))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    Arep = (Ahi.double() + Alo.double()) / sa[:, None]
    Brep = (Bhi.double() + Blo.double()) / sb[:, None]
    ref = Arep @ Brep.T
    out = C[:, :N].double().cpu()
    assert torch.isfinite(out).all()
    assert float((out - ref).norm() / ref.norm()) < 5e-6
    # the represented operands are the originals to 2^-22 relative
    assert float((Arep - A).norm() / A.norm()) < 1e-6


def test_tc_gemm_constant_row_multiplier(cuda_lib):
    """row_mul NULL: every row uses row_mul_const (the forward GEMM's form)."""
    g = torch.Generator().manual_seed(5)
    M, N, K = 256, 256, 256
    A = torch.rand(M, K, generator=g, dtype=torch.float64)
    Bs = torch.randn(N, K, generator=g, dtype=torch.float64)
    sa = torch.full((M,), 2.0 ** 14, dtype=torch.float64)
    sb = pow2_scale(Bs.abs().amax(1))
    Ahi, Alo = split16(A, sa)
    Bhi, Blo = split16(Bs, sb)
    Ahi_d, Alo_d, Bhi_d, Blo_d = (t.contiguous().to(DEV) for t in (Ahi, Alo, Bhi, Blo))
    col_mul = (1.0 / sb).float().to(DEV)
    C = torch.empty(M, N, dtype=torch.float32, device=DEV)
    rc = cuda_lib.bgb_crosscov_gemm_f16x3(M, N, K, Ahi_d.data_ptr(), Alo_d.data_ptr(), K,
                                          Bhi_d.data_ptr(), Blo_d.data_ptr(), K, C.data_ptr(), N,
                                          None, 2.0 ** -14, col_mul.data_ptr(), 0, None,
                                          nat.stream_handle(DEV))
    assert rc == 0
    ref = ((Ahi.double() + Alo.double()) / 2.0 ** 14) @ ((Bhi.double() + Blo.double()) / sb[:, None]).T
    out = C.double().cpu()
    assert float((out - ref).norm() / ref.norm()) < 5e-6


def test_mixed_tensor_core_and_ffma_paths_against_fp64(cuda_lib):
    """Both float32 GEMM forms of the mixed path against the float64 GPU path on a
    Branin-sum workload (n=1024, d=20, q=8, y_std ~ 160). Values hold 2e-5; the
    gradient is dominated by t-batches within ~100 tau_relu of the incumbent
    (see test_qlognei_differentiation_config), so its bound is 1e-2."""
    from botorch_gb300 import testing as T
    from tests.test_gpu_parity import gpu_model
    from botorch_gb300 import SobolQMCNormalSampler, qLogNoisyExpectedImprovement

    w = T.qlognei_branin(n=1024, b=256, q=8, d=20)
    gm = gpu_model(w)
    out = {}
    for name, precision, tc in (("fp64", "fp64", False), ("tc", "mixed", True), ("ffma", "mixed", False)):
        torch.manual_seed(0)
        a = qLogNoisyExpectedImprovement(gm, w.train_X, sampler=SobolQMCNormalSampler(
            torch.Size([512]), seed=0), precision=precision)
        a.use_tensor_cores = tc
        X = w.X.to(DEV).requires_grad_(True)
        v = a(X)
        v.sum().backward()
        out[name] = (v.detach().cpu(), X.grad.cpu())
    v64, g64 = out["fp64"]
    for name in ("tc", "ffma"):
        v, g = out[name]
        ev = float((v - v64).norm() / v64.norm())
        eg = float((g - g64).norm() / g64.norm())
        assert ev < 2e-5 and eg < 1e-2, (name, ev, eg)
