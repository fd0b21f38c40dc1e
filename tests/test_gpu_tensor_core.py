"""The tcgen05 3xTF32 cross-covariance GEMM through the C ABI.

Float32 accuracy is the bar: ||C - C_ref|| / ||C_ref|| below 5e-6 against a
float64 product of the same (float32) operands.
"""

import ctypes

import pytest
import torch

from botorch_gb300 import _native as nat

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def split(x: torch.Tensor):
    """tf32 round-to-nearest split in float64 arithmetic: hi = tf32(x), lo = tf32(x - hi)."""
    def tf32(t):
        i = t.float().contiguous().view(torch.int32)
        i = (i + 0x1000) & ~0x1FFF
        return i.view(torch.float32)
    hi = tf32(x)
    lo = tf32(x.double() - hi.double())
    return hi, lo


@pytest.mark.parametrize("M,N,K", [(300, 512, 384), (128, 256, 32), (1000, 777, 777), (64, 64, 64)])
@pytest.mark.parametrize("kmode", [0, 1, 3])
def test_tc_gemm_matches_float64(cuda_lib, M, N, K, kmode):
    g = torch.Generator().manual_seed(M + N + K + kmode)
    A = torch.rand(M, K, generator=g, dtype=torch.float64) - 0.3
    Bs = torch.randn(N, K, generator=g, dtype=torch.float64)
    jj, kk = torch.meshgrid(torch.arange(N), torch.arange(K), indexing="ij")
    if kmode == 3:    # op(B) upper triangular: op(B)[k][j] = Bs[j][k] != 0 only for k <= j
        Bs = Bs * (kk <= jj)
    elif kmode == 1:  # op(B) lower triangular: k >= j
        Bs = Bs * (kk >= jj)
    lda = (K + 7) // 8 * 8
    ldc = (N + 7) // 8 * 8
    Ahi, Alo = split(A)
    Bhi, Blo = split(Bs)
    pad = lambda t, ld: torch.nn.functional.pad(t, (0, ld - t.shape[1])).contiguous().to(DEV)  # noqa: E731
    Ahi_d, Alo_d, Bhi_d, Blo_d = pad(Ahi, lda), pad(Alo, lda), pad(Bhi, lda), pad(Blo, lda)
    C = torch.full((M, ldc), float("nan"), dtype=torch.float32, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    rc = cuda_lib.bgb_crosscov_gemm_tf32x3(M, N, K, Ahi_d.data_ptr(), Alo_d.data_ptr(), lda,
                                           Bhi_d.data_ptr(), Blo_d.data_ptr(), lda, C.data_ptr(),
                                           ldc, kmode, err.data_ptr(), nat.stream_handle(DEV))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = (Ahi.double() + Alo.double()) @ (Bhi.double() + Blo.double()).T
    out = C[:, :N].double().cpu()
    assert torch.isfinite(out).all()
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
