"""SingleTaskGP drop-in whose training cache and posterior run on the CUDA library.

Mirrors ``botorch.models.SingleTaskGP`` (botorch/models/gp_regression.py:108-214)
with fixed hyperparameters: the Standardize outcome transform is fitted on
train_Y (botorch/models/transforms/outcome.py:312-345), the training
covariance K + noise I is factorised once with psd_safe_cholesky semantics,
and ``posterior(X)`` returns the untransformed joint posterior of each
t-batch (botorch/models/gpytorch.py:544-611). All compute is in
libbotorch_gb300.so; this module only moves tensors and checks return codes.
"""

from __future__ import annotations

import ctypes

import torch
from torch import Tensor

from botorch_gb300 import _native as nat
from botorch_gb300.exceptions import UnsupportedError
from botorch_gb300.kernels import (ConstantMean, GaussianLikelihood, default_covar_module,
                                   default_likelihood, unpack_covar_module)

_DEFAULT = object()


class Standardize:
    """Outcome transform state: Y -> (Y - mean) / std (outcome.py:236-345).

    ``std`` is the unbiased standard deviation, replaced by 1 when below
    ``min_stdv`` or when there is a single observation.
    """

    def __init__(self, m: int = 1, min_stdv: float = 1e-8) -> None:
        if m != 1:
            raise UnsupportedError("only single-output models are supported")
        self.m = m
        self.min_stdv = min_stdv
        self.means: float | None = None
        self.stdvs: float | None = None

    def fit(self, Y: Tensor) -> Tensor:
        Y = Y.to(torch.float64)
        std = 1.0 if Y.shape[-2] == 1 else float(Y.std(dim=-2).item())
        if not std >= self.min_stdv:
            std = 1.0
        self.means = float(Y.mean().item())
        self.stdvs = std
        return (Y - self.means) / self.stdvs


class GPyTorchPosterior:
    """Posterior over ``batch x q`` points: mean, variance, covariance and reparameterised
    samples (botorch/posteriors/gpytorch.py:33-127)."""

    def __init__(self, mean: Tensor, covariance: Tensor) -> None:
        self._mean = mean            # batch x q
        self._covar = covariance     # batch x q x q

    @property
    def mean(self) -> Tensor:
        return self._mean.unsqueeze(-1)

    @property
    def variance(self) -> Tensor:
        return self._covar.diagonal(dim1=-2, dim2=-1).unsqueeze(-1)

    @property
    def covariance_matrix(self) -> Tensor:
        return self._covar

    @property
    def device(self) -> torch.device:
        return self._mean.device

    @property
    def dtype(self) -> torch.dtype:
        return self._mean.dtype

    @property
    def base_sample_shape(self) -> torch.Size:
        return self._mean.shape + torch.Size([1])

    @property
    def batch_range(self) -> tuple[int, int]:
        return (0, -2)

    def _extended_shape(self, sample_shape: torch.Size = torch.Size()) -> torch.Size:  # noqa: B008
        return sample_shape + self._mean.shape + torch.Size([1])

    def rsample_from_base_samples(self, sample_shape: torch.Size, base_samples: Tensor) -> Tensor:
        """``sample_shape x batch x q x 1`` samples mean + L z, L = psd_safe_cholesky of each
        batch member's covariance (botorch/posteriors/gpytorch.py:86-127, gpytorch
        MultivariateNormal.rsample), computed by ``bgb_mvn_rsample``. ``base_samples``:
        ``sample_shape x (1 ...) x q x 1`` (batch dimensions collapsed to 1, as the
        reference's QMC samplers draw them) or ``sample_shape x q x 1``."""
        sample_shape = torch.Size(sample_shape)
        if base_samples.shape[: len(sample_shape)] != sample_shape:
            raise RuntimeError("sample_shape disagrees with shape of base_samples.")
        q = self._mean.shape[-1]
        batch_shape = self._mean.shape[:-1]
        rest = base_samples.shape[len(sample_shape):]
        if rest[-2:] != torch.Size([q, 1]) or any(s != 1 for s in rest[:-2]):
            raise UnsupportedError("base samples must be sample_shape x (1 ...) x q x 1: the same "
                                   "base samples for every batch member")
        S = int(sample_shape.numel())
        b = int(batch_shape.numel())
        dev = self._mean.device
        Z = base_samples.detach().reshape(S, q).to(dev, torch.float64).contiguous()
        mean = self._mean.detach().reshape(b, q).to(torch.float64).contiguous()
        cov = self._covar.detach().reshape(b, q, q).to(torch.float64).contiguous()
        out = torch.empty(S, b, q, dtype=torch.float64, device=dev)
        status = torch.empty(b, dtype=torch.int32, device=dev)
        lib = nat.lib()
        with torch.cuda.device(dev):
            rc = lib.bgb_mvn_rsample(nat.ptr(mean), nat.ptr(cov), b, q, nat.ptr(Z), S, 6,
                                     nat.ptr(out), nat.ptr(status), nat.stream_handle(dev))
        nat.check(rc, "posterior samples")
        worst = int(status.max().item()) if b > 0 else 0
        if worst != nat.BGB_OK:
            nat.check(worst, "posterior samples (psd_safe_cholesky)")
        return out.reshape(*sample_shape, *batch_shape, q, 1).to(self._mean.dtype)

    def rsample(self, sample_shape: torch.Size | None = None) -> Tensor:
        """Samples from i.i.d. standard normal base samples (torch.randn on the device)."""
        sample_shape = torch.Size([1]) if sample_shape is None else torch.Size(sample_shape)
        q = self._mean.shape[-1]
        z = torch.randn(*sample_shape, *([1] * (self._mean.dim() - 1)), q, 1, dtype=torch.float64,
                        device=self._mean.device)
        return self.rsample_from_base_samples(sample_shape, z)


class SingleTaskGP:
    """Exact GP with fixed hyperparameters on one CUDA device.

    Args mirror the reference: ``train_X`` (n x d), ``train_Y`` (n x 1),
    ``likelihood`` (GaussianLikelihood), ``covar_module`` (ScaleKernel /
    MaternKernel / RBFKernel), ``mean_module`` (ConstantMean),
    ``outcome_transform`` (Standardize by default, ``None`` to disable).
    ``train_Yvar`` and ``input_transform`` are not supported on this path.
    """

    def __init__(self, train_X: Tensor, train_Y: Tensor, train_Yvar: Tensor | None = None,
                 likelihood: GaussianLikelihood | None = None, covar_module=None,
                 mean_module: ConstantMean | None = None, outcome_transform=_DEFAULT,
                 input_transform=None, device: torch.device | str | None = None) -> None:
        if train_Yvar is not None:
            raise UnsupportedError("train_Yvar (fixed noise) is not supported on this path")
        if input_transform is not None:
            raise UnsupportedError("input transforms are not supported on this path")
        if train_X.dim() != 2 or train_Y.dim() != 2 or train_Y.shape[-1] != 1:
            raise UnsupportedError("expected train_X n x d and train_Y n x 1 (no batch, one output)")
        if device is None:
            device = train_X.device if train_X.is_cuda else torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise UnsupportedError("botorch_gb300 runs on CUDA devices only")
        n, d = train_X.shape
        self.n, self.d = n, d
        # the reference's defaults: LogNormal-prior noise and a dimension-scaled-prior RBF
        # kernel (botorch/models/gp_regression.py:173-201)
        self.likelihood = likelihood if likelihood is not None else default_likelihood()
        self.covar_module = covar_module if covar_module is not None else default_covar_module(d)
        self.mean_module = mean_module if mean_module is not None else ConstantMean()
        kind, ls, outputscale = unpack_covar_module(self.covar_module)
        if ls.numel() not in (1, d):
            raise ValueError(f"lengthscale has {ls.numel()} entries, expected 1 or {d}")
        self.kernel_kind = kind
        self.lengthscale = ls.expand(d).clone() if ls.numel() == 1 else ls.clone()
        self.outputscale = outputscale
        self.noise = self.likelihood.noise
        self.mean_constant = self.mean_module.constant
        if outcome_transform is _DEFAULT:
            outcome_transform = Standardize(m=1)
        self.outcome_transform = outcome_transform
        Y = train_Y.to(torch.float64)
        if outcome_transform is not None:
            Y = outcome_transform.fit(Y)
            self.y_mean, self.y_std = outcome_transform.means, outcome_transform.stdvs
        else:
            self.y_mean, self.y_std = 0.0, 1.0
        dev = self.device
        self.train_inputs = (train_X.detach().to(dev, torch.float64).contiguous(),)
        self.train_targets = Y.squeeze(-1).detach().to(dev).contiguous()
        self.inv_lengthscale = (1.0 / self.lengthscale).to(dev, torch.float64).contiguous()
        self._ws = nat.Workspace(dev)
        self._fit()

    # ------------------------------------------------------------------ C ABI
    def gp_struct(self) -> nat.BgbGP:
        return nat.BgbGP(n=self.n, d=self.d, kernel=nat.KERNELS[self.kernel_kind],
                         outputscale=self.outputscale, mean_constant=self.mean_constant,
                         y_mean=self.y_mean, y_std=self.y_std,
                         train_X=nat.ptr(self.train_inputs[0]),
                         inv_lengthscale=nat.ptr(self.inv_lengthscale))

    def set_hyperparameters(self, lengthscale=None, outputscale: float | None = None,
                            noise: float | None = None, mean_constant: float | None = None) -> None:
        """New hyperparameter values (standardised outcome space) and a refit of the
        training cache; operands built for acquisition functions are dropped, so
        acquisition functions are built after fitting, as in the reference."""
        if lengthscale is not None:
            ls = torch.as_tensor(lengthscale, dtype=torch.float64).reshape(-1)
            self.lengthscale = (ls.expand(self.d) if ls.numel() == 1 else ls).clone().cpu()
            self.inv_lengthscale = (1.0 / self.lengthscale).to(self.device, torch.float64).contiguous()
        if outputscale is not None:
            self.outputscale = float(outputscale)
        if noise is not None:
            self.noise = float(noise)
        if mean_constant is not None:
            self.mean_constant = float(mean_constant)
        self._fit()

    def _fit(self) -> None:
        lib = nat.lib()
        n, dev = self.n, self.device
        self.L = torch.empty(n, n, dtype=torch.float64, device=dev)
        self.Linv = torch.empty(n, n, dtype=torch.float64, device=dev)
        self.alpha = torch.empty(n, dtype=torch.float64, device=dev)
        self.beta = torch.empty(n, dtype=torch.float64, device=dev)
        jitter = ctypes.c_double(0.0)
        ws, wsb = self._ws.get(lib.bgb_gp_fit_workspace_bytes(n))
        gp = self.gp_struct()
        with torch.cuda.device(dev):
            rc = lib.bgb_gp_fit(ctypes.byref(gp), nat.ptr(self.train_targets), self.noise, 6,
                                nat.ptr(self.L), nat.ptr(self.Linv), nat.ptr(self.alpha),
                                nat.ptr(self.beta), ctypes.byref(jitter), ws, wsb,
                                nat.stream_handle(dev))
        nat.check(rc, "SingleTaskGP training covariance")
        self.train_jitter = jitter.value
        self._ws.buf = None  # the fit scratch (n^2 doubles) is not needed afterwards
        self._operands: dict[str, tuple] = {}

    def operands(self, precision: str):
        """Model-level operands of the C ABI, built once per precision.

        Returns (B64, B32, ldb, Linv32, beta32, tc, Xs64, Xs32) with B = L^-T,
        float32 copies of L^-1 and beta, for the mixed path ``tc`` = (Lhi, Llo,
        LThi, LTlo, Lmul, LTmul, ldl, beta_absmax): the row-scaled float16 hi/lo
        split of L^-1 and L^-T used by the tensor-core GEMMs with the inverse row
        scales, and max |beta|; and the training inputs scaled by 1 / lengthscale.
        """
        if precision in self._operands:
            return self._operands[precision]
        lib = nat.lib()
        n = self.n
        ldb = ((n + 7) // 8) * 8
        dev = self.device
        B64 = torch.empty(n, ldb, dtype=torch.float64, device=dev)
        mixed = precision == "mixed"
        B32 = torch.empty(n, ldb, dtype=torch.float32, device=dev) if mixed else None
        L32 = torch.empty(n, n, dtype=torch.float32, device=dev) if mixed else None
        b32 = torch.empty(n, dtype=torch.float32, device=dev) if mixed else None
        Xs64 = torch.empty(self.d, n, dtype=torch.float64, device=dev)
        Xs32 = torch.empty(self.d, n, dtype=torch.float32, device=dev) if mixed else None
        gp = self.gp_struct()
        with torch.cuda.device(dev):
            rc = lib.bgb_gp_operands(ctypes.byref(gp), nat.ptr(self.Linv), nat.ptr(self.beta),
                                     nat.ptr(B64), nat.ptr(B32), ldb, nat.ptr(L32), nat.ptr(b32),
                                     nat.ptr(Xs64), nat.ptr(Xs32), nat.stream_handle(dev))
            nat.check(rc, "model operands")
            tc = None
            if mixed:
                halves = tuple(torch.empty(n, ldb, dtype=torch.float16, device=dev) for _ in range(4))
                muls = tuple(torch.empty(n, dtype=torch.float32, device=dev) for _ in range(2))
                rc = lib.bgb_gp_tc_operands(ctypes.byref(gp), nat.ptr(self.Linv), ldb,
                                            *(nat.ptr(t) for t in halves + muls),
                                            nat.stream_handle(dev))
                nat.check(rc, "tensor-core operands")
                tc = halves + muls + (ldb, float(self.beta.abs().max()))
        self._operands[precision] = (B64, B32, ldb, L32, b32, tc, Xs64, Xs32)
        return self._operands[precision]

    def acq_struct_base(self, precision: str, tensor_cores: bool = True) -> dict:
        """Keyword arguments of BgbAcq shared by every acquisition call on this model."""
        B64, B32, ldb, L32, b32, tc, Xs64, Xs32 = self.operands(precision)
        kw = dict(gp=self.gp_struct(), precision=nat.PRECISIONS[precision], ldb=ldb,
                  B64=nat.ptr(B64), B32=nat.ptr(B32), Linv64=nat.ptr(self.Linv),
                  Linv32=nat.ptr(L32), beta64=nat.ptr(self.beta), beta32=nat.ptr(b32),
                  Xs64=nat.ptr(Xs64), Xs32=nat.ptr(Xs32))
        if tc is not None:
            kw.update(Lhi=nat.ptr(tc[0]), Llo=nat.ptr(tc[1]), LThi=nat.ptr(tc[2]),
                      LTlo=nat.ptr(tc[3]), Lmul=nat.ptr(tc[4]), LTmul=nat.ptr(tc[5]), ldl=tc[6],
                      beta_absmax=tc[7])
        if not tensor_cores:
            kw["flags"] = nat.BGB_FLAG_SIMT
        return kw

    def baseline_operands(self, X_baseline: Tensor, precision: str):
        """(Vb64, Vb32, VbT64, VbT32) with Vb = K(X_baseline, Xt) L^-T."""
        lib = nat.lib()
        r = int(X_baseline.shape[0])
        Xb = X_baseline.detach().to(self.device, torch.float64).contiguous()
        dev = self.device
        Vb64 = torch.empty(r, self.n, dtype=torch.float64, device=dev)
        VbT64 = torch.empty(self.n, r, dtype=torch.float64, device=dev)
        mixed = precision == "mixed"
        Vb32 = torch.empty(r, self.n, dtype=torch.float32, device=dev) if mixed else None
        VbT32 = torch.empty(self.n, r, dtype=torch.float32, device=dev) if mixed else None
        ws = nat.Workspace(dev)
        wp, wb = ws.get(lib.bgb_baseline_operands_workspace_bytes(self.n, r))
        gp = self.gp_struct()
        with torch.cuda.device(dev):
            rc = lib.bgb_baseline_operands(ctypes.byref(gp), nat.ptr(self.Linv), nat.ptr(Xb), r,
                                           nat.ptr(Vb64), nat.ptr(Vb32), nat.ptr(VbT64),
                                           nat.ptr(VbT32), wp, wb, nat.stream_handle(dev))
        nat.check(rc, "baseline operands")
        return Vb64, Vb32, VbT64, VbT32

    def posterior_joint(self, X: Tensor) -> tuple[Tensor, Tensor]:
        """Joint posterior (mean m, covariance m x m) over m points, float64."""
        lib = nat.lib()
        X = X.detach().to(self.device, torch.float64).contiguous()
        m = X.shape[0]
        mean = torch.empty(m, dtype=torch.float64, device=self.device)
        cov = torch.empty(m, m, dtype=torch.float64, device=self.device)
        ws = nat.Workspace(self.device)
        wp, wb = ws.get(lib.bgb_posterior_joint_workspace_bytes(self.n, m))
        gp = self.gp_struct()
        with torch.cuda.device(self.device):
            rc = lib.bgb_posterior_joint(ctypes.byref(gp), nat.ptr(self.Linv), nat.ptr(self.alpha),
                                         nat.ptr(X), m, nat.ptr(mean), nat.ptr(cov), wp, wb,
                                         nat.stream_handle(self.device))
        nat.check(rc, "joint posterior")
        return mean, cov

    # ------------------------------------------------------------ reference API
    @property
    def num_outputs(self) -> int:
        return 1

    @property
    def batch_shape(self) -> torch.Size:
        return torch.Size([])

    def posterior(self, X: Tensor, output_indices=None, observation_noise: bool = False,
                  posterior_transform=None, precision: str = "fp64") -> GPyTorchPosterior:
        """Posterior at ``batch x q x d`` (or ``q x d``) points.

        Forward-only: the returned tensors carry no autograd graph (the
        acquisition functions of this package differentiate through their own
        fused adjoint kernels).
        """
        if output_indices not in (None, [0]) or posterior_transform is not None:
            raise UnsupportedError("output_indices / posterior_transform are not supported")
        if observation_noise is not False and observation_noise is not True:
            raise UnsupportedError("observation_noise must be a bool (a noise tensor is not supported)")
        squeeze = X.dim() == 2
        Xb = X.unsqueeze(0) if squeeze else X
        batch_shape = Xb.shape[:-2]
        q = Xb.shape[-2]
        Xf = Xb.reshape(-1, q, self.d).detach().to(self.device, torch.float64).contiguous()
        b = Xf.shape[0]
        lib = nat.lib()
        acq = nat.BgbAcq(acqf=nat.ACQF_QEI, q=q, r=0, n_samples=1,
                         **self.acq_struct_base(precision))
        mean = torch.empty(b, q, dtype=torch.float64, device=self.device)
        cov = torch.empty(b, q, q, dtype=torch.float64, device=self.device)
        wp, wb = self._ws.get(lib.bgb_acq_workspace_bytes(ctypes.byref(acq), b))
        with torch.cuda.device(self.device):
            rc = lib.bgb_posterior(ctypes.byref(acq), nat.ptr(Xf), b, nat.ptr(mean), nat.ptr(cov),
                                   wp, wb, nat.stream_handle(self.device))
        nat.check(rc, "posterior")
        if observation_noise:
            # the likelihood's noise on the diagonal, then the outcome untransform
            # (gpytorch likelihood(mvn) followed by Standardize.untransform_posterior)
            cov.diagonal(dim1=-2, dim2=-1).add_(self.noise * self.y_std * self.y_std)
        mean = mean.reshape(*batch_shape, q)
        cov = cov.reshape(*batch_shape, q, q)
        if squeeze:
            mean, cov = mean[0], cov[0]
        return GPyTorchPosterior(mean.to(X.dtype), cov.to(X.dtype))
