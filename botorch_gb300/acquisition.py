"""qExpectedImprovement and qLogNoisyExpectedImprovement on the CUDA library.

The classes keep the reference's constructor arguments and ``forward``
contract (``batch_shape x q x d`` -> ``batch_shape``) so they drop into
``optimize_acqf`` / ``gen_candidates_scipy`` (botorch/generation/gen.py:423-487).
``forward`` is differentiable in X: when X requires grad, one fused call
computes the value and the hand-written adjoint gradient, and the gradient is
handed to autograd by ``_FusedValueGrad``.

References: botorch/acquisition/monte_carlo.py:268-305 and :374-437 (qEI),
botorch/acquisition/logei.py:246-565 (qLogNEI with cached root),
botorch/acquisition/cached_cholesky.py:126-192, botorch/utils/low_rank.py:84-172,
botorch/acquisition/utils.py:97-141 and :347-437 (best_f and pruning).
"""

from __future__ import annotations

import ctypes
import math
import warnings

import torch
from torch import Tensor

from botorch_gb300 import _native as nat
from botorch_gb300.exceptions import BotorchWarning, NanError, NotPSDError, UnsupportedError
from botorch_gb300.gp_regression import SingleTaskGP
from botorch_gb300.sampling import SobolQMCNormalSampler, draw_sobol_normal_samples

TAU_RELU = 1e-6
TAU_MAX = 1e-2


class _FusedValueGrad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X: Tensor, acqf: "_MCAcquisition") -> Tensor:
        need_grad = ctx.needs_input_grad[0]
        value, grad = acqf._run(X, need_grad)
        if need_grad:
            ctx.save_for_backward(grad)
        return value

    @staticmethod
    def backward(ctx, g: Tensor):
        (grad,) = ctx.saved_tensors
        return g.reshape(*g.shape, 1, 1) * grad, None


class _MCAcquisition:
    """Shared plumbing: t-batch handling, device buffers, C ABI calls."""

    acqf_id = -1

    def __init__(self, model: SingleTaskGP, sampler: SobolQMCNormalSampler | None,
                 objective, posterior_transform, constraints, precision: str) -> None:
        if not isinstance(model, SingleTaskGP):
            raise UnsupportedError("model must be a botorch_gb300 SingleTaskGP")
        if objective is not None and type(objective).__name__ != "IdentityMCObjective":
            raise UnsupportedError("only the identity MC objective is supported on this path")
        if posterior_transform is not None or constraints is not None:
            raise UnsupportedError("posterior transforms and constraints are not supported")
        if precision not in nat.PRECISIONS:
            raise ValueError(f"precision must be one of {list(nat.PRECISIONS)}")
        self.model = model
        self.sampler = sampler
        self.precision = precision
        self.device = model.device
        self._ws = nat.Workspace(self.device)
        self._Z: dict[int, Tensor] = {}
        self._structs: dict = {}  # (q, tensor cores) -> (BgbAcq, its Z tensor, {b: workspace bytes})
        self._graphs: dict = {}   # (b, q, need_grad, tensor cores) -> captured call
        self.check_status = True
        self.use_tensor_cores = True  # mixed path: tcgen05 GEMMs (False: FFMA GEMMs)
        # forward through CUDA graphs captured per (b, q): for loops that call with
        # a fixed shape (the restarts of an optimiser); each shape keeps its own
        # workspace while captured
        self.use_cuda_graphs = False
        # schedule knob: CTAs per SM the adjoint contraction aims for (0: library default)
        self.adjoint_ctas_per_sm = 0
        self.X_pending: Tensor | None = None

    # -------------------------------------------------------------- override
    def _base_samples(self, q: int) -> Tensor:
        raise NotImplementedError

    def _acq_struct(self, q: int) -> nat.BgbAcq:
        raise NotImplementedError

    # ------------------------------------------------------------------ call
    def __call__(self, X: Tensor) -> Tensor:
        return self.forward(X)

    def forward(self, X: Tensor) -> Tensor:
        if X.dim() < 2:
            raise ValueError(f"{type(self).__name__} requires X to have at least 2 dimensions,"
                             f" but received X with only {X.dim()} dimensions.")
        X3 = X if X.dim() > 2 else X.unsqueeze(0)
        return _FusedValueGrad.apply(X3, self)

    def _prepare_X(self, X: Tensor) -> Tensor:
        return X

    def _run(self, X: Tensor, need_grad: bool) -> tuple[Tensor, Tensor | None]:
        batch_shape = X.shape[:-2]
        Xf = self._prepare_X(X)
        q, d = Xf.shape[-2], Xf.shape[-1]
        if d != self.model.d:
            raise ValueError(f"expected d={self.model.d}, got {d}")
        Xd = Xf.detach().reshape(-1, q, d).to(self.device, torch.float64).contiguous()
        b = Xd.shape[0]
        if self.use_cuda_graphs and b > 0:
            value, grad = self.graphed_value_and_grad(Xd, need_grad)
            value = value.clone()  # the graph's buffers are overwritten by the next replay
            grad = grad.clone() if grad is not None else None
        else:
            value, grad = self.value_and_grad_raw(Xd, need_grad)
        value = value.reshape(batch_shape).to(X.dtype)
        if grad is not None:
            grad = grad[:, : X.shape[-2], :]  # pending points (appended last) carry no gradient
            grad = grad.reshape(X.shape).to(X.dtype)
        return value, grad

    def value_and_grad_raw(self, Xd: Tensor, need_grad: bool, check: bool | None = None,
                           out: tuple | None = None, ws: "nat.Workspace | None" = None):
        """Native call on a contiguous float64 ``b x q x d`` device tensor.

        With the status check on (``check``, default ``self.check_status``), a
        t-batch whose sampling failed raises NotPSDError / NanError, after the
        fallback of ``_fall_back`` where the acquisition function has one.
        """
        b, q, d = Xd.shape
        if b == 0:
            empty = torch.empty(0, dtype=torch.float64, device=self.device)
            return empty, (torch.empty(0, q, d, dtype=torch.float64, device=self.device) if need_grad else None)
        acq, ws_bytes = self._call_struct(q)
        value, grad, status = self._native_call(Xd, need_grad, acq, ws_bytes, out, ws)
        if (self.check_status if check is None else check):
            value, grad = self._checked(Xd, need_grad, value, grad, status)
        return value, grad

    def _checked(self, Xd: Tensor, need_grad: bool, value: Tensor, grad, status: Tensor):
        """Raise for failed t-batches, or return the fallback's results."""
        worst = int(status.max().item()) if status.numel() > 0 else 0
        if worst in (nat.BGB_NOT_PSD, nat.BGB_NAN):
            fb = self._fall_back(Xd, need_grad)
            if fb is not None:
                value, grad, status = fb
        self._raise_for_status(status)
        return value, grad

    def _fall_back(self, Xd: Tensor, need_grad: bool):
        """(value, grad, status) of another sampling route after a failed call, or None."""
        return None

    def _native_call(self, Xd: Tensor, need_grad: bool, acq, ws_bytes: dict, out=None, ws=None):
        lib = nat.lib()
        b, q, d = Xd.shape
        if out is None:
            value = torch.empty(b, dtype=torch.float64, device=self.device)
            grad = torch.empty(b, q, d, dtype=torch.float64, device=self.device) if need_grad else None
            status = torch.empty(b, dtype=torch.int32, device=self.device)
        else:
            value, grad, status = out
        if b not in ws_bytes:
            ws_bytes[b] = lib.bgb_acq_workspace_bytes(ctypes.byref(acq), b)
        wt = (ws or self._ws).tensor(ws_bytes[b])
        packed = nat.struct_bytes(acq)
        if need_grad:
            rc = nat.ops().acq_forward_backward(packed, Xd, value, grad, status, wt)
        else:
            rc = nat.ops().acq_forward(packed, Xd, value, status, wt)
        nat.check(rc, type(self).__name__)
        return value, grad, status

    @staticmethod
    def _raise_for_status(status: Tensor) -> None:
        worst = int(status.max().item()) if status.numel() > 0 else 0
        if worst == nat.BGB_NOT_PSD:
            raise NotPSDError("q x q posterior covariance not positive definite after jitter")
        if worst == nat.BGB_NAN:
            raise NanError("Samples contain nans or infs.")
        if worst == nat.BGB_DEVICE_TIMEOUT:
            raise RuntimeError("a bounded wait in a tensor-core GEMM expired")

    def graphed_value_and_grad(self, Xd: Tensor, need_grad: bool = True,
                               check: bool | None = None) -> tuple[Tensor, Tensor | None]:
        """``value_and_grad_raw`` replayed from a CUDA graph.

        The first call for a (b, q, need_grad) shape runs the call once to set up
        the library's state, then captures it into a CUDA graph with its own
        input, output and workspace buffers; later calls copy ``Xd`` into the
        captured input and replay the graph (one launch for the whole call).
        The returned tensors are the graph's output buffers: the next replay for
        the same shape overwrites them. A new baseline or pending points give new
        base samples and a new capture.
        """
        b, q, d = Xd.shape
        key = (b, q, bool(need_grad), bool(self.use_tensor_cores), int(self.adjoint_ctas_per_sm))
        entry = self._graphs.get(key)
        acq, _ = self._call_struct(q)
        if entry is not None and entry["acq"] is not acq:
            entry = None  # the call struct changed: capture again
        if entry is None:
            dev = self.device
            Xs = Xd.detach().clone()
            out = (torch.empty(b, dtype=torch.float64, device=dev),
                   torch.empty(b, q, d, dtype=torch.float64, device=dev) if need_grad else None,
                   torch.empty(b, dtype=torch.int32, device=dev))
            ws = nat.Workspace(dev)
            side = torch.cuda.Stream(dev)
            side.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(side):
                self.value_and_grad_raw(Xs, need_grad, check=False, out=out, ws=ws)
            torch.cuda.current_stream(dev).wait_stream(side)
            torch.cuda.synchronize(dev)
            lib = nat.lib()
            graph = torch.cuda.CUDAGraph()
            n0 = lib.bgb_launch_count()
            with torch.cuda.graph(graph):
                self.value_and_grad_raw(Xs, need_grad, check=False, out=out, ws=ws)
            # keep the base samples the captured struct points to alive with the graph
            entry = dict(graph=graph, X=Xs, out=out, ws=ws, acq=acq, Z=self._Z.get(q),
                         launches=lib.bgb_launch_count() - n0)
            self._graphs[key] = entry
        entry["X"].copy_(Xd)
        entry["graph"].replay()
        value, grad, status = entry["out"]
        if (self.check_status if check is None else check):
            value, grad = self._checked(Xd, need_grad, value, grad, status)
        return value, grad

    def graph_launches(self, b: int, q: int, need_grad: bool = True) -> int:
        """Kernel launches of this library inside the captured graph for one shape."""
        entry = self._graphs.get((b, q, bool(need_grad), bool(self.use_tensor_cores),
                                  int(self.adjoint_ctas_per_sm)))
        return 0 if entry is None else int(entry["launches"])

    def _call_struct(self, q: int, flags: int = 0):
        """The call struct for q points, rebuilt only when its base samples change
        (a new baseline or pending points) or the GEMM form is switched. ``flags``:
        extra BGB_FLAG_* bits (the sampling route)."""
        key = (q, bool(self.use_tensor_cores), int(self.adjoint_ctas_per_sm), flags)
        hit = self._structs.get(key)
        if hit is None or hit[1] is not self._Z.get(q):
            acq = self._acq_struct(q)
            acq.flags |= (int(self.adjoint_ctas_per_sm) << nat.BGB_FLAG_ADJ_CTAS_SHIFT) & nat.BGB_FLAG_ADJ_CTAS_MASK
            acq.flags |= flags
            if flags & nat.BGB_FLAG_JOINT_SAMPLING:
                self._set_joint_operands(acq)
            hit = (acq, self._Z.get(q), {})
            self._structs[key] = hit
        return hit[0], hit[2]

    def _set_joint_operands(self, acq: nat.BgbAcq) -> None:
        raise UnsupportedError("joint sampling needs a baseline")

    def _device_Z(self, q: int) -> Tensor:
        if q not in self._Z:
            self._Z[q] = self._base_samples(q).to(self.device, torch.float64).contiguous()
        return self._Z[q]


class qExpectedImprovement(_MCAcquisition):
    """MC-based batch Expected Improvement (botorch/acquisition/monte_carlo.py:374-437).

    qEI(X) = mean_s max_q (Y_s - best_f)_+ with Y_s = mu + chol(Sigma) z_s.
    """

    acqf_id = nat.ACQF_QEI

    def __init__(self, model: SingleTaskGP, best_f: float | Tensor,
                 sampler: SobolQMCNormalSampler | None = None, objective=None,
                 posterior_transform=None, X_pending: Tensor | None = None, constraints=None,
                 eta: float = 1e-3, precision: str = "mixed") -> None:
        super().__init__(model, sampler, objective, posterior_transform, constraints, precision)
        # torch.as_tensor without a dtype, as the reference's register_buffer
        # (monte_carlo.py:420): a Python float becomes a tensor of the default
        # dtype first, and that value is what the improvement is measured from.
        bf = torch.as_tensor(best_f)
        if bf.numel() != 1:
            raise UnsupportedError("a scalar best_f is supported")
        self.best_f = bf.reshape(())
        self._best_f_dev = bf.reshape(1).to(self.device, torch.float64)
        self.set_X_pending(X_pending)

    def set_X_pending(self, X_pending: Tensor | None = None) -> None:
        self.X_pending = None if X_pending is None else X_pending.detach().clone()

    def _prepare_X(self, X: Tensor) -> Tensor:
        if self.X_pending is None:
            return X
        Xp = self.X_pending.to(X).expand(*X.shape[:-2], *self.X_pending.shape)
        return torch.cat([X, Xp], dim=-2)

    def _base_samples(self, q: int) -> Tensor:
        if self.sampler is None:
            self.sampler = SobolQMCNormalSampler(torch.Size([512]))
        return self.sampler.base_samples(q)

    def _acq_struct(self, q: int) -> nat.BgbAcq:
        m = self.model
        Z = self._device_Z(q)
        return nat.BgbAcq(acqf=nat.ACQF_QEI, q=q, r=0, n_samples=Z.shape[0], Z=nat.ptr(Z),
                          best_f=nat.ptr(self._best_f_dev), tau_relu=TAU_RELU, tau_max=TAU_MAX,
                          **m.acq_struct_base(self.precision, self.use_tensor_cores))


def prune_inferior_points(model: SingleTaskGP, X: Tensor, num_samples: int = 2048,
                          max_frac: float = 1.0, sampler: SobolQMCNormalSampler | None = None) -> Tensor:
    """Points of X that are the sampled argmax at least once (acquisition/utils.py:347-437).

    The posterior, its psd_safe_cholesky, the samples and the argmax counts
    run in the CUDA library; the sampler seed comes from the global torch RNG
    when no sampler is given, as in the reference.
    """
    if X.dim() != 2:
        raise UnsupportedError("Batched inputs `X` are currently unsupported by `prune_inferior_points`")
    if X.shape[-2] == 0:
        raise ValueError("X must have at least one point.")
    if max_frac <= 0 or max_frac > 1.0:
        raise ValueError(f"max_frac must take values in (0, 1], is {max_frac}")
    max_points = math.ceil(max_frac * X.shape[-2])
    m = X.shape[0]
    if sampler is None:
        sampler = SobolQMCNormalSampler(torch.Size([num_samples]))
    Z = sampler.base_samples(m).to(model.device).contiguous()
    Xd = X.detach().to(model.device, torch.float64).contiguous()
    counts = torch.empty(m, dtype=torch.int32, device=model.device)
    lib = nat.lib()
    ws = nat.Workspace(model.device)
    wp, wb = ws.get(lib.bgb_prune_counts_workspace_bytes(model.n, m, sampler.num_samples))
    gp = model.gp_struct()
    with torch.cuda.device(model.device):
        rc = lib.bgb_prune_counts(ctypes.byref(gp), nat.ptr(model.Linv), nat.ptr(model.alpha),
                                  nat.ptr(Xd), m, nat.ptr(Z), sampler.num_samples, 6,
                                  nat.ptr(counts), wp, wb, nat.stream_handle(model.device))
    nat.check(rc, "prune_inferior_points")
    counts = counts.cpu()
    idcs = torch.nonzero(counts > 0).squeeze(-1)
    if len(idcs) > max_points:
        # the reference's ordering step (acquisition/utils.py:432-434)
        sel_counts, order_idcs = torch.sort(counts[idcs], stable=True, descending=True)
        idcs = order_idcs[:max_points]
    return X[idcs.to(X.device)]


class qLogNoisyExpectedImprovement(_MCAcquisition):
    """MC-based batch Log Noisy Expected Improvement with cached root (logei.py:246-565)."""

    acqf_id = nat.ACQF_QLOGNEI

    def __init__(self, model: SingleTaskGP, X_baseline: Tensor,
                 sampler: SobolQMCNormalSampler | None = None, objective=None,
                 posterior_transform=None, X_pending: Tensor | None = None, constraints=None,
                 eta: float = 1e-3, fat: bool = True, prune_baseline: bool = True,
                 cache_root: bool | None = None, tau_max: float = TAU_MAX,
                 tau_relu: float = TAU_RELU, marginalize_dim: int | None = None,
                 incremental: bool = True, precision: str = "mixed") -> None:
        super().__init__(model, sampler, objective, posterior_transform, constraints, precision)
        if not fat:
            raise UnsupportedError("fat=False (logsumexp q-reduction) is not supported on this path")
        # cache_root=False: every call samples the joint (r+q)-dim posterior and takes
        # the incumbent from its own baseline samples (logei.py:543-553)
        self.cache_root = cache_root is not False
        if not incremental:
            raise UnsupportedError("incremental=False is not supported on this path")
        if not (tau_max > 0 and tau_relu > 0):
            raise ValueError("tau_max and tau_relu must be positive")
        self.tau_max = float(tau_max)
        self.tau_relu = float(tau_relu)
        self.prune_baseline = prune_baseline
        self._init_baseline(X_baseline, X_pending)

    def _init_baseline(self, X_baseline: Tensor, X_pending: Tensor | None) -> None:
        m = self.model
        X_baseline = X_baseline.detach()
        if self.prune_baseline:
            X_baseline = prune_inferior_points(m, X_baseline)
        self._X_baseline = X_baseline
        full = X_baseline if X_pending is None else torch.cat([X_baseline, X_pending.detach().to(X_baseline)], dim=-2)
        self._full_X_baseline = full
        if self.sampler is None:
            self.sampler = SobolQMCNormalSampler(torch.Size([512]))
        r = full.shape[0]
        self.r = r
        S = self.sampler.num_samples
        dev = self.device
        self._Xb = full.to(dev, torch.float64).contiguous()
        Zb = self.sampler.base_samples(r)
        self._Zb = Zb
        self._Lb = torch.empty(r, r, dtype=torch.float64, device=dev)
        self._Lb_inv = torch.empty(r, r, dtype=torch.float64, device=dev)
        self._best_f = torch.empty(S, dtype=torch.float64, device=dev)
        Zb_dev = Zb.to(dev).contiguous()
        lib = nat.lib()
        ws = nat.Workspace(dev)
        wp, wb = ws.get(lib.bgb_qlognei_baseline_workspace_bytes(m.n, r, S))
        jit = ctypes.c_double(0.0)
        gp = m.gp_struct()
        with torch.cuda.device(dev):
            rc = lib.bgb_qlognei_baseline(ctypes.byref(gp), nat.ptr(m.Linv), nat.ptr(m.alpha),
                                          nat.ptr(self._Xb), r, nat.ptr(Zb_dev), S, 6,
                                          nat.ptr(self._Lb), nat.ptr(self._Lb_inv),
                                          nat.ptr(self._best_f), ctypes.byref(jit), wp, wb,
                                          nat.stream_handle(dev))
        nat.check(rc, "qLogNEI baseline")
        self.baseline_jitter = jit.value
        self._Vb64, self._Vb32, self._VbT64, self._VbT32 = m.baseline_operands(self._Xb, self.precision)
        self._joint = None  # per-level operands of joint sampling, built on first use
        self._Z = {}

    @property
    def X_baseline(self) -> Tensor:
        return self._full_X_baseline

    @property
    def best_f(self) -> Tensor:
        """Per-sample incumbent max over the baseline samples (acquisition/utils.py:137-141)."""
        return self._best_f

    def set_X_pending(self, X_pending: Tensor | None = None) -> None:
        """Pending points join the baseline (incremental qLogNEI, logei.py:470-499)."""
        if X_pending is None and self._full_X_baseline.shape[-2] == self._X_baseline.shape[-2]:
            return
        saved = self.prune_baseline
        self.prune_baseline = False
        try:
            self._init_baseline(self._X_baseline, X_pending)
        finally:
            self.prune_baseline = saved

    def _sampling_flags(self) -> int:
        if self.cache_root:
            return 0
        return nat.BGB_FLAG_JOINT_SAMPLING | nat.BGB_FLAG_UNCACHED_ROOT

    def _call_struct(self, q: int, flags: int | None = None):
        return super()._call_struct(q, self._sampling_flags() if flags is None else flags)

    def _set_joint_operands(self, acq: nat.BgbAcq) -> None:
        """Per-jitter-level inverse roots of the baseline covariance and incumbents
        (bgb_qlognei_joint_levels), computed once per baseline."""
        if self._joint is None:
            m, r, S, dev = self.model, self.r, self.sampler.num_samples, self.device
            Lb_inv_lv = torch.empty(nat.JOINT_LEVELS, r, r, dtype=torch.float64, device=dev)
            best_f_lv = torch.empty(nat.JOINT_LEVELS, S, dtype=torch.float64, device=dev)
            Zb_dev = self._Zb.to(dev, torch.float64).contiguous()
            lib = nat.lib()
            ws = nat.Workspace(dev)
            wp, wb = ws.get(lib.bgb_qlognei_joint_levels_workspace_bytes(m.n, r, S))
            gp = m.gp_struct()
            with torch.cuda.device(dev):
                rc = lib.bgb_qlognei_joint_levels(ctypes.byref(gp), nat.ptr(m.Linv), nat.ptr(m.alpha),
                                                  nat.ptr(self._Xb), r, nat.ptr(Zb_dev), S,
                                                  nat.ptr(Lb_inv_lv), nat.ptr(best_f_lv), wp, wb,
                                                  nat.stream_handle(dev))
            nat.check(rc, "qLogNEI joint sampling operands")
            self._joint = (Lb_inv_lv, best_f_lv)
        acq.Lb_inv_lv = nat.ptr(self._joint[0])
        acq.best_f_lv = nat.ptr(self._joint[1])

    def _fall_back(self, Xd: Tensor, need_grad: bool):
        """The reference's fallback (botorch/acquisition/cached_cholesky.py:143-158): when
        the low-rank update of the cached root fails for a t-batch of the call (NaN
        samples or a non-PSD Schur complement), the whole call is sampled again from
        the joint (r+q)-dim posterior with the cached incumbent, with a warning."""
        if not self.cache_root:
            return None
        warnings.warn("Low-rank cholesky updates failed due NaNs or due to an ill-conditioned "
                      "covariance matrix. Falling back to standard sampling.", BotorchWarning,
                      stacklevel=4)
        acq, ws_bytes = self._call_struct(Xd.shape[1], nat.BGB_FLAG_JOINT_SAMPLING)
        return self._native_call(Xd, need_grad, acq, ws_bytes)

    def _base_samples(self, q: int) -> Tensor:
        """S x (r+q): the (r+q)-dim draw with its first r columns replaced by the baseline draw."""
        full = draw_sobol_normal_samples(self.r + q, self.sampler.num_samples, self.sampler.seed)
        full[:, : self.r] = self._Zb
        return full

    def _acq_struct(self, q: int) -> nat.BgbAcq:
        m = self.model
        Z = self._device_Z(q)
        return nat.BgbAcq(acqf=nat.ACQF_QLOGNEI, q=q, r=self.r, n_samples=Z.shape[0],
                          Vb64=nat.ptr(self._Vb64), Vb32=nat.ptr(self._Vb32),
                          VbT64=nat.ptr(self._VbT64), VbT32=nat.ptr(self._VbT32),
                          X_baseline=nat.ptr(self._Xb), Lb_inv=nat.ptr(self._Lb_inv), Z=nat.ptr(Z),
                          best_f=nat.ptr(self._best_f), tau_relu=self.tau_relu, tau_max=self.tau_max,
                          **m.acq_struct_base(self.precision, self.use_tensor_cores))
