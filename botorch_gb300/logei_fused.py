"""Fused log-areas of qLogEHVI / qLogNEHVI on the GPU.

Drop-in for the reference's fused CPU extension (the module-level ``_C`` of
botorch/acquisition/multi_objective/logei.py:59-104, built from
botorch/csrc/logei_fused.cpp): ``forward`` and ``backward`` take the same
arguments, check them the same way and return the same shapes, for CUDA
tensors. ``FusedLogAreas`` mirrors the reference's ``_FusedLogAreas``
autograd function (logei.py:107-165).

    forward(obj_subsets, cell_lower, cell_upper, tau_relu, tau_max)
        obj_subsets (B, n_sub, i, m), cells (nc, m) or (B, nc, m) -> (B, nc, n_sub)
    backward(grad_output, obj_subsets, cell_lower, cell_upper, tau_relu, tau_max)
        -> gradient w.r.t. obj_subsets, (B, n_sub, i, m)

float64 and float32 inputs compute in their own type, as the reference's
AT_DISPATCH_FLOATING_TYPES. ``forward`` and ``backward`` run through the
library's torch operators (``torch.ops.botorch_gb300.log_areas_forward`` /
``log_areas_backward``, registered for CUDA only). There is no CPU path: CPU
tensors raise.

``FusedLogAreas`` differs from the reference in one respect: when the input
needs a gradient and the Jacobian fits ``JACOBIAN_BUDGET_BYTES``, its forward
also keeps d area / d obj (``forward_with_jacobian``) and its backward is
the contraction of grad_output with it (``backward_from_jacobian``), instead
of recomputing the forward quantities. On GB300 the recomputation is bound
by the float64 pipe while the Jacobian costs 8 i m bytes of HBM per area.
"""

from __future__ import annotations

import torch
from torch import Tensor

from botorch_gb300 import _native as nat

MAX_I = 32  # largest subset size (the reference's _FUSED_MAX_I / MAX_I)
MAX_M = 8   # largest number of objectives (the reference's MAX_M)
JACOBIAN_BUDGET_BYTES = 8 << 30  # largest Jacobian FusedLogAreas keeps for its backward


def _prepare(obj_subsets: Tensor, cell_lower: Tensor, cell_upper: Tensor):
    obj = obj_subsets.contiguous()
    cl = cell_lower.contiguous()
    cu = cell_upper.contiguous()
    if obj.dim() != 4:
        raise RuntimeError("obj_subsets must be 4-D")
    if not ((cl.dim() == 2 or cl.dim() == 3) and cl.dim() == cu.dim()):
        raise RuntimeError("cell bounds must be 2-D or 3-D")
    B, n_sub, isz, m = obj.shape
    if isz > MAX_I or m > MAX_M:
        raise RuntimeError("subset_size or m too large")
    if obj.dtype not in (torch.float64, torch.float32):
        raise RuntimeError(f"fused log-areas: unsupported dtype {obj.dtype}")
    if obj.device.type != "cuda":
        raise RuntimeError("fused log-areas: the inputs must be CUDA tensors (no CPU path)")
    if cl.dtype != obj.dtype or cu.dtype != obj.dtype or cl.device != obj.device or cu.device != obj.device:
        raise RuntimeError("fused log-areas: cell bounds must match obj_subsets in dtype and device")
    if cl.shape != cu.shape or cl.shape[-1] != m:
        raise RuntimeError("fused log-areas: cell bounds must be (..., num_cells, m) and of equal shape")
    B_cells = cl.shape[0] if cl.dim() == 3 else 1
    nc = cl.shape[-2]
    if cl.dim() == 3 and B_cells != B:
        raise RuntimeError("fused log-areas: batched cell bounds need one batch per obj_subsets batch")
    return obj, cl, cu, (B, n_sub, isz, m, B_cells, nc)


def forward(obj_subsets: Tensor, cell_lower: Tensor, cell_upper: Tensor, tau_relu: float,
            tau_max: float) -> Tensor:
    """Log areas (B, nc, n_sub) of every cell and q-subset (logei_fused.cpp:184-264)."""
    obj, cl, cu, _ = _prepare(obj_subsets, cell_lower, cell_upper)
    return nat.ops().log_areas_forward(obj, cl, cu, float(tau_relu), float(tau_max))


def backward(grad_output: Tensor, obj_subsets: Tensor, cell_lower: Tensor, cell_upper: Tensor,
             tau_relu: float, tau_max: float) -> Tensor:
    """Gradient of sum(grad_output * forward(...)) w.r.t. obj_subsets (logei_fused.cpp:266-374)."""
    obj, cl, cu, (B, n_sub, isz, m, B_cells, nc) = _prepare(obj_subsets, cell_lower, cell_upper)
    go = grad_output.contiguous()
    if tuple(go.shape) != (B, nc, n_sub) or go.dtype != obj.dtype or go.device != obj.device:
        raise RuntimeError("fused log-areas: grad_output must be (B, num_cells, n_sub) like the forward output")
    return nat.ops().log_areas_backward(go, obj, cl, cu, float(tau_relu), float(tau_max))


def forward_with_jacobian(obj_subsets: Tensor, cell_lower: Tensor, cell_upper: Tensor, tau_relu: float,
                          tau_max: float) -> tuple[Tensor, Tensor]:
    """``forward`` plus the Jacobian (B, nc, n_sub, i, m) of every area with respect to
    its subset's objective values."""
    obj, cl, cu, (B, n_sub, isz, m, B_cells, nc) = _prepare(obj_subsets, cell_lower, cell_upper)
    out = torch.empty(B, nc, n_sub, dtype=obj.dtype, device=obj.device)
    jac = torch.empty(B, nc, n_sub, isz, m, dtype=obj.dtype, device=obj.device)
    fn = (nat.lib().bgb_log_areas_forward_jac if obj.dtype == torch.float64
          else nat.lib().bgb_log_areas_forward_jac_f32)
    with torch.cuda.device(obj.device):
        rc = fn(obj.data_ptr(), B, n_sub, isz, m, cl.data_ptr(), cu.data_ptr(), B_cells, nc,
                float(tau_relu), float(tau_max), out.data_ptr(), jac.data_ptr(),
                nat.stream_handle(obj.device))
    nat.check(rc, "bgb_log_areas_forward_jac")
    return out, jac


def backward_from_jacobian(grad_output: Tensor, jac: Tensor) -> Tensor:
    """Gradient w.r.t. obj_subsets (B, n_sub, i, m) from the Jacobian of
    ``forward_with_jacobian``: sum over cells of grad_output x Jacobian."""
    if jac.dim() != 5:
        raise RuntimeError("fused log-areas: the Jacobian must be (B, num_cells, n_sub, i, m)")
    B, nc, n_sub, isz, m = jac.shape
    go = grad_output.contiguous()
    if tuple(go.shape) != (B, nc, n_sub) or go.dtype != jac.dtype or go.device != jac.device:
        raise RuntimeError("fused log-areas: grad_output must be (B, num_cells, n_sub) like the forward output")
    jac = jac.contiguous()
    g_obj = torch.empty(B, n_sub, isz, m, dtype=jac.dtype, device=jac.device)
    fn = (nat.lib().bgb_log_areas_backward_jac if jac.dtype == torch.float64
          else nat.lib().bgb_log_areas_backward_jac_f32)
    with torch.cuda.device(jac.device):
        rc = fn(go.data_ptr(), jac.data_ptr(), B, n_sub, isz, m, nc, g_obj.data_ptr(),
                nat.stream_handle(jac.device))
    nat.check(rc, "bgb_log_areas_backward_jac")
    return g_obj


class FusedLogAreas(torch.autograd.Function):
    """Autograd wrapper with the reference's ``_FusedLogAreas`` contract:
    ``obj_subsets`` (*batch, n_sub, i, m) and cell bounds (nc, m) or
    (*batch, nc, m) -> (*batch, nc, n_sub); only ``obj_subsets`` gets a gradient."""

    @staticmethod
    def forward(ctx, obj_subsets: Tensor, cell_lower: Tensor, cell_upper: Tensor, tau_relu: float,
                tau_max: float) -> Tensor:
        batch_shape = obj_subsets.shape[:-3]
        B = max(1, int(torch.Size(batch_shape).numel()))
        obj_flat = obj_subsets.reshape(B, *obj_subsets.shape[-3:])
        nc, m_cells = cell_lower.shape[-2], cell_lower.shape[-1]
        if cell_lower.ndim > 2:
            cell_lower = cell_lower.reshape(-1, nc, m_cells)
            cell_upper = cell_upper.reshape(-1, nc, m_cells)
        n_sub, isz, m = obj_flat.shape[-3:]
        jac_bytes = B * nc * n_sub * isz * m * obj_flat.element_size()
        if ctx.needs_input_grad[0] and jac_bytes <= JACOBIAN_BUDGET_BYTES:
            result, jac = forward_with_jacobian(obj_flat, cell_lower, cell_upper, tau_relu, tau_max)
            ctx.save_for_backward(jac)
            ctx.with_jacobian = True
        else:
            result = forward(obj_flat, cell_lower, cell_upper, tau_relu, tau_max)
            ctx.save_for_backward(obj_flat, cell_lower, cell_upper)
            ctx.with_jacobian = False
        ctx.tau_relu = tau_relu
        ctx.tau_max = tau_max
        ctx.orig_shape = obj_subsets.shape
        return result.reshape(*batch_shape, result.shape[-2], result.shape[-1])

    @staticmethod
    def backward(ctx, grad_output: Tensor):
        if ctx.with_jacobian:
            (jac,) = ctx.saved_tensors
            grad_flat = grad_output.reshape(jac.shape[0], *grad_output.shape[-2:])
            grad_obj = backward_from_jacobian(grad_flat, jac)
            return grad_obj.reshape(ctx.orig_shape), None, None, None, None
        obj_flat, cell_lower, cell_upper = ctx.saved_tensors
        B = obj_flat.shape[0]
        grad_flat = grad_output.reshape(B, *grad_output.shape[-2:])
        grad_obj = backward(grad_flat, obj_flat, cell_lower, cell_upper, ctx.tau_relu, ctx.tau_max)
        return grad_obj.reshape(ctx.orig_shape), None, None, None, None
