"""ORACLE (test infrastructure; also the CPU baseline of the fused log-areas
benchmark): ctypes front end of ``oracle/log_areas.c``, the plain-C
restatement of botorch/csrc/logei_fused.cpp:184-374.

``forward`` / ``backward`` take CPU tensors with the reference extension's
argument order and shapes. ``threads`` > 1 splits the (b, subset) range
over host threads the way the reference's ``at::parallel_for`` does
(ctypes releases the GIL during each call).
"""

from __future__ import annotations

import ctypes
from concurrent.futures import ThreadPoolExecutor

import torch
from torch import Tensor

from oracle.build import build_oracle

_lib = None
_vp, _i64, _f64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double


def lib():
    global _lib
    if _lib is None:
        h = ctypes.CDLL(str(build_oracle()))
        for suf in ("f64", "f32"):
            f = getattr(h, f"oracle_log_areas_forward_{suf}")
            f.restype = None
            f.argtypes = [_vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64, _i64, _f64, _f64, _vp, _i64, _i64]
            g = getattr(h, f"oracle_log_areas_backward_{suf}")
            g.restype = None
            g.argtypes = [_vp, _vp, _i64, _i64, _i64, _i64, _vp, _vp, _i64, _i64, _f64, _f64, _vp, _i64,
                          _i64]
        _lib = h
    return _lib


def _shapes(obj: Tensor, cl: Tensor):
    B, n_sub, isz, m = obj.shape
    B_cells = cl.shape[0] if cl.dim() == 3 else 1
    return B, n_sub, isz, m, B_cells, cl.shape[-2]


def _run(fn, total: int, threads: int) -> None:
    if threads <= 1 or total < 2:
        fn(0, total)
        return
    step = -(-total // threads)
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda lo: fn(lo, min(total, lo + step)), range(0, total, step)))


def forward(obj: Tensor, cell_lower: Tensor, cell_upper: Tensor, tau_relu: float, tau_max: float,
            threads: int = 1) -> Tensor:
    obj, cl, cu = obj.contiguous(), cell_lower.contiguous(), cell_upper.contiguous()
    B, n_sub, isz, m, B_cells, nc = _shapes(obj, cl)
    out = torch.empty(B, nc, n_sub, dtype=obj.dtype)
    f = getattr(lib(), "oracle_log_areas_forward_" + ("f64" if obj.dtype == torch.float64 else "f32"))
    _run(lambda lo, hi: f(obj.data_ptr(), B, n_sub, isz, m, cl.data_ptr(), cu.data_ptr(), B_cells, nc,
                          tau_relu, tau_max, out.data_ptr(), lo, hi), B * n_sub, threads)
    return out


def backward(grad_out: Tensor, obj: Tensor, cell_lower: Tensor, cell_upper: Tensor, tau_relu: float,
             tau_max: float, threads: int = 1) -> Tensor:
    go, obj = grad_out.contiguous(), obj.contiguous()
    cl, cu = cell_lower.contiguous(), cell_upper.contiguous()
    B, n_sub, isz, m, B_cells, nc = _shapes(obj, cl)
    g = torch.zeros_like(obj)
    f = getattr(lib(), "oracle_log_areas_backward_" + ("f64" if obj.dtype == torch.float64 else "f32"))
    _run(lambda lo, hi: f(go.data_ptr(), obj.data_ptr(), B, n_sub, isz, m, cl.data_ptr(), cu.data_ptr(),
                          B_cells, nc, tau_relu, tau_max, g.data_ptr(), lo, hi), B * n_sub, threads)
    return g


def python_path_log_areas(obj: Tensor, cell_lower: Tensor, cell_upper: Tensor, tau_relu: float,
                          tau_max: float) -> Tensor:
    """Steps 1-4 of the reference's unfused path (botorch/acquisition/multi_objective/
    logei.py:437-480 with fat=True): log_fatplus of obj - lower, fatmin over the
    subset, fatmin with the log cell lengths, sum over objectives. Torch, autograd
    through it gives the gradient. obj (B, n_sub, i, m), cells (nc, m) or (B, nc, m)
    -> (B, nc, n_sub)."""
    from oracle.safe_math import fatmax, log_fatplus

    def fatmin(x: Tensor, dim: int) -> Tensor:  # safe_math.py:358-381
        return -fatmax(-x, dim=dim, tau=tau_max)

    cl = cell_lower if cell_lower.dim() == 3 else cell_lower.unsqueeze(0)
    cu = cell_upper if cell_upper.dim() == 3 else cell_upper.unsqueeze(0)
    clamp = 1e10 if obj.dtype == torch.float64 else 1e8
    # (B, 1, n_sub, i, m) - (B or 1, nc, 1, 1, m)
    li = log_fatplus(obj.unsqueeze(1) - cl[:, :, None, None, :], tau=tau_relu)
    lim = fatmin(li, dim=-2)                                   # (B, nc, n_sub, m)
    lcl = (cu.clamp_max(clamp) - cl).log()[:, :, None, :]      # (B or 1, nc, 1, m)
    pair = torch.stack(torch.broadcast_tensors(lim, lcl), dim=-1)
    return fatmin(pair, dim=-1).sum(-1)
