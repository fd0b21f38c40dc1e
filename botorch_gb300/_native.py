"""ctypes binding of libbotorch_gb300.so (the C ABI in include/botorch_gb300.h).

The library is the only compute path of this package: there is no CPU or
PyTorch fallback. ``lib()`` raises ``NativeLibraryError`` when the library
was not built (``python -m botorch_gb300.build``) or cannot be loaded.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

import torch

from botorch_gb300.exceptions import NanError, NotPSDError

BGB_OK = 0
BGB_NOT_PSD = 1
BGB_NAN = 2
BGB_DEVICE_TIMEOUT = 3
BGB_FLAG_SIMT = 1
BGB_FLAG_ADJ_CTAS_SHIFT = 8
BGB_FLAG_ADJ_CTAS_MASK = 0xFF00
BGB_FLAG_JOINT_SAMPLING = 2     # joint (r+q) sampling, cached incumbent: the fallback path
BGB_FLAG_UNCACHED_ROOT = 4      # with JOINT_SAMPLING: cache_root=False
JOINT_LEVELS = 7                # psd_safe_cholesky: plain + 6 jitter levels
BGB_ERR_ARG = -1
BGB_ERR_WORKSPACE = -2
BGB_ERR_CUDA = -3
BGB_ERR_UNSUPPORTED = -4
BGB_ERR_SCRATCH_LIMIT = -5
BGB_NOALLOC_SCRATCH_BYTES = 32 << 20   # fixed scratch of bgb_acq_forward_backward_noalloc

KERNELS = {"matern52": 0, "matern32": 1, "matern12": 2, "rbf": 3}
PRECISIONS = {"fp64": 0, "mixed": 1}
ACQF_QEI = 0
ACQF_QLOGNEI = 1

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libbotorch_gb300.so"
_lib = None

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_f64 = ctypes.c_double
c_vp = ctypes.c_void_p
c_size = ctypes.c_size_t


class NativeLibraryError(RuntimeError):
    """The CUDA library is missing or failed to load."""


class BgbGP(ctypes.Structure):
    _fields_ = [("n", c_i64), ("d", c_i32), ("kernel", c_i32), ("outputscale", c_f64),
                ("mean_constant", c_f64), ("y_mean", c_f64), ("y_std", c_f64),
                ("train_X", c_vp), ("inv_lengthscale", c_vp)]


class BgbAcq(ctypes.Structure):
    _fields_ = [("gp", BgbGP), ("acqf", c_i32), ("precision", c_i32), ("q", c_i32), ("r", c_i32),
                ("n_samples", c_i32), ("flags", c_i32), ("ldb", c_i64), ("B64", c_vp),
                ("B32", c_vp), ("Linv64", c_vp), ("Linv32", c_vp), ("Vb64", c_vp), ("Vb32", c_vp),
                ("VbT64", c_vp), ("VbT32", c_vp), ("beta64", c_vp), ("beta32", c_vp),
                ("Xs64", c_vp), ("Xs32", c_vp),
                ("Lhi", c_vp), ("Llo", c_vp), ("LThi", c_vp), ("LTlo", c_vp), ("Lmul", c_vp),
                ("LTmul", c_vp), ("ldl", c_i64), ("beta_absmax", c_f64),
                ("X_baseline", c_vp), ("Lb_inv", c_vp),
                ("Z", c_vp), ("best_f", c_vp), ("tau_relu", c_f64), ("tau_max", c_f64),
                ("Lb_inv_lv", c_vp), ("best_f_lv", c_vp)]


class BgbLbfgsbOpts(ctypes.Structure):
    _fields_ = [("restarts", c_i64), ("n", c_i64), ("m", c_i32), ("maxls", c_i32),
                ("maxiter", c_i64), ("maxfun", c_i64), ("factr", c_f64), ("pgtol", c_f64)]


BGB_LBFGSB_MESSAGES = {
    0: "RUNNING",
    1: "CONVERGENCE: NORM OF PROJECTED GRADIENT <= PGTOL",
    2: "CONVERGENCE: RELATIVE REDUCTION OF F <= FACTR*EPSMCH",
    3: "ABNORMAL: ABNORMAL_TERMINATION_IN_LNSRCH",
    4: "STOP: TOTAL NO. OF ITERATIONS REACHED LIMIT",
    5: "STOP: TOTAL NO. OF F,G EVALUATIONS EXCEEDS LIMIT",
    6: "ERROR: NON-FINITE VALUE OR GRADIENT",
}


_SIGNATURES = {
    "bgb_version": (c_i32, []),
    "bgb_kernel_matrix": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_i64, c_vp, c_i64, c_f64, c_vp,
                                  c_i64, c_vp]),
    "bgb_cholesky": (c_i32, [c_vp, c_i64, c_i64, ctypes.POINTER(c_i32), c_vp, c_size, c_vp]),
    "bgb_cholesky_workspace_bytes": (c_size, [c_i64]),
    "bgb_psd_safe_cholesky": (c_i32, [c_vp, c_i64, c_i64, c_vp, c_i64, c_i32, c_f64,
                                      ctypes.POINTER(c_f64), c_vp, c_size, c_vp]),
    "bgb_tri_inverse": (c_i32, [c_vp, c_i64, c_i64, c_vp, c_size, c_vp]),
    "bgb_tri_inverse_workspace_bytes": (c_size, [c_i64]),
    "bgb_gp_fit": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_f64, c_i32, c_vp, c_vp, c_vp, c_vp,
                           ctypes.POINTER(c_f64), c_vp, c_size, c_vp]),
    "bgb_gp_fit_workspace_bytes": (c_size, [c_i64]),
    "bgb_gp_operands": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp,
                                c_vp, c_vp, c_vp]),
    "bgb_gp_mll": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_vp, c_vp,
                           ctypes.POINTER(ctypes.c_double), c_vp, c_size, c_vp]),
    "bgb_gp_mll_workspace_bytes": (c_size, [c_i64, c_i32]),
    "bgb_gp_tc_operands": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_i64, c_vp, c_vp, c_vp, c_vp,
                                   c_vp, c_vp, c_vp]),
    "bgb_crosscov_gemm_f16x3": (c_i32, [c_i64, c_i64, c_i64, c_vp, c_vp, c_i64, c_vp, c_vp, c_i64,
                                        c_vp, c_i64, c_vp, ctypes.c_float, c_vp, c_i32, c_vp,
                                        c_vp]),
    "bgb_baseline_operands": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_i32, c_vp, c_vp, c_vp,
                                      c_vp, c_vp, c_size, c_vp]),
    "bgb_baseline_operands_workspace_bytes": (c_size, [c_i64, c_i32]),
    "bgb_posterior_joint": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_vp, c_i64, c_vp, c_vp,
                                    c_vp, c_size, c_vp]),
    "bgb_posterior_joint_workspace_bytes": (c_size, [c_i64, c_i64]),
    "bgb_prune_counts": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_vp, c_i64, c_vp, c_i32,
                                 c_i32, c_vp, c_vp, c_size, c_vp]),
    "bgb_prune_counts_workspace_bytes": (c_size, [c_i64, c_i64, c_i32]),
    "bgb_qlognei_baseline": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_vp, c_i32, c_vp, c_i32,
                                     c_i32, c_vp, c_vp, c_vp, ctypes.POINTER(c_f64), c_vp, c_size,
                                     c_vp]),
    "bgb_qlognei_baseline_workspace_bytes": (c_size, [c_i64, c_i32, c_i32]),
    "bgb_qlognei_joint_levels": (c_i32, [ctypes.POINTER(BgbGP), c_vp, c_vp, c_vp, c_i32, c_vp,
                                         c_i32, c_vp, c_vp, c_vp, c_size, c_vp]),
    "bgb_qlognei_joint_levels_workspace_bytes": (c_size, [c_i64, c_i32, c_i32]),
    "bgb_posterior": (c_i32, [ctypes.POINTER(BgbAcq), c_vp, c_i64, c_vp, c_vp, c_vp, c_size,
                              c_vp]),
    "bgb_mvn_rsample": (c_i32, [c_vp, c_vp, c_i64, c_i32, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp]),
    "bgb_acq_workspace_bytes": (c_size, [ctypes.POINTER(BgbAcq), c_i64]),
    "bgb_acq_forward": (c_i32, [ctypes.POINTER(BgbAcq), c_vp, c_i64, c_vp, c_vp, c_vp, c_size,
                                c_vp]),
    "bgb_acq_forward_backward": (c_i32, [ctypes.POINTER(BgbAcq), c_vp, c_i64, c_vp, c_vp, c_vp,
                                         c_vp, c_size, c_vp]),
    "bgb_acq_forward_backward_timed": (c_i32, [ctypes.POINTER(BgbAcq), c_vp, c_i64, c_vp, c_vp,
                                               c_vp, c_vp, c_size, ctypes.POINTER(ctypes.c_float),
                                               c_vp]),
    "bgb_acq_forward_backward_noalloc": (c_i32, [ctypes.POINTER(BgbAcq), c_vp, c_i64, c_vp, c_vp,
                                                 c_vp, c_vp]),
    "bgb_group_workspace_bytes": (c_size, [ctypes.POINTER(BgbAcq), ctypes.POINTER(c_i64), c_i32]),
    "bgb_group_create": (c_i32, [ctypes.POINTER(BgbAcq), ctypes.POINTER(c_i64), c_i32,
                                 ctypes.POINTER(c_vp), ctypes.POINTER(c_vp), ctypes.POINTER(c_vp),
                                 ctypes.POINTER(c_vp), c_vp, c_size, c_vp, ctypes.POINTER(c_vp)]),
    "bgb_group_run": (c_i32, [c_vp, c_vp]),
    "bgb_group_launches": (c_i32, [c_vp]),
    "bgb_group_destroy": (None, [c_vp]),
    "bgb_lbfgsb_workspace_bytes": (c_size, [ctypes.POINTER(BgbLbfgsbOpts)]),
    "bgb_lbfgsb_init": (c_i32, [ctypes.POINTER(BgbLbfgsbOpts), c_vp, c_vp, c_vp, c_vp, c_size, c_vp]),
    "bgb_lbfgsb_step": (c_i32, [ctypes.POINTER(BgbLbfgsbOpts), c_vp, c_vp, c_f64, c_vp, c_vp, c_i32,
                                c_vp, c_size, c_vp, c_vp]),
    "bgb_lbfgsb_results": (c_i32, [ctypes.POINTER(BgbLbfgsbOpts), c_vp, c_size, c_vp, c_vp, c_vp,
                                   c_vp, c_vp]),
    "bgb_log_areas_forward": (c_i32, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_i64, c_i64,
                                      c_f64, c_f64, c_vp, c_vp]),
    "bgb_log_areas_forward_f32": (c_i32, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_i64,
                                          c_i64, c_f64, c_f64, c_vp, c_vp]),
    "bgb_log_areas_backward": (c_i32, [c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_i64,
                                       c_i64, c_f64, c_f64, c_vp, c_vp]),
    "bgb_log_areas_backward_f32": (c_i32, [c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp,
                                           c_i64, c_i64, c_f64, c_f64, c_vp, c_vp]),
    "bgb_log_areas_forward_jac": (c_i32, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_i64,
                                          c_i64, c_f64, c_f64, c_vp, c_vp, c_vp]),
    "bgb_log_areas_forward_jac_f32": (c_i32, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_i64,
                                              c_i64, c_f64, c_f64, c_vp, c_vp, c_vp]),
    "bgb_log_areas_backward_jac": (c_i32, [c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_vp,
                                           c_vp]),
    "bgb_log_areas_backward_jac_f32": (c_i32, [c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_vp,
                                               c_vp]),
    "bgb_sobol_box": (c_i32, [c_vp, c_vp, c_vp, c_i32, c_i32, c_i64, c_i64, c_vp, c_vp, c_i32, c_vp, c_vp]),
    "bgb_launch_count": (ctypes.c_ulonglong, []),
}


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def lib_path() -> Path:
    return _LIB_PATH


def lib():
    """Load (once) and return the CUDA library; raise if it is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise NativeLibraryError(
            f"{_LIB_PATH} is missing: build it with `python -m botorch_gb300.build` "
            "(botorch_gb300 has no CPU fallback).")
    try:
        handle = ctypes.CDLL(str(_LIB_PATH))
    except OSError as e:  # pragma: no cover - depends on the machine
        raise NativeLibraryError(f"cannot load {_LIB_PATH}: {e}") from e
    for name, (restype, argtypes) in _SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _lib = handle
    return handle


_ops = None


def ext_path() -> Path:
    return _LIB_PATH.parent / "libbotorch_gb300_torch.so"


def ops():
    """Load (once) the thin torch extension over the library and return its
    operators, ``torch.ops.botorch_gb300``: the acquisition's value (+ adjoint)
    call and the fused log-areas contract run through the dispatcher; raise if
    the extension is unavailable."""
    global _ops
    if _ops is not None:
        return _ops
    lib()  # the extension links against the library
    path = ext_path()
    if not path.exists():
        raise NativeLibraryError(
            f"{path} is missing: build it with `python -m botorch_gb300.build` "
            "(botorch_gb300 has no CPU fallback).")
    try:
        torch.ops.load_library(str(path))
    except OSError as e:  # pragma: no cover - depends on the machine
        raise NativeLibraryError(f"cannot load {path}: {e}") from e
    _ops = torch.ops.botorch_gb300
    return _ops


def struct_bytes(s: ctypes.Structure) -> torch.Tensor:
    """The bytes of a ctypes struct as a CPU uint8 tensor sharing its memory (the
    form in which the torch operators take a bgb_acq_t)."""
    return torch.frombuffer(s, dtype=torch.uint8)


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def check(rc: int, what: str) -> None:
    """Map a C ABI return code to the reference's exception types."""
    if rc == BGB_OK:
        return
    if rc == BGB_NOT_PSD:
        raise NotPSDError(f"{what}: matrix not positive definite after adding jitter")
    if rc == BGB_NAN:
        raise NanError(f"{what}: NaN encountered")
    names = {BGB_ERR_ARG: "invalid argument", BGB_ERR_WORKSPACE: "workspace too small",
             BGB_ERR_CUDA: "CUDA error", BGB_ERR_UNSUPPORTED: "unsupported size",
             BGB_ERR_SCRATCH_LIMIT: "needs more than the fixed no-allocation scratch"}
    raise RuntimeError(f"{what}: {names.get(rc, rc)} (code {rc})")


class Workspace:
    """Grow-only device scratch buffer handed to the C ABI calls."""

    def __init__(self, device: torch.device) -> None:
        self.device = device
        self.buf: torch.Tensor | None = None

    def get(self, nbytes: int) -> tuple[int, int]:
        t = self.tensor(nbytes)
        return t.data_ptr(), t.numel()

    def tensor(self, nbytes: int) -> torch.Tensor:
        nbytes = max(int(nbytes), 256)
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        return self.buf
