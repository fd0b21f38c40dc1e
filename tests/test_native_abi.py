"""The C ABI library loads and exports every symbol include/botorch_gb300.h declares (no GPU calls)."""

import ctypes
import re
from pathlib import Path

import pytest

from botorch_gb300 import _native

HEADER = Path(__file__).resolve().parents[1] / "include" / "botorch_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bgb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_functions():
    assert set(declared_functions()) == set(_native.exported_symbols())


def test_library_exports_every_declared_symbol():
    if not _native.lib_path().exists():
        from botorch_gb300.build import build
        build()
    lib = _native.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.bgb_version() >= 100


def test_struct_layouts_match_the_header(tmp_path):
    """ctypes mirrors of bgb_gp_t / bgb_acq_t have the C compiler's layout."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in _native.BgbAcq._fields_]
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "botorch_gb300.h"\n'
        "int main(void) {\n"
        '  printf("%zu %zu\\n", sizeof(bgb_gp_t), sizeof(bgb_acq_t));\n'
        + "".join(f'  printf("%zu\\n", offsetof(bgb_acq_t, {f}));\n' for f in fields)
        + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(_native.BgbGP)
    assert int(out[1]) == ctypes.sizeof(_native.BgbAcq)
    for f, off in zip(fields, out[2:]):
        assert getattr(_native.BgbAcq, f).offset == int(off), f


def test_workspace_queries_need_no_gpu():
    lib = _native.lib()
    n = 4096
    assert lib.bgb_gp_fit_workspace_bytes(n) >= n * n * 8
    gp = _native.BgbGP(n=n, d=20, kernel=0, outputscale=1.0, mean_constant=0.0, y_mean=0.0,
                       y_std=1.0, train_X=1, inv_lengthscale=1)
    acq = _native.BgbAcq(gp=gp, acqf=1, precision=1, q=8, r=2, n_samples=512, ldb=n + 8)
    ws = lib.bgb_acq_workspace_bytes(ctypes.byref(acq), 4096)
    assert ws >= 4096 * 8 * n * 4 * 2


def test_invalid_arguments_are_rejected_without_touching_the_device():
    lib = _native.lib()
    assert lib.bgb_kernel_matrix(None, None, 0, None, 0, 0.0, None, 0, None) == _native.BGB_ERR_ARG
    acq = _native.BgbAcq()
    assert lib.bgb_acq_forward(ctypes.byref(acq), None, 1, None, None, None, 0, None) == _native.BGB_ERR_ARG


def test_product_requires_cuda():
    import torch

    from botorch_gb300 import SingleTaskGP, UnsupportedError

    if torch.cuda.is_available():
        pytest.skip("CPU-only check")
    with pytest.raises((UnsupportedError, RuntimeError, AssertionError)):
        SingleTaskGP(torch.rand(4, 2, dtype=torch.float64), torch.rand(4, 1, dtype=torch.float64),
                     device="cpu")


def test_header_constants_match_the_bindings():
    """Return codes and sizes defined in the header equal their Python mirrors."""
    text = HEADER.read_text()
    defs = dict(re.findall(r"#define (BGB_[A-Z0-9_]+)\s+(\S[^/\n]*?)\s*(?:/\*.*)?$", text, flags=re.M))
    for name in ("BGB_OK", "BGB_NOT_PSD", "BGB_NAN", "BGB_DEVICE_TIMEOUT", "BGB_ERR_ARG",
                 "BGB_ERR_WORKSPACE", "BGB_ERR_CUDA", "BGB_ERR_UNSUPPORTED", "BGB_ERR_SCRATCH_LIMIT",
                 "BGB_FLAG_SIMT", "BGB_FLAG_ADJ_CTAS_SHIFT", "BGB_FLAG_ADJ_CTAS_MASK",
                 "BGB_FLAG_JOINT_SAMPLING", "BGB_FLAG_UNCACHED_ROOT"):
        assert int(eval(defs[name])) == getattr(_native, name), name
    assert eval(defs["BGB_NOALLOC_SCRATCH_BYTES"].replace("(size_t)", "")) == _native.BGB_NOALLOC_SCRATCH_BYTES


def test_lbfgsb_options_layout_and_queries(tmp_path):
    """bgb_lbfgsb_opts has the C compiler's layout; the size query and the argument
    checks need no GPU."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in _native.BgbLbfgsbOpts._fields_]
    src = tmp_path / "lb.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "botorch_gb300.h"\n'
        "int main(void) {\n"
        '  printf("%zu\\n", sizeof(bgb_lbfgsb_opts));\n'
        + "".join(f'  printf("%zu\\n", offsetof(bgb_lbfgsb_opts, {f}));\n' for f in fields)
        + '  printf("%d %d %d\\n", BGB_LBFGSB_CONV_PGTOL, BGB_LBFGSB_ABNORMAL, BGB_LBFGSB_NONFINITE);\n'
        + "  return 0;\n}\n")
    exe = tmp_path / "lb"
    subprocess.run([cc, "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(_native.BgbLbfgsbOpts)
    for f, off in zip(fields, out[1:1 + len(fields)]):
        assert getattr(_native.BgbLbfgsbOpts, f).offset == int(off), f
    codes = [int(v) for v in out[1 + len(fields):]]
    assert [_native.BGB_LBFGSB_MESSAGES[c].split(":")[0] for c in codes] == ["CONVERGENCE", "ABNORMAL", "ERROR"]

    lib = _native.lib()
    opts = _native.BgbLbfgsbOpts(restarts=64, n=800, m=10, maxls=20, maxiter=100, maxfun=15000, factr=1e7,
                                 pgtol=1e-5)
    wsb = lib.bgb_lbfgsb_workspace_bytes(ctypes.byref(opts))
    assert wsb >= 64 * (2 * 10 * 800 + 7 * 800) * 8
    too_big = _native.BgbLbfgsbOpts(restarts=1, n=8193, m=10, maxls=20, maxiter=1, maxfun=1, factr=1e7, pgtol=0)
    assert lib.bgb_lbfgsb_workspace_bytes(ctypes.byref(too_big)) == 0
    assert lib.bgb_lbfgsb_init(ctypes.byref(too_big), 1, 1, 1, 1, 1 << 30, None) == _native.BGB_ERR_UNSUPPORTED
    bad = _native.BgbLbfgsbOpts(restarts=1, n=4, m=0, maxls=20, maxiter=1, maxfun=1, factr=1e7, pgtol=0)
    assert lib.bgb_lbfgsb_step(ctypes.byref(bad), 1, 1, 1.0, 1, None, 0, 1, 1 << 30, None, None) == \
        _native.BGB_ERR_ARG
    assert lib.bgb_lbfgsb_init(ctypes.byref(opts), None, 1, 1, 1, wsb, None) == _native.BGB_ERR_ARG
    assert lib.bgb_lbfgsb_init(ctypes.byref(opts), 1, 1, 1, 1, wsb - 1, None) == _native.BGB_ERR_WORKSPACE


def test_torch_extension_registers_the_operators():
    """The thin torch extension loads and registers the hot path's operators with
    their schemas; with no CPU kernel registered, CPU tensors raise in the dispatcher."""
    import torch

    if not _native.ext_path().exists():
        from botorch_gb300.build import build
        build()
    ops = _native.ops()
    schemas = {n: str(getattr(ops, n).default._schema) for n in
               ("acq_forward_backward", "acq_forward", "log_areas_forward", "log_areas_backward")}
    assert schemas["acq_forward_backward"].startswith("botorch_gb300::acq_forward_backward(Tensor acq, Tensor X, "
                                                      "Tensor(a!) value, Tensor(b!) grad, Tensor(c!) status")
    assert schemas["log_areas_forward"] == ("botorch_gb300::log_areas_forward(Tensor obj_subsets, Tensor cell_lower, "
                                            "Tensor cell_upper, float tau_relu, float tau_max) -> Tensor")
    assert "-> Tensor" in schemas["log_areas_backward"] and "-> int" in schemas["acq_forward"]
    with pytest.raises(NotImplementedError):
        ops.log_areas_forward(torch.zeros(1, 1, 1, 1), torch.zeros(1, 1), torch.ones(1, 1), 1e-6, 1e-2)
    acq = _native.BgbAcq(q=2)
    packed = _native.struct_bytes(acq)
    assert packed.numel() == ctypes.sizeof(_native.BgbAcq) and int(packed[ctypes.sizeof(_native.BgbGP) + 8]) == 2
