"""ORACLE build recipe (test infrastructure).

* ``build_oracle()``: the plain-C restatement ``oracle/log_areas.c`` ->
  ``oracle/_lib/liboracle_log_areas.so`` (gcc, no FMA contraction, so that
  the arithmetic is the same on x86-64 and aarch64 hosts).
* ``build_reference(root)``: the reference's own fused CPU kernel,
  ``botorch/csrc/logei_fused.cpp``, compiled from where it lies in the
  reference checkout whose root is ``root`` (or the environment variable
  ``BOTORCH_REFERENCE_ROOT``) as the reference loads it (a torch C++
  extension, botorch/acquisition/multi_objective/logei.py:85-94), with its
  output only in ``oracle/_ref/``. Without a checkout it imports the module
  an earlier build left in ``oracle/_ref/``, else returns None. Used to pin
  the restatement and to write the golden fixtures in ``tests/golden/``.
"""

from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
LIB_DIR = ORACLE / "_lib"
REF_DIR = ORACLE / "_ref"
REFERENCE_KERNEL = Path("botorch") / "csrc" / "logei_fused.cpp"  # within the reference checkout
REF_MODULE = "logei_fused_ref"
ORACLE_LIB = LIB_DIR / "liboracle_log_areas.so"


def build_oracle(force: bool = False) -> Path:
    src = ORACLE / "log_areas.c"
    if not force and ORACLE_LIB.exists() and ORACLE_LIB.stat().st_mtime >= src.stat().st_mtime:
        return ORACLE_LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("a C compiler (gcc) is required to build the oracle")
    LIB_DIR.mkdir(exist_ok=True)
    cmd = [cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c99", str(src), "-lm",
           "-o", str(ORACLE_LIB)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return ORACLE_LIB


def reference_source(root: str | os.PathLike | None = None) -> Path | None:
    """The reference kernel's source under ``root`` (or $BOTORCH_REFERENCE_ROOT), if present."""
    root = root if root is not None else os.environ.get("BOTORCH_REFERENCE_ROOT")
    if not root:
        return None
    src = Path(root) / REFERENCE_KERNEL
    return src if src.exists() else None


def _prebuilt_reference():
    so = sorted(REF_DIR.glob(f"{REF_MODULE}*.so"))
    if not so:
        return None
    spec = importlib.util.spec_from_file_location(REF_MODULE, so[0])
    mod = importlib.util.module_from_spec(spec)
    import torch  # noqa: F401  (the extension links against torch's libraries)

    spec.loader.exec_module(mod)
    return mod


def build_reference(root: str | os.PathLike | None = None, verbose: bool = False):
    """Compile and import the reference's fused kernel from the checkout at ``root``.

    Without a checkout, the module an earlier build wrote into ``oracle/_ref/``
    is imported; None when neither exists.
    """
    src = reference_source(root)
    if src is None:
        return _prebuilt_reference()
    from torch.utils.cpp_extension import load

    REF_DIR.mkdir(exist_ok=True)
    return load(name=REF_MODULE, sources=[str(src)], extra_cflags=["-O3"],
                build_directory=str(REF_DIR), verbose=verbose)


if __name__ == "__main__":
    import sys

    print(build_oracle(force=True))
    print(build_reference(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True))
