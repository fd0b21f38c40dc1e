"""ORACLE build recipe (test infrastructure).

* ``build_oracle()``: the plain-C restatement ``oracle/log_areas.c`` ->
  ``oracle/_lib/liboracle_log_areas.so`` (gcc, no FMA contraction, so that
  the arithmetic is the same on x86-64 and aarch64 hosts).
* ``build_reference()``: the reference's own fused CPU kernel,
  ``botorch/csrc/logei_fused.cpp``, compiled from where it lies in the
  reference checkout (``/root/reference``) as the reference loads it (a torch
  C++ extension, botorch/acquisition/multi_objective/logei.py:85-94), with its
  output only in ``oracle/_ref/``. Skipped, returning None, where the
  checkout is absent. Used to pin the restatement and to write the golden
  fixtures in ``tests/golden/``.
"""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
LIB_DIR = ORACLE / "_lib"
REF_DIR = ORACLE / "_ref"
REFERENCE_SRC = Path("/root/reference/botorch/csrc/logei_fused.cpp")
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


def build_reference(verbose: bool = False):
    """Compile and import the reference's fused kernel; None where its source is absent."""
    if not REFERENCE_SRC.exists():
        return None
    from torch.utils.cpp_extension import load

    REF_DIR.mkdir(exist_ok=True)
    return load(name="logei_fused_ref", sources=[str(REFERENCE_SRC)], extra_cflags=["-O3"],
                build_directory=str(REF_DIR), verbose=verbose)


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(verbose=True))
