"""Build the CUDA library in tree: botorch_gb300/_lib/libbotorch_gb300.so (sm_103a only),
and the thin torch extension over it, botorch_gb300/_lib/libbotorch_gb300_torch.so.

Each .cu translation unit is compiled by its own nvcc process (in parallel),
then linked into one shared library with the shared CUDA runtime, the same
libcudart that PyTorch loads; the library exposes a plain C ABI
(include/botorch_gb300.h). The extension (csrc/torch_ext.cpp) is compiled by
the host compiler against torch's headers in the same parallel batch and
linked against the library: it registers the hot path's entry points as
dispatcher operators (torch.ops.botorch_gb300.*). No cmake, no ninja.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB_NAME = "libbotorch_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(ROOT / "include")]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build botorch_gb300")
    return cand


EXT_NAME = "libbotorch_gb300_torch.so"
EXT_SOURCE = CSRC / "torch_ext.cpp"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def ext_path() -> Path:
    """The thin torch extension (dispatcher operators over the C ABI)."""
    return OUT_DIR / EXT_NAME


def _torch_flags() -> tuple[list[str], list[str]]:
    """Compile and link flags of a torch extension built with the host compiler
    (torch's headers and libraries; no Python headers: the operators are
    registered with the dispatcher, not bound through pybind)."""
    import torch
    from torch.utils import cpp_extension as ce

    cuda_home = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    inc = [p for p in ce.include_paths() if Path(p).exists()] + [str(cuda_home / "include"), str(ROOT / "include")]
    cflags = ["-O2", "-std=c++17", "-fPIC", f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}"]
    cflags += sum([["-I", p] for p in inc], [])
    tlib = ce.library_paths()[0]
    ldflags = ["-L", str(OUT_DIR), "-lbotorch_gb300", "-L", tlib, "-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu",
               "-ltorch_cuda", "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{tlib}"]
    return cflags, ldflags


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> Path:
    nvcc = nvcc_path()
    OUT_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "botorch_gb300.h"]
    objs = []
    jobs = []
    for src in sources():
        obj = OUT_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    ext_obj = OUT_DIR / "torch_ext.o"
    cflags, ldflags = _torch_flags()
    if force or _stale(ext_obj, [EXT_SOURCE, ROOT / "include" / "botorch_gb300.h"]):
        cxx = shutil.which("g++") or shutil.which("c++")
        if cxx is None:
            raise RuntimeError("a C++ compiler is required to build the torch extension")
        jobs.append([cxx, *cflags, "-c", str(EXT_SOURCE), "-o", str(ext_obj)])
    lib = lib_path()
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, res in zip(jobs, results):
            if verbose or ptxas_verbose or res.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError(f"compile failed for {cmd[-3]}")
    if force or jobs or _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(lib), *map(str, objs),
               "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
    ext = ext_path()
    if force or _stale(ext, [ext_obj, lib]):
        cxx = shutil.which("g++") or shutil.which("c++")
        res = subprocess.run([cxx, "-shared", "-o", str(ext), str(ext_obj), *ldflags], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("torch extension link failed:\n" + res.stdout + res.stderr)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
