"""Build the in-tree CUDA library ``asend3d_gb300/libasend_gpu.so`` for sm_103a
and the job-file CLI ``asend3d_gb300/asend_run_job`` on its C ABI.

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel, then
linked into one shared library exporting the C ABI of
``include/asend_gpu.h``.  Outputs stay in-tree (``asend3d_gb300/_build`` and
the ``.so`` next to this file); both are git-ignored.
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
BUILD = PKG / "_build"
LIB = PKG / "libasend_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libasend_gpu.so")


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    if obj.exists() and obj.stat().st_mtime > max(src.stat().st_mtime, _newest_header()):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def _newest_header() -> float:
    hdrs = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return max((h.stat().st_mtime for h in hdrs), default=0.0)


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    try:
        build_cli(verbose)
    except (RuntimeError, OSError) as err:  # the library stays usable; the CLI's own tests report it
        print(f"warning: asend_run_job was not built: {err}", file=sys.stderr)
    return LIB


CLI_SRC = PKG / "cli" / "asend_run_job.cpp"
CLI = PKG / "asend_run_job"


def build_cli(verbose: bool = False) -> Path:
    """The job-file CLI (host C++ on the C ABI), linked against the library."""
    newest = max(CLI_SRC.stat().st_mtime, (ROOT / "include" / "asend_gpu.h").stat().st_mtime, LIB.stat().st_mtime)
    if CLI.exists() and CLI.stat().st_mtime >= newest:
        return CLI
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cuda_lib = Path(nvcc()).resolve().parent.parent / "lib64"  # libcudart, needed by the library
    cmd = [cxx, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(CLI_SRC), f"-L{PKG}", "-lasend_gpu",
           f"-L{cuda_lib}", f"-Wl,-rpath-link,{cuda_lib}", "-Wl,-rpath,$ORIGIN", "-o", str(CLI)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"asend_run_job build failed:\n{res.stdout}\n{res.stderr}")
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
