"""Build recipe for the FP64 CPU oracle (test infrastructure).

Compiles ``oracle/asend_oracle.cpp`` (the C++ restatement of the reference's
CPU algorithms) into ``oracle/liboracle.so`` with g++.  The reference itself is
Rust and cannot be compiled in this environment (no cargo/rustc), so there is
no ``oracle/_ref`` build.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "asend_oracle.cpp"
LIB = HERE / "liboracle.so"


def build(verbose: bool = False) -> Path:
    deps = [SRC, HERE / "asend_oracle.h"]
    if LIB.exists() and LIB.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return LIB
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("no C++ compiler found for the oracle")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(LIB), str(SRC)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
