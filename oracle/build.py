"""Build the CPU oracle (test infrastructure) into oracle/build/liboracle.so.

g++ with OpenMP, -ffp-contract=off so that only the explicit std::fma calls (the Julia
`muladd` sites) fuse, on x86-64 and aarch64 alike.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "chmy_oracle.cpp"
HDR = HERE.parent / "include" / "chmy_gb300.h"
OUT_DIR = HERE / "build"
LIB = OUT_DIR / "liboracle.so"

FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime > max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), *FLAGS, str(SRC), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
