"""In-tree build of libchmy_gb300.so (sm_103a) with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel to an object under ``_build/``
and linked into ``chmy_gb300/lib/libchmy_gb300.so``. Objects are rebuilt only when their
source or a header is newer. No CMake, no torch extension machinery: the library is plain
CUDA C++ behind a C ABI and can be loaded from any host language.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT_DIR = PKG_DIR.parent  # chmy.jl_gb300/
CSRC = ROOT_DIR / "csrc"
INCLUDE = ROOT_DIR.parent / "include"
BUILD_DIR = ROOT_DIR / "_build"
LIB_DIR = PKG_DIR / "lib"
LIB_PATH = LIB_DIR / "libchmy_gb300.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
    "-DNDEBUG",
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libchmy_gb300")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(nvcc: str, src: Path, obj: Path, verbose_ptxas: bool) -> tuple[Path, str]:
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return obj, proc.stderr


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> Path:
    """Compile every csrc/*.cu for sm_103a and link libchmy_gb300.so; return its path."""
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    if not sources:
        raise RuntimeError(f"no CUDA sources under {CSRC}")
    deps = _headers()
    todo = []
    objs = []
    for src in sources:
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or verbose_ptxas or _stale(obj, src, deps):
            todo.append((src, obj))
    logs = []
    if todo:
        workers = jobs or min(len(todo), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, verbose_ptxas) for s, o in todo]
            for f in futs:
                obj, log = f.result()
                if log.strip():
                    logs.append(f"--- {obj.name}\n{log}")
    if todo or not LIB_PATH.exists() or any(o.stat().st_mtime > LIB_PATH.stat().st_mtime for o in objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs)]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
        os.replace(tmp, LIB_PATH)
    if verbose_ptxas and logs:
        sys.stderr.write("\n".join(logs))
    return LIB_PATH


if __name__ == "__main__":
    force = "--force" in sys.argv
    ptx = "--ptxas" in sys.argv
    print(build(force=force, verbose_ptxas=ptx))
