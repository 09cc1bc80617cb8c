"""The C-ABI library loads and exports every entry point include/chmy_gb300.h declares.
No compute calls: runs without a GPU."""

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from chmy_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    if not _abi.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    return _abi.load_library()


def test_header_declares_entry_points():
    syms = _abi.header_symbols()
    assert "cg_init" in syms and "cg_bc_apply" in syms and "cg_stokes_solve" in syms
    assert len(syms) >= 20


def test_library_exports_every_header_symbol(lib):
    for name in _abi.header_symbols():
        assert hasattr(lib, name), f"{name} declared in include/chmy_gb300.h but not exported"


def test_ctypes_signatures_cover_header():
    assert set(_abi.header_symbols()) <= set(_abi.SIGNATURES), set(_abi.header_symbols()) - set(_abi.SIGNATURES)


def test_abi_version(lib):
    assert lib.cg_abi_version() == _abi.ABI_VERSION


def test_struct_layouts_match_header():
    """Compile a probe against the header with the host compiler and compare sizeof/offsetof."""
    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "chmy_gb300.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(cg_field), sizeof(cg_grid), sizeof(cg_bc),
             sizeof(cg_stokes_fields), sizeof(cg_stokes_params), sizeof(cg_solve_opts), sizeof(cg_solve_result),
             offsetof(cg_field, stride));
      return 0;
    }
    """
    tmp = ROOT / "oracle" / "build"
    tmp.mkdir(parents=True, exist_ok=True)
    c = tmp / "layout_probe.c"
    exe = tmp / "layout_probe"
    c.write_text(src)
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    want = [
        ctypes.sizeof(_abi.cg_field),
        ctypes.sizeof(_abi.cg_grid),
        ctypes.sizeof(_abi.cg_bc),
        ctypes.sizeof(_abi.cg_stokes_fields),
        ctypes.sizeof(_abi.cg_stokes_params),
        ctypes.sizeof(_abi.cg_solve_opts),
        ctypes.sizeof(_abi.cg_solve_result),
        _abi.cg_field.stride.offset,
    ]
    assert [int(x) for x in out] == want


def test_error_status_without_context(lib):
    """A NULL context is rejected with CG_ERR_ARG and a message, never a crash."""
    rc = lib.cg_sync(None)
    assert rc == _abi.CG_ERR_ARG
    assert b"ctx" in lib.cg_last_error(None)
    rc = lib.cg_bc_apply(None, None, 0, None, None)
    assert rc == _abi.CG_ERR_ARG


def test_no_closed_copy_calls_in_sources():
    """The sources issue one cudaMemcpy(2D)Async per copy; no batched copy API is used."""
    pat = re.compile(r"Memcpy\w*Batch")
    for p in list((ROOT / "chmy.jl_gb300" / "csrc").glob("*")) + [ROOT / "include" / "chmy_gb300.h"]:
        assert not pat.search(p.read_text()), p
