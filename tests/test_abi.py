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
      printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(cg_field), sizeof(cg_grid), sizeof(cg_bc),
             sizeof(cg_stokes_fields), sizeof(cg_stokes_params), sizeof(cg_solve_opts), sizeof(cg_solve_result),
             offsetof(cg_field, stride), sizeof(cg_function), sizeof(cg_mask), sizeof(cg_bc_fn),
             offsetof(cg_bc_fn, full_dims));
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
        ctypes.sizeof(_abi.cg_function),
        ctypes.sizeof(_abi.cg_mask),
        ctypes.sizeof(_abi.cg_bc_fn),
        _abi.cg_bc_fn.full_dims.offset,
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


def _field2d(nx, ny, loc=(0, 0), dtype=_abi.CG_F64, halo=1, pitch=None):
    """A host descriptor with no data (layout only), as the size queries read it."""
    f = _abi.cg_field()
    f.dtype, f.ndim = dtype, 2
    ext = [nx + loc[0], ny + loc[1]]
    f.n[0], f.n[1], f.n[2] = ext[0], ext[1], 1
    f.loc[0], f.loc[1] = loc
    f.halo[0], f.halo[1] = halo, halo
    f.stride[0], f.stride[1] = 1, pitch or (ext[0] + 4 * halo)
    return f


def _grid2d(nx, ny):
    g = _abi.cg_grid()
    g.ndim = 2
    g.n[0], g.n[1], g.n[2] = nx, ny, 1
    for d in range(2):
        g.extent[d] = 2.0
        g.spacing[d] = 2.0 / (nx, ny)[d]
        g.inv_spacing[d] = 1.0 / g.spacing[d]
    return g


def test_sia_tape_sizes(lib):
    """The tape-size queries (no context, no device work) follow the documented layouts: a
    256-byte header, then per step 256 bytes of words and 9 arrays of H's allocation (row
    stride x (n_y + 4 halo) elements), each rounded up to 256 bytes; an ensemble tape holds
    every member's step block in turn. Bad arguments give CG_ERR_ARG."""

    def r256(b):
        return (b + 255) // 256 * 256

    for dt, el in ((_abi.CG_F64, 8), (_abi.CG_F32, 4)):
        H = _field2d(37, 21, dtype=dt, pitch=64)
        g = _grid2d(37, 21)
        step = 256 + 9 * r256(64 * (21 + 4) * el)
        out = ctypes.c_size_t()
        assert lib.cg_sia_tape_bytes(ctypes.byref(g), ctypes.byref(H), 5, ctypes.byref(out)) == 0
        assert out.value == 256 + 5 * step
        assert lib.cg_sia_tape_bytes(ctypes.byref(g), ctypes.byref(H), 0, ctypes.byref(out)) == 0
        assert out.value == 256
        assert lib.cg_sia_tape_bytes(ctypes.byref(g), ctypes.byref(H), -1, ctypes.byref(out)) == _abi.CG_ERR_ARG
        mem = (_abi.cg_sia_member * 2)()
        sizes = [(37, 21, 64), (50, 33, 57)]
        for k, (nx, ny, pitch) in enumerate(sizes):
            mem[k].grid = _grid2d(nx, ny)
            mem[k].H = _field2d(nx, ny, dtype=dt, pitch=pitch)
        per = sum(256 + 9 * r256(p * (ny + 4) * el) for nx, ny, p in sizes)
        assert lib.cg_sia_ensemble_tape_bytes(2, mem, 7, ctypes.byref(out)) == 0
        assert out.value == 256 + 7 * per
        assert lib.cg_sia_ensemble_tape_bytes(0, mem, 7, ctypes.byref(out)) == _abi.CG_ERR_ARG
