"""Helpers shared by the GPU parity tests: mirror oracle fields onto the device."""

from __future__ import annotations

import numpy as np

from _oracle import NpField
from chmy_gb300 import Field


def to_gpu(arch, f: NpField, pitch_align: int = 0, plane_rows: int = 0) -> Field:
    g = Field(arch, f.grid, f.loc, f.dtype, f.halo, pitch_align=pitch_align, plane_rows=plane_rows)
    g.from_numpy(f.a)
    return g


def random_field(grid, loc, dtype, rng, scale=1.0, offset=0.0) -> NpField:
    f = NpField(grid, loc, dtype)
    f.a[...] = (offset + scale * rng.standard_normal(f.a.shape)).astype(dtype)
    return f


def assert_close(gpu: Field, ref: NpField, rtol: float, what: str = "", exact: bool = False) -> None:
    a = gpu.to_numpy()
    b = ref.a
    if exact:
        bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
        assert bad.size == 0, f"{what}: {len(bad)} mismatches, first at {bad[:3].tolist()}: gpu {a[tuple(bad[0])]} ref {b[tuple(bad[0])]}"
        return
    scale = max(float(np.max(np.abs(b))), 1e-300)
    err = float(np.max(np.abs(a.astype(np.float64) - b.astype(np.float64))))
    assert err <= rtol * scale, f"{what}: max|gpu-ref| = {err:.3e} > {rtol:.1e} * {scale:.3e}"


def rtol_for(dtype) -> float:
    """Per-launch tolerance, normwise relative to max|reference|: FP64 1e-12 (FMA contraction
    aside the arithmetic is the reference's), FP32 2e-5."""
    return 1e-12 if dtype == np.float64 else 2e-5
