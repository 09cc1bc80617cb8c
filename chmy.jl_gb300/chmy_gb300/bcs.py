"""Dirichlet / Neumann boundary conditions, batches and bc! (Chmy.jl src/BoundaryConditions).

Python spelling of Chmy's pairs: `(field, Neumann())` for all sides, or
`(field, {"x": Dirichlet(), "y": (Neumann(), Neumann(1.0))})` per dimension and side.
A batch applies as ONE library launch (cg_bc_apply) with the result of Chmy's 2N
per-side launches.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _abi

_AXES = ("x", "y", "z")


@dataclass(frozen=True)
class Dirichlet:
    """FirstOrderBC{DirichletKind}(value) (first_order_boundary_condition.jl:14-22)."""

    value: float | None = None
    kind = _abi.CG_BC_DIRICHLET


@dataclass(frozen=True)
class Neumann:
    """FirstOrderBC{NeumannKind}(value) (first_order_boundary_condition.jl:15-29)."""

    value: float | None = None
    kind = _abi.CG_BC_NEUMANN


@dataclass(frozen=True)
class Periodic:
    """Periodic ghost fill: ghost <- periodic image. Both sides of a dimension at once.
    (Chmy declares a Periodic connectivity but gives it no batch rule.)"""

    value: float | None = None
    kind = _abi.CG_BC_PERIODIC


def _expand(bc):
    if bc is None:
        return (None, None)
    if isinstance(bc, tuple):
        if len(bc) != 2:
            raise ValueError("a per-dimension BC tuple holds (left, right)")
        return bc
    return (bc, bc)


def regularise(ndim: int, spec) -> list[tuple]:
    """Per-field spec -> [(left, right)] per dimension (batch.jl:202-214)."""
    if spec is None or isinstance(spec, (Dirichlet, Neumann, Periodic)):
        return [(spec, spec) for _ in range(ndim)]
    if isinstance(spec, dict):
        out = [(None, None) for _ in range(ndim)]
        for k, v in spec.items():
            d = _AXES.index(k) if isinstance(k, str) else int(k) - 1
            if d >= ndim:
                raise ValueError(f"dimension {k!r} not in a {ndim}D grid")
            out[d] = _expand(v)
        return out
    raise TypeError(f"unsupported boundary-condition spec {spec!r}")


def to_cg_bc(ndim: int, spec) -> _abi.cg_bc:
    b = _abi.cg_bc()
    for d, (l, r) in enumerate(regularise(ndim, spec)):
        for s, bc in enumerate((l, r)):
            if bc is None:
                b.kind[d][s] = _abi.CG_BC_NONE
                b.value[d][s] = 0.0
            else:
                b.kind[d][s] = bc.kind
                b.value[d][s] = 0.0 if bc.value is None else float(bc.value)
    return b


class Batch:
    """A FieldBatch over all dimensions and sides (batch.jl:129-136,156-160)."""

    def __init__(self, grid, pairs):
        self.grid = grid
        self.fields = []
        self.bcs = []
        for f, spec in pairs:
            b = to_cg_bc(grid.ndim, spec)
            if all(b.kind[d][s] == _abi.CG_BC_NONE for d in range(grid.ndim) for s in range(2)):
                continue  # prune (batch.jl:235-239)
            self.fields.append(f)
            self.bcs.append(b)

    def __len__(self):
        return len(self.fields)

    def descs(self):
        n = len(self.fields)
        fa = (_abi.cg_field * max(n, 1))(*[f.desc() for f in self.fields])
        ba = (_abi.cg_bc * max(n, 1))(*self.bcs)
        return n, fa, ba


def batch(grid, *pairs, exchange=None) -> Batch:
    """batch(grid, f => bc, ...; exchange) (batch.jl:156-160). `exchange` (MPI halo exchange)
    has no meaning on one GPU and is accepted and ignored."""
    return Batch(grid, pairs)


def apply_batch(arch, grid, b: Batch) -> None:
    if len(b) == 0:
        return
    n, fa, ba = b.descs()
    g = grid.desc()
    # the library takes up to 8 fields per launch
    for start in range(0, n, 8):
        cnt = min(8, n - start)
        fsub = (_abi.cg_field * cnt)(*fa[start : start + cnt])
        bsub = (_abi.cg_bc * cnt)(*ba[start : start + cnt])
        arch.call("cg_bc_apply", ctypes.byref(g), cnt, fsub, bsub)


def bc_(arch, grid, *pairs_or_batch, exchange=None) -> None:
    """bc!(arch, grid, f => bc...) or bc!(arch, grid, batch) (batch.jl:104,241)."""
    if len(pairs_or_batch) == 1 and isinstance(pairs_or_batch[0], Batch):
        apply_batch(arch, grid, pairs_or_batch[0])
    else:
        apply_batch(arch, grid, Batch(grid, pairs_or_batch))
