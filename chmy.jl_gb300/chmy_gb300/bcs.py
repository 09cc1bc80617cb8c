"""Dirichlet / Neumann boundary conditions, batches and bc! (Chmy.jl src/BoundaryConditions).

Python spelling of Chmy's pairs: `(field, Neumann())` for all sides, or
`(field, {"x": Dirichlet(), "y": (Neumann(), Neumann(1.0))})` per dimension and side.
A batch applies as ONE library launch (cg_bc_apply) with the result of Chmy's 2N
per-side launches.

A condition's value is `None` (0), a number, a BoundaryFunction, or per-point values: a
lower-dimensional Field (Chmy's FirstOrderBC{<:AbstractField}, read at remove_dim(dim, I)) or
a host array over the tangential logical indices 0..n_t+2 ([z, y, x] storage order without
the condition's dimension). Functions and arrays become per-point value arrays of the
field's type, passed to the library in cg_bc.values.
"""

from __future__ import annotations

import ctypes
import numbers
from dataclasses import dataclass

import numpy as np

from . import _abi
from .grids import Center, Vertex, expand_loc, flip

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


class Dim:
    """Chmy's Dim(D) (1-based), which tells coord(grid, loc, Dim(d), i) apart from
    coord(grid, loc, I...)."""

    def __init__(self, d: int):
        self.d = int(d)

    def __index__(self):
        return self.d

    def __repr__(self):
        return f"Dim({self.d})"


def coord(grid, loc, *args):
    """coord(grid, loc, I...) -> the point's coordinates, every dimension at location `loc`
    (src/Grids/structured_grid.jl:103-107); coord(grid, loc, Dim(d), i) -> the coordinate along
    dimension d at index i (:115-119). Indices are Chmy's (1-based interior)."""
    if args and isinstance(args[0], Dim):
        return grid.coord(loc, args[0].d, int(args[1]))
    locs = expand_loc(grid.ndim, loc)
    return tuple(grid.axes[k].coord(locs[k], int(i)) for k, i in enumerate(args))


class BoundaryFunction:
    """BoundaryFunction(fun; discrete=false, parameters=nothing, reduce_dims=true)
    (src/BoundaryConditions/boundary_function.jl:34-76). Called as bf(grid, loc, dim, I...)
    with dim a Dim (or a 1-based int) and I the point's indices, one per dimension.
    - Continuous: fun(coords..., params...) at coord(grid, loc, I...), with the coordinate
      along `dim` removed when reduce_dims.
    - Discrete: fun(grid, loc, dim, I..., params...), with the index along `dim` removed when
      reduce_dims.
    `parameters` is a value or a tuple of values, splatted after the coordinates."""

    def __init__(self, fun, discrete: bool = False, parameters=None, reduce_dims: bool = True):
        self.fun, self.discrete, self.parameters, self.reduce_dims = fun, bool(discrete), parameters, bool(reduce_dims)

    def _params(self) -> tuple:
        p = self.parameters
        if p is None:
            return ()
        return tuple(p) if isinstance(p, (tuple, list)) else (p,)

    def __call__(self, grid, loc, dim, *I):
        d0 = int(dim) - 1
        dimv = dim if isinstance(dim, Dim) else Dim(int(dim))
        if self.discrete:
            idx = tuple(i for k, i in enumerate(I) if not (self.reduce_dims and k == d0))
            return self.fun(grid, loc, dimv, *idx, *self._params())
        c = coord(grid, loc, *I)
        if self.reduce_dims:
            c = tuple(x for k, x in enumerate(c) if k != d0)
        return self.fun(*c, *self._params())


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


def _constant(v) -> bool:
    return v is None or isinstance(v, numbers.Number)


def to_cg_bc(ndim: int, spec) -> _abi.cg_bc:
    """Conditions with constant values (`None` or a number) as a cg_bc; per-point values
    need the field: materialize_bc."""
    b = _abi.cg_bc()
    for d, (l, r) in enumerate(regularise(ndim, spec)):
        for s, bc in enumerate((l, r)):
            if bc is None:
                b.kind[d][s] = _abi.CG_BC_NONE
                b.value[d][s] = 0.0
            else:
                if not _constant(bc.value):
                    raise TypeError("a per-point boundary value needs its field: use materialize_bc or a Batch")
                b.kind[d][s] = bc.kind
                b.value[d][s] = 0.0 if bc.value is None else float(bc.value)
    return b


def bc_values(grid, loc, dtype, d: int, side: int, bc) -> np.ndarray:
    """The per-point values of condition `bc` on side `side` of dimension d (0-based) for a
    field at `loc`: a host array over the tangential logical indices 0..n_t+2 ([z, y, x] order
    without dimension d), as the library's cg_bc.values reads it.
    - BoundaryFunction: evaluated at the points the condition writes
      (first_order_boundary_condition.jl:46-84). The location is the field's along d for
      Dirichlet and its flip for Neumann, applied to every dimension. The index along d is
      the boundary node (Vertex Dirichlet: 1 or n+1), else the ghost (0 or n+1 for Center,
      0 or n+2 for Vertex).
    - A lower-dimensional Field: its logical indices 0..n_t+2.
    - An array: taken as is (shape checked)."""
    nd = grid.ndim
    locs = expand_loc(nd, loc)
    tdims = [t for t in range(nd) if t != d]
    shape = tuple(grid.dims[t] + 3 for t in reversed(tdims))
    v = bc.value
    if isinstance(v, BoundaryFunction):
        ext = grid.axes[d].size(locs[d])
        vtx = isinstance(locs[d], Vertex)
        if bc.kind == _abi.CG_BC_DIRICHLET and vtx:
            gi = 1 if side == 0 else ext
        else:
            gi = 0 if side == 0 else ext + 1
        eval_loc = locs[d] if bc.kind == _abi.CG_BC_DIRICHLET else flip(locs[d])
        out = np.empty(shape, dtype=dtype)
        for flat in range(out.size):
            rem = flat
            I = [0] * nd
            I[d] = gi
            for t in tdims:
                I[t] = rem % (grid.dims[t] + 3)
                rem //= grid.dims[t] + 3
            out.reshape(-1)[flat] = v(grid, eval_loc, Dim(d + 1), *I)
        return out
    if hasattr(v, "to_numpy") and hasattr(v, "halo"):
        a = v.to_numpy()
        sl = tuple(slice(2 * h - 1, 2 * h - 1 + n) for h, n in zip(reversed(v.halo), shape))
        out = np.ascontiguousarray(a[sl], dtype=dtype)
    else:
        out = np.ascontiguousarray(np.asarray(v, dtype=dtype))
    if out.shape != shape:
        raise ValueError(f"per-point boundary values on dimension {d + 1}: expected shape {shape}, got {out.shape}")
    return out


def device_function_of(bc):
    """The cg_function of a condition whose value is a continuous BoundaryFunction over a form
    the library evaluates on the device (functions.constant / ball / affine), else None."""
    from .functions import DeviceFunction

    v = getattr(bc, "value", None)
    if isinstance(v, BoundaryFunction) and not v.discrete and isinstance(v.fun, DeviceFunction):
        return v
    return None


def materialize_bc(grid, loc, dtype, spec, device=None, fns=None):
    """A cg_bc for a field at `loc` whose conditions may carry per-point values. The value
    arrays live in host memory (device=None, for the oracle) or on `device` (a torch device).
    With `fns` (a cg_bc_fn), a continuous BoundaryFunction over a device form is recorded
    there, to be evaluated by the boundary-condition kernel (cg_bc_apply_fn), instead of being
    evaluated on the host. Returns (cg_bc, keep): `keep` holds the arrays, and must stay alive
    while the cg_bc is used."""
    nd = grid.ndim
    b = _abi.cg_bc()
    keep = []
    for d, (l, r) in enumerate(regularise(nd, spec)):
        for s, bc in enumerate((l, r)):
            if bc is None:
                b.kind[d][s] = _abi.CG_BC_NONE
                continue
            b.kind[d][s] = bc.kind
            if _constant(bc.value):
                b.value[d][s] = 0.0 if bc.value is None else float(bc.value)
                continue
            dfn = device_function_of(bc) if fns is not None else None
            if dfn is not None and bc.kind in (_abi.CG_BC_DIRICHLET, _abi.CG_BC_NEUMANN):
                nargs = nd if not dfn.reduce_dims else nd - 1
                fns.fn[d][s].kind = dfn.fun.kind
                for q, val in enumerate(dfn.fun.pack(nargs, dfn.parameters)):
                    fns.fn[d][s].p[q] = val
                fns.full_dims[d][s] = 0 if dfn.reduce_dims else 1
                continue
            arr = bc_values(grid, loc, dtype, d, s, bc)
            if device is not None:
                import torch

                t = torch.from_numpy(arr).to(device)
                keep.append(t)
                b.values[d][s] = t.data_ptr()
            else:
                keep.append(arr)
                b.values[d][s] = arr.ctypes.data
    return b, keep


class Batch:
    """A FieldBatch over all dimensions and sides (batch.jl:129-136,156-160)."""

    def __init__(self, grid, pairs):
        self.grid = grid
        self.fields = []
        self.bcs = []
        self.fns = []  # BoundaryFunction sides evaluated by the kernel (cg_bc_fn per field)
        self._keep = []  # per-point value arrays on the fields' device
        for f, spec in pairs:
            dev = getattr(getattr(f, "arch", None), "device", None)
            fn = _abi.cg_bc_fn() if dev is not None else None
            b, keep = materialize_bc(grid, f.loc, f.dtype, spec, dev, fn)
            self._keep.extend(keep)
            if all(b.kind[d][s] == _abi.CG_BC_NONE for d in range(grid.ndim) for s in range(2)):
                continue  # prune (batch.jl:235-239)
            self.fields.append(f)
            self.bcs.append(b)
            self.fns.append(fn if fn is not None else _abi.cg_bc_fn())

    def __len__(self):
        return len(self.fields)

    def descs(self):
        n = len(self.fields)
        fa = (_abi.cg_field * max(n, 1))(*[f.desc() for f in self.fields])
        ba = (_abi.cg_bc * max(n, 1))(*self.bcs)
        return n, fa, ba

    def has_functions(self) -> bool:
        return any(fn.fn[d][s].kind != _abi.CG_FN_NONE for fn in self.fns for d in range(3) for s in range(2))


def batch(grid, *pairs, exchange=None) -> Batch:
    """batch(grid, f => bc, ...; exchange) (batch.jl:156-160). `exchange` (MPI halo exchange)
    has no meaning on one GPU and is accepted and ignored."""
    return Batch(grid, pairs)


def apply_batch(arch, grid, b: Batch) -> None:
    if len(b) == 0:
        return
    n, fa, ba = b.descs()
    g = grid.desc()
    with_fn = b.has_functions()
    # the library takes up to 8 fields per launch
    for start in range(0, n, 8):
        cnt = min(8, n - start)
        fsub = (_abi.cg_field * cnt)(*fa[start : start + cnt])
        bsub = (_abi.cg_bc * cnt)(*ba[start : start + cnt])
        if with_fn:
            nsub = (_abi.cg_bc_fn * cnt)(*b.fns[start : start + cnt])
            arch.call("cg_bc_apply_fn", ctypes.byref(g), cnt, fsub, bsub, nsub)
        else:
            arch.call("cg_bc_apply", ctypes.byref(g), cnt, fsub, bsub)


def bc_(arch, grid, *pairs_or_batch, exchange=None) -> None:
    """bc!(arch, grid, f => bc...) or bc!(arch, grid, batch) (batch.jl:104,241)."""
    if len(pairs_or_batch) == 1 and isinstance(pairs_or_batch[0], Batch):
        apply_batch(arch, grid, pairs_or_batch[0])
    else:
        apply_batch(arch, grid, Batch(grid, pairs_or_batch))
